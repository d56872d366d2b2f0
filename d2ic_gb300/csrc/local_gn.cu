// Local Gauss-Newton sweeps (d2ic/solver_local_gn.py LocalGaussNewtonSolver):
//
//   central_diff   gradient images of the deformed image by central differences,
//                  zero on the first/last column (x) and row (y) (:195-201);
//   lgn_chunks     one warp per chunk of the element-major pixel list: at
//                  x_def = x + sum_a N_a u_a, r = I2(x_def) - I1 and the gradient
//                  images sampled at x_def with the same interpolator (:214-256);
//                  per local node a the terms of its 2x2 normal equations,
//                  J = (gx, gy) N_a:  r Jx, r Jy, Jx^2, Jx Jy, Jy^2, reduced over
//                  the chunk and stored in the chunk's slot of that node (the
//                  same chunk -> slot -> node layout as the CG engine: no atomics,
//                  fixed order); the chunk's sum of r^2 for the history;
//   lgn_nodes      per node: the K slots summed in slot order, Levenberg term
//                  lam * trace, springs alpha * rho_i * sum_j w_ij (u_i - u_j),
//                  +1e-8 I, the 2x2 solve, the step clipped to max_step, relaxed
//                  by omega (:316-414); per-block sum of squared steps.
#include "common.cuh"

namespace d2ic {

__global__ void central_diff_kernel(const float *__restrict__ im, int H, int W, float *__restrict__ gx,
                                    float *__restrict__ gy) {
    const size_t n = (size_t)H * W;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / W), j = (int)(k % W);
        gx[k] = (j > 0 && j < W - 1) ? 0.5f * (im[k + 1] - im[k - 1]) : 0.f;
        gy[k] = (i > 0 && i < H - 1) ? 0.5f * (im[k + W] - im[k - W]) : 0.f;
    }
}

// value only of the halo'd sampling array (cubic coefficients or padded image)
template <int KIND>
__device__ __forceinline__ float sample_value(const Img &im, int ix, int iy, float tx, float ty) {
    float gx, gy;
    return sample<KIND>(im, ix, iy, tx, ty, gx, gy);
}

template <int KIND>
__global__ void __launch_bounds__(256) lgn_chunks_kernel(const d2ic_frame_t *__restrict__ F,
                                                         const float *__restrict__ cgx, const float *__restrict__ cgy,
                                                         const float2 *__restrict__ u, float4 *__restrict__ slots,
                                                         double *__restrict__ chunk_r2) {
    const int lane = threadIdx.x & 31;
    const int nc = F->n_chunks, Nn = F->n_nodes;
    const Img i2{F->coeff, F->W, F->H, F->cpitch, F->pad};
    const Img igx{cgx, F->W, F->H, F->cpitch, F->pad};
    const Img igy{cgy, F->W, F->H, F->cpitch, F->pad};
    const uint4 *pix = reinterpret_cast<const uint4 *>(F->pix);
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nc; c += (gridDim.x * blockDim.x) >> 5) {
        int nd = 0, slot = 0;
        float2 un = make_float2(0.f, 0.f);
        if (lane < 4) {
            nd = __ldg(F->chunk_nodes + 4 * c + lane);
            slot = (int)(((unsigned)__ldg(F->chunk_slot + c) >> (8 * lane)) & 0xffu);
            un = u[nd];
        }
        float ux[4], uy[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            ux[a] = __shfl_sync(0xffffffffu, un.x, a);
            uy[a] = __shfl_sync(0xffffffffu, un.y, a);
        }
        float acc[4][5];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int q = 0; q < 5; ++q) acc[a][q] = 0.f;
        float r2 = 0.f;
        const int pb = __ldg(F->chunk_begin + c), pe = __ldg(F->chunk_begin + c + 1);
        for (int p = pb + lane; p < pe; p += 32) {
            const uint4 r4 = __ldg(pix + p);
            const int x = (int)(r4.x & 0xffffu), y = (int)(r4.x >> 16);
            const float I1 = __uint_as_float(r4.y), xi = __uint_as_float(r4.z), eta = __uint_as_float(r4.w);
            const float a0 = 0.5f * (1.f - xi), a1 = 0.5f * (1.f + xi);
            const float b0 = 0.5f * (1.f - eta), b1 = 0.5f * (1.f + eta);
            const float N[4] = {a0 * b0, a1 * b0, a1 * b1, a0 * b1};
            const float dx = N[0] * ux[0] + N[1] * ux[1] + N[2] * ux[2] + N[3] * ux[3];
            const float dy = N[0] * uy[0] + N[1] * uy[1] + N[2] * uy[2] + N[3] * uy[3];
            int ix, iy;
            float tx, ty;
            split_coord(x, dx, ix, tx);
            split_coord(y, dy, iy, ty);
            const float r = sample_value<KIND>(i2, ix, iy, tx, ty) - I1;
            const float gx = sample_value<KIND>(igx, ix, iy, tx, ty);
            const float gy = sample_value<KIND>(igy, ix, iy, tx, ty);
            r2 += r * r;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float jx = gx * N[a], jy = gy * N[a];
                acc[a][0] += r * jx;
                acc[a][1] += r * jy;
                acc[a][2] += jx * jx;
                acc[a][3] += jx * jy;
                acc[a][4] += jy * jy;
            }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int q = 0; q < 5; ++q) acc[a][q] = warp_sum_f(acc[a][q]);
        const DF rs = df_warp_sum(DF{r2, 0.f});
        if (lane == 0) chunk_r2[c] = df_to_double(rs);
        if (lane < 4) {
            float v[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) v[q] = lane == 0 ? acc[0][q] : lane == 1 ? acc[1][q] : lane == 2 ? acc[2][q] : acc[3][q];
            float4 *s = slots + 2 * ((size_t)slot * Nn + nd);
            s[0] = make_float4(v[0], v[1], v[2], v[3]);
            s[1] = make_float4(v[4], 0.f, 0.f, 0.f);
        }
    }
}

__global__ void __launch_bounds__(256) lgn_nodes_kernel(int Nn, int K, const float4 *__restrict__ slots,
                                                        const float2 *__restrict__ u, const int *__restrict__ has_pix,
                                                        const int *__restrict__ nbr, const float *__restrict__ nbw,
                                                        int md, const float *__restrict__ rho, float lam,
                                                        float max_step, float alpha_reg, float omega,
                                                        float2 *__restrict__ u_next, double *__restrict__ step_part) {
    __shared__ double s_red[8];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    double st = 0.0;
    if (n < Nn) {
        float g0 = 0.f, g1 = 0.f, h00 = 0.f, h01 = 0.f, h11 = 0.f;
        for (int k = 0; k < K; ++k) {
            const float4 a = slots[2 * ((size_t)k * Nn + n)];
            const float4 b = slots[2 * ((size_t)k * Nn + n) + 1];
            g0 += a.x;
            g1 += a.y;
            h00 += a.z;
            h01 += a.w;
            h11 += b.x;
        }
        const float lam_loc = lam * (h00 + h11 + 1e-12f);
        const float2 ui = u[n];
        const float al = alpha_reg * rho[n];
        float sw = 0.f, rx = 0.f, ry = 0.f;
        int deg = 0;
        for (int k = 0; k < md; ++k) {
            const int j = nbr[(size_t)k * Nn + n];
            if (j < 0) break;
            const float w = nbw[(size_t)k * Nn + n];
            const float2 uj = u[j];
            sw += w;
            rx += w * (ui.x - uj.x);
            ry += w * (ui.y - uj.y);
            ++deg;
        }
        const float hr = al * sw;
        const float a11 = h00 + lam_loc + hr + 1e-8f, a22 = h11 + lam_loc + hr + 1e-8f, a12 = h01;
        const float b0 = g0 + al * rx, b1 = g1 + al * ry;
        const float det = a11 * a22 - a12 * a12;
        float dx = -(a22 * b0 - a12 * b1) / det;
        float dy = -(a11 * b1 - a12 * b0) / det;
        const bool upd = has_pix[n] != 0 || (alpha_reg != 0.f && deg > 0);
        if (!upd) dx = dy = 0.f;
        const float f = fminf(1.f, max_step / (sqrtf(dx * dx + dy * dy) + 1e-12f));
        dx *= f;
        dy *= f;
        const float sx = omega * dx, sy = omega * dy;
        u_next[n] = make_float2(ui.x + sx, ui.y + sy);
        st = (double)sx * sx + (double)sy * sy;
    }
    st = warp_sum_d(st);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = st;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
        step_part[blockIdx.x] = t;
    }
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_central_gradient(const float *img, int H, int W, float *gx, float *gy, void *stream) {
    D2IC_REQUIRE(img && gx && gy && H >= 1 && W >= 1, "d2ic_central_gradient: bad arguments");
    const size_t n = (size_t)H * W;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    central_diff_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(img, H, W, gx, gy);
    D2IC_CHECK_LAUNCH("central_diff_kernel");
    return D2IC_OK;
}

extern "C" size_t d2ic_local_gn_slot_bytes(int n_nodes, int node_chunk_k) {
    return sizeof(float) * 8 * (size_t)(n_nodes > 0 ? n_nodes : 1) * (size_t)(node_chunk_k > 0 ? node_chunk_k : 1);
}

extern "C" int d2ic_local_gn_sweep(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                                   int interp_kind, const float *coeff_gx, const float *coeff_gy, const float *u,
                                   float *slots, double *chunk_r2, const int *has_pix, const int *nbr_index,
                                   const float *nbr_weight, int max_deg, const float *node_reg_weight, float lam,
                                   float max_step, float alpha_reg, float omega, float *u_next, double *step_part,
                                   void *stream) {
    D2IC_REQUIRE(frame_dev && coeff_gx && coeff_gy && u && slots && chunk_r2 && has_pix && node_reg_weight && u_next &&
                     step_part,
                 "d2ic_local_gn_sweep: null pointer");
    D2IC_REQUIRE(n_nodes >= 1 && n_chunks >= 0 && node_chunk_k >= 1 && max_deg >= 0,
                 "d2ic_local_gn_sweep: bad sizes");
    D2IC_REQUIRE(max_deg == 0 || (nbr_index && nbr_weight), "d2ic_local_gn_sweep: null spring table");
    D2IC_REQUIRE(interp_kind == D2IC_INTERP_CUBIC || interp_kind == D2IC_INTERP_LINEAR,
                 "d2ic_local_gn_sweep: unknown interpolation %d", interp_kind);
    D2IC_REQUIRE(u != u_next, "d2ic_local_gn_sweep: u and u_next must differ");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_chunks > 0) {
        int blocks = (n_chunks + 7) / 8;
        if (blocks > 65535) blocks = 65535;
        if (interp_kind == D2IC_INTERP_CUBIC)
            lgn_chunks_kernel<D2IC_INTERP_CUBIC><<<blocks, 256, 0, s>>>(frame_dev, coeff_gx, coeff_gy, (const float2 *)u,
                                                                        (float4 *)slots, chunk_r2);
        else
            lgn_chunks_kernel<D2IC_INTERP_LINEAR><<<blocks, 256, 0, s>>>(frame_dev, coeff_gx, coeff_gy,
                                                                         (const float2 *)u, (float4 *)slots, chunk_r2);
        D2IC_CHECK_LAUNCH("lgn_chunks_kernel");
    }
    lgn_nodes_kernel<<<(n_nodes + 255) / 256, 256, 0, s>>>(n_nodes, node_chunk_k, (const float4 *)slots,
                                                           (const float2 *)u, has_pix, nbr_index, nbr_weight, max_deg,
                                                           node_reg_weight, lam, max_step, alpha_reg, omega,
                                                           (float2 *)u_next, step_part);
    D2IC_CHECK_LAUNCH("lgn_nodes_kernel");
    return D2IC_OK;
}
