// Implicit-function derivative of the converged solve (uncertainty propagation).
//
// At the converged u*, grad_u J(u*, I2) = 0 defines u*(I2); its derivative is
//     du* = -H^-1 (d grad_u J / dI2) dI,
// H the exact Hessian of J.  Kernels:
//   * hessian_chunks: one pixel pass at u*; per chunk the 10 distinct 2x2 blocks
//     N_a N_b (grad I2 grad I2^T + r hess I2) summed over the chunk's pixels
//     (3 numbers each: xx, xy, yy), i.e. the element Hessian of the pixel term;
//   * hv_chunks / hv_nodes: H V for K right-hand sides at once (V: n_nodes x 2 x K,
//     K fastest): chunk blocks times the chunk's 4 nodal vectors into the same
//     per-node slots the CG engine uses, then a node pass that sums the slots
//     and adds the spring Hessian (no atomics);
//   * mixed_chunks / slots_to_nodes: (d grad_u J / dI2) dI for an image
//     direction given by its B-spline coefficients;
//   * mixed_T_scatter + prefilter_T: the adjoint of that map (the backward of
//     the bicubic sampling): per pixel the coefficient-space weights, scattered
//     with atomics, then the transpose of the clamped separable prefilter.
#include "common.cuh"

namespace d2ic {

constexpr int KF_T = 16;                    // prefilter half-length (matches image_ops.cu)
__constant__ float c_fir_t[2 * KF_T + 1];
__constant__ float c_cum_lo[2 * KF_T + 2];  // c_cum_lo[m + KF] = sum_{k <= m} h[k], m in [-KF, KF]
static bool g_firt_ready[64] = {false};

static int ensure_fir_t() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && g_firt_ready[dev]) return D2IC_OK;
    float h[2 * KF_T + 1], cl[2 * KF_T + 2];
    const double z = 1.7320508075688772 - 2.0;
    double acc = 0.0;
    for (int k = -KF_T; k <= KF_T; ++k) {
        double v = 1.7320508075688772;
        for (int i = 0; i < (k < 0 ? -k : k); ++i) v *= z;
        h[k + KF_T] = (float)v;
    }
    for (int k = -KF_T; k <= KF_T; ++k) {
        acc += h[k + KF_T];
        cl[k + KF_T] = (float)acc;
    }
    cl[2 * KF_T + 1] = (float)acc;
    cudaError_t e = cudaMemcpyToSymbol(c_fir_t, h, sizeof(h));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_cum_lo, cl, sizeof(cl));
    if (e != cudaSuccess) return cuda_status(e, "adjoint constants");
    if (dev >= 0 && dev < 64) g_firt_ready[dev] = true;
    return D2IC_OK;
}

__device__ __forceinline__ void bspline_w2(float t, float w2[4]) {
    w2[0] = 1.f - t;
    w2[1] = 3.f * t - 2.f;
    w2[2] = -3.f * t + 1.f;
    w2[3] = t;
}

// value, gradient and Hessian of the cubic B-spline (taps clamped as the forward sampler)
__device__ __forceinline__ void sample_cubic_h(const Img &im, int ix, int iy, float tx, float ty, float o[6]) {
    float wx[4], dwx[4], wy[4], dwy[4], ddx[4], ddy[4];
    bspline_w(tx, wx, dwx);
    bspline_w(ty, wy, dwy);
    bspline_w2(tx, ddx);
    bspline_w2(ty, ddy);
    for (int i = 0; i < 6; ++i) o[i] = 0.f;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int r = clampi(iy - 1 + a, -im.pad, im.H - 1 + im.pad);
        float rv = 0.f, rd = 0.f, rdd = 0.f;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const float c = im.at(r, clampi(ix - 1 + b, -im.pad, im.W - 1 + im.pad));
            rv += wx[b] * c;
            rd += dwx[b] * c;
            rdd += ddx[b] * c;
        }
        o[0] += wy[a] * rv;     // value
        o[1] += wy[a] * rd;     // d/dx
        o[2] += dwy[a] * rv;    // d/dy
        o[3] += wy[a] * rdd;    // d2/dx2
        o[4] += dwy[a] * rd;    // d2/dxdy
        o[5] += ddy[a] * rv;    // d2/dy2
    }
}

struct ChunkPix {
    int x, y;
    float I1, N[4];
};
__device__ __forceinline__ ChunkPix unpack(const uint4 r) {
    ChunkPix p;
    p.x = (int)(r.x & 0xffffu);
    p.y = (int)(r.x >> 16);
    p.I1 = __uint_as_float(r.y);
    const float xi = __uint_as_float(r.z), eta = __uint_as_float(r.w);
    const float a0 = 0.5f * (1.f - xi), a1 = 0.5f * (1.f + xi), b0 = 0.5f * (1.f - eta), b1 = 0.5f * (1.f + eta);
    p.N[0] = a0 * b0;
    p.N[1] = a1 * b0;
    p.N[2] = a1 * b1;
    p.N[3] = a0 * b1;
    return p;
}

__device__ __forceinline__ void chunk_nodes_u(const d2ic_frame_t &F, const float2 *u, int c, int lane, float ux[4],
                                              float uy[4], int &nd, int &slot) {
    float2 uc = make_float2(0.f, 0.f);
    nd = 0;
    slot = 0;
    if (lane < 4) {
        nd = __ldg(F.chunk_nodes + 4 * c + lane);
        slot = (int)(((unsigned)__ldg(F.chunk_slot + c) >> (8 * lane)) & 0xffu);
        uc = u[nd];
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        ux[a] = __shfl_sync(0xffffffffu, uc.x, a);
        uy[a] = __shfl_sync(0xffffffffu, uc.y, a);
    }
}

// pair (a <= b) index in 0..9
__device__ __forceinline__ int pair_index(int a, int b) { return a * 4 - (a * (a - 1)) / 2 + (b - a); }

__global__ void __launch_bounds__(256) hessian_chunks(const d2ic_frame_t *__restrict__ fp, const float2 *__restrict__ u,
                                                      int exact, float *__restrict__ out) {
    const d2ic_frame_t &F = *fp;
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= F.n_chunks) return;
    float ux[4], uy[4];
    int nd, slot;
    chunk_nodes_u(F, u, c, lane, ux, uy, nd, slot);
    const Img im{F.coeff, F.W, F.H, F.cpitch, F.pad};
    float acc[30];
#pragma unroll
    for (int i = 0; i < 30; ++i) acc[i] = 0.f;
    const int pb = __ldg(F.chunk_begin + c), pe = __ldg(F.chunk_begin + c + 1);
    for (int p = pb + lane; p < pe; p += 32) {
        const ChunkPix q = unpack(__ldg(reinterpret_cast<const uint4 *>(F.pix) + p));
        const float dx = q.N[0] * ux[0] + q.N[1] * ux[1] + q.N[2] * ux[2] + q.N[3] * ux[3];
        const float dy = q.N[0] * uy[0] + q.N[1] * uy[1] + q.N[2] * uy[2] + q.N[3] * uy[3];
        int ix, iy;
        float tx, ty;
        split_coord(q.x, dx, ix, tx);
        split_coord(q.y, dy, iy, ty);
        float o[6];
        sample_cubic_h(im, ix, iy, tx, ty, o);
        const float r = o[0] - q.I1;
        float mxx = o[1] * o[1], mxy = o[1] * o[2], myy = o[2] * o[2];
        if (exact) {
            mxx += r * o[3];
            mxy += r * o[4];
            myy += r * o[5];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = a; b < 4; ++b) {
                const float nn = q.N[a] * q.N[b];
                const int k = 3 * pair_index(a, b);
                acc[k] += nn * mxx;
                acc[k + 1] += nn * mxy;
                acc[k + 2] += nn * myy;
            }
    }
#pragma unroll
    for (int i = 0; i < 30; ++i) acc[i] = warp_sum_f(acc[i]);
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < 30; ++i) out[32 * (size_t)c + i] = acc[i];
        out[32 * (size_t)c + 30] = 0.f;
        out[32 * (size_t)c + 31] = 0.f;
    }
}

// H V, pixel part: for chunk c and right-hand side k, y_a = sum_b K_ab v_b into node slots.
// V, slots: (node, comp, k) with k fastest; slots: node_chunk_k planes of n_nodes * 2 * K.
__global__ void hv_chunks(const d2ic_frame_t *__restrict__ fp, const float *__restrict__ hess, const float *__restrict__ V,
                          int K, float *__restrict__ slots) {
    const d2ic_frame_t &F = *fp;
    const int c = blockIdx.x;
    __shared__ float Kc[32];
    __shared__ int s_nd[4], s_sl[4];
    if (threadIdx.x < 32) Kc[threadIdx.x] = hess[32 * (size_t)c + threadIdx.x];
    if (threadIdx.x < 4) {
        s_nd[threadIdx.x] = __ldg(F.chunk_nodes + 4 * c + threadIdx.x);
        s_sl[threadIdx.x] = (int)(((unsigned)__ldg(F.chunk_slot + c) >> (8 * threadIdx.x)) & 0xffu);
    }
    __syncthreads();
    const size_t Nn = F.n_nodes;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        float vx[4], vy[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            vx[b] = V[((size_t)s_nd[b] * 2 + 0) * K + k];
            vy[b] = V[((size_t)s_nd[b] * 2 + 1) * K + k];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            float yx = 0.f, yy = 0.f;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int pi = 3 * (a <= b ? pair_index(a, b) : pair_index(b, a));
                yx += Kc[pi] * vx[b] + Kc[pi + 1] * vy[b];
                yy += Kc[pi + 1] * vx[b] + Kc[pi + 2] * vy[b];
            }
            float *sp = slots + ((size_t)s_sl[a] * Nn + s_nd[a]) * 2 * K;
            sp[k] = yx;
            sp[K + k] = yy;
        }
    }
}

// H V, node part: slots (in slot order) / Np + alpha * spring Hessian V; Y (node, comp, k).
__global__ void hv_nodes(const d2ic_frame_t *__restrict__ fp, const float *__restrict__ slots, const float *__restrict__ V,
                         int K, float inv_np, float alpha, float *__restrict__ Y) {
    const d2ic_frame_t &F = *fp;
    const size_t Nn = F.n_nodes;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Nn * K) return;
    const int n = (int)(t / K), k = (int)(t % K);
    float sx = 0.f, sy = 0.f;
    for (int s = 0; s < F.node_chunk_k; ++s) {
        const float *sp = slots + ((size_t)s * Nn + n) * 2 * K;
        sx += sp[k];
        sy += sp[K + k];
    }
    const float vx = V[((size_t)n * 2) * K + k], vy = V[((size_t)n * 2 + 1) * K + k];
    float rx = 0.f, ry = 0.f;
    for (int q = 0; q < F.max_deg; ++q) {
        const int j = __ldg(F.nbr_index + (size_t)q * Nn + n);
        if (j < 0) break;
        const float w = __ldg(F.nbr_weight + (size_t)q * Nn + n);
        rx += w * (vx - V[((size_t)j * 2) * K + k]);
        ry += w * (vy - V[((size_t)j * 2 + 1) * K + k]);
    }
    Y[((size_t)n * 2) * K + k] = sx * inv_np + alpha * rx;
    Y[((size_t)n * 2 + 1) * K + k] = sy * inv_np + alpha * ry;
}

// (d grad_u J / dI2) dI for the images of a batch, one block per chunk: its pixels are located and
// sampled in the frame once (position, residual r, gradient g; one pixel per thread, kept in shared
// memory), then warp w takes images w, w + 8, ...: per pixel dv and grad dv of the image's
// coefficients at the same position, t = dv g + r grad dv, and the chunk's node sums N_a t (lane
// order, then a warp sum) into the image's node slots.  The frame sample is shared by all images
// of the batch instead of being repeated per image.
__global__ void __launch_bounds__(256) mixed_chunks(const d2ic_frame_t *__restrict__ fp, const float2 *__restrict__ u,
                                                    const float *__restrict__ dcoeff, float2 *__restrict__ slots,
                                                    size_t coeff_stride, size_t slot_stride, int n_images) {
    __shared__ int s_ix[D2IC_CHUNK_MAX], s_iy[D2IC_CHUNK_MAX];
    __shared__ float s_tx[D2IC_CHUNK_MAX], s_ty[D2IC_CHUNK_MAX];
    __shared__ float s_r[D2IC_CHUNK_MAX], s_gx[D2IC_CHUNK_MAX], s_gy[D2IC_CHUNK_MAX];
    __shared__ float s_N[4][D2IC_CHUNK_MAX];
    const d2ic_frame_t &F = *fp;
    const int c = blockIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float ux[4], uy[4];
    int nd, slot;
    chunk_nodes_u(F, u, c, lane, ux, uy, nd, slot);
    const int pb = __ldg(F.chunk_begin + c), n = min(__ldg(F.chunk_begin + c + 1) - pb, D2IC_CHUNK_MAX);
    if ((int)threadIdx.x < n) {
        const int i = threadIdx.x;
        const ChunkPix q = unpack(__ldg(reinterpret_cast<const uint4 *>(F.pix) + pb + i));
        const float dx = q.N[0] * ux[0] + q.N[1] * ux[1] + q.N[2] * ux[2] + q.N[3] * ux[3];
        const float dy = q.N[0] * uy[0] + q.N[1] * uy[1] + q.N[2] * uy[2] + q.N[3] * uy[3];
        int ix, iy;
        float tx, ty;
        split_coord(q.x, dx, ix, tx);
        split_coord(q.y, dy, iy, ty);
        const Img im{F.coeff, F.W, F.H, F.cpitch, F.pad};
        float gx, gy;
        s_r[i] = sample_cubic(im, ix, iy, tx, ty, gx, gy) - q.I1;
        s_gx[i] = gx;
        s_gy[i] = gy;
        s_ix[i] = ix;
        s_iy[i] = iy;
        s_tx[i] = tx;
        s_ty[i] = ty;
#pragma unroll
        for (int a = 0; a < 4; ++a) s_N[a][i] = q.N[a];
    }
    __syncthreads();
    for (int b = w; b < n_images; b += 8) {
        const Img dm{dcoeff + (size_t)b * coeff_stride, F.W, F.H, F.cpitch, F.pad};
        float ax[4] = {0.f, 0.f, 0.f, 0.f}, ay[4] = {0.f, 0.f, 0.f, 0.f};
        for (int i = lane; i < n; i += 32) {
            float dgx, dgy;
            const float dv = sample_cubic(dm, s_ix[i], s_iy[i], s_tx[i], s_ty[i], dgx, dgy);
            const float r = s_r[i];
            const float txv = dv * s_gx[i] + r * dgx, tyv = dv * s_gy[i] + r * dgy;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                ax[a] += s_N[a][i] * txv;
                ay[a] += s_N[a][i] * tyv;
            }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            ax[a] = warp_sum_f(ax[a]);
            ay[a] = warp_sum_f(ay[a]);
        }
        if (lane < 4) {
            const float gx = lane == 0 ? ax[0] : lane == 1 ? ax[1] : lane == 2 ? ax[2] : ax[3];
            const float gy = lane == 0 ? ay[0] : lane == 1 ? ay[1] : lane == 2 ? ay[2] : ay[3];
            slots[(size_t)b * slot_stride + (size_t)slot * F.n_nodes + nd] = make_float2(gx, gy);
        }
    }
}

// node sum of float2 slots, scaled; writes column k of out (node, comp, K)
__global__ void slots_to_nodes(const d2ic_frame_t *__restrict__ fp, const float2 *__restrict__ slots, float scale,
                               float *__restrict__ out, int K, int k0, size_t slot_stride) {
    const d2ic_frame_t &F = *fp;
    slots += blockIdx.y * slot_stride;                 // image blockIdx.y of a batch -> column k0 + y
    const int k = k0 + (int)blockIdx.y;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= F.n_nodes) return;
    float sx = 0.f, sy = 0.f;
    for (int s = 0; s < F.node_chunk_k; ++s) {
        const float2 v = slots[(size_t)s * F.n_nodes + n];
        sx += v.x;
        sy += v.y;
    }
    out[((size_t)n * 2) * K + k] = sx * scale;
    out[((size_t)n * 2 + 1) * K + k] = sy * scale;
}

// adjoint of mixed: per pixel the weights of lambda . (d grad_u J / dI2) on the coefficient taps
__global__ void __launch_bounds__(256) mixed_T_scatter(const d2ic_frame_t *__restrict__ fp, const float2 *__restrict__ u,
                                                       const float2 *__restrict__ lam, float scale,
                                                       float *__restrict__ gcoeff) {
    const d2ic_frame_t &F = *fp;
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= F.n_chunks) return;
    float ux[4], uy[4], lx[4], ly[4];
    int nd, slot;
    chunk_nodes_u(F, u, c, lane, ux, uy, nd, slot);
    chunk_nodes_u(F, lam, c, lane, lx, ly, nd, slot);
    const Img im{F.coeff, F.W, F.H, F.cpitch, F.pad};
    const int pb = __ldg(F.chunk_begin + c), pe = __ldg(F.chunk_begin + c + 1);
    for (int p = pb + lane; p < pe; p += 32) {
        const ChunkPix q = unpack(__ldg(reinterpret_cast<const uint4 *>(F.pix) + p));
        const float dx = q.N[0] * ux[0] + q.N[1] * ux[1] + q.N[2] * ux[2] + q.N[3] * ux[3];
        const float dy = q.N[0] * uy[0] + q.N[1] * uy[1] + q.N[2] * uy[2] + q.N[3] * uy[3];
        const float Lx = q.N[0] * lx[0] + q.N[1] * lx[1] + q.N[2] * lx[2] + q.N[3] * lx[3];
        const float Ly = q.N[0] * ly[0] + q.N[1] * ly[1] + q.N[2] * ly[2] + q.N[3] * ly[3];
        int ix, iy;
        float tx, ty;
        split_coord(q.x, dx, ix, tx);
        split_coord(q.y, dy, iy, ty);
        float gx, gy;
        const float r = sample_cubic(im, ix, iy, tx, ty, gx, gy) - q.I1;
        float wx[4], dwx[4], wy[4], dwy[4];
        bspline_w(tx, wx, dwx);
        bspline_w(ty, wy, dwy);
        const float gl = (gx * Lx + gy * Ly) * scale, rl_x = r * Lx * scale, rl_y = r * Ly * scale;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int rr = clampi(iy - 1 + a, -im.pad, im.H - 1 + im.pad) + im.pad;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int cc = clampi(ix - 1 + b, -im.pad, im.W - 1 + im.pad) + im.pad;
                const float w = wy[a] * wx[b] * gl + wy[a] * dwx[b] * rl_x + dwy[a] * wx[b] * rl_y;
                atomicAdd(gcoeff + (size_t)rr * im.cp + cc, w);
            }
        }
    }
}

// transpose of one clamped FIR pass: out[j] = sum over (i, k) with clamp(i - pad + k, 0, n - 1) == j of h[k] in[i],
// i in [0, n + 2 pad); lines are rows (stride 1) or columns (stride = pitch); `lines` independent lines.
__global__ void fir_T(const float *__restrict__ in, int in_len, int in_step, int in_line, float *__restrict__ out,
                      int n, int out_step, int out_line, int lines, int pad) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (j >= n || l >= lines) return;
    const float *src = in + (size_t)l * in_line;
    float acc = 0.f;
    if (j > 0 && j < n - 1) {
        for (int k = -KF_T; k <= KF_T; ++k) {
            const int i = j + pad - k;
            if (i >= 0 && i < in_len) acc += c_fir_t[k + KF_T] * src[(size_t)i * in_step];
        }
    } else if (j == 0) {       // every tap whose index clamps to 0: k <= pad - i
        for (int i = 0; i < in_len && i <= pad + KF_T; ++i) {
            const int m = pad - i;
            if (m < -KF_T) break;
            acc += c_cum_lo[min(m, KF_T) + KF_T] * src[(size_t)i * in_step];
        }
        if (n == 1) {          // a single sample takes every tap
            acc = 0.f;
            for (int i = 0; i < in_len; ++i) acc += c_cum_lo[2 * KF_T] * src[(size_t)i * in_step];
        }
    }
    if (j == n - 1 && n > 1) { // every tap whose index clamps to n - 1: k >= n - 1 + pad - i
        for (int i = in_len - 1; i >= 0; --i) {
            const int m = n - 1 + pad - i;  // need k >= m
            if (m > KF_T) break;
            const float above = c_cum_lo[2 * KF_T] - (m - 1 >= -KF_T ? c_cum_lo[min(m - 1, KF_T) + KF_T] : 0.f);
            acc += above * src[(size_t)i * in_step];
        }
    }
    out[(size_t)l * out_line + (size_t)j * out_step] = acc;
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_hessian_chunks(const d2ic_frame_t *frame_dev, int n_chunks, const float *u, int exact,
                                   float *chunk_hess, void *stream) {
    D2IC_REQUIRE(frame_dev && u && chunk_hess && n_chunks >= 0, "d2ic_hessian_chunks: bad arguments");
    if (n_chunks == 0) return D2IC_OK;
    hessian_chunks<<<(n_chunks * 32 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(frame_dev, (const float2 *)u, exact,
                                                                                  chunk_hess);
    D2IC_CHECK_LAUNCH("hessian_chunks");
    return D2IC_OK;
}

extern "C" int d2ic_hessian_matvec(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, const float *chunk_hess,
                                   const float *V, int K, float inv_np, float alpha_reg, float *slots, float *Y,
                                   void *stream) {
    D2IC_REQUIRE(frame_dev && chunk_hess && V && slots && Y && K >= 1 && n_nodes >= 1, "d2ic_hessian_matvec: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_chunks > 0) {
        hv_chunks<<<n_chunks, K < 128 ? 32 * ((K + 31) / 32) : 128, 0, s>>>(frame_dev, chunk_hess, V, K, slots);
        D2IC_CHECK_LAUNCH("hv_chunks");
    }
    const size_t nt = (size_t)n_nodes * K;
    hv_nodes<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(frame_dev, slots, V, K, inv_np, alpha_reg, Y);
    D2IC_CHECK_LAUNCH("hv_nodes");
    return D2IC_OK;
}

extern "C" int d2ic_mixed_term(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, const float *u,
                               const float *dcoeff, float scale, float *slots, float *out, int K, int k, void *stream) {
    D2IC_REQUIRE(frame_dev && u && dcoeff && slots && out && K >= 1 && k >= 0 && k < K && n_nodes >= 1,
                 "d2ic_mixed_term: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_chunks > 0) {
        mixed_chunks<<<n_chunks, 256, 0, s>>>(frame_dev, (const float2 *)u, dcoeff, (float2 *)slots, 0, 0, 1);
        D2IC_CHECK_LAUNCH("mixed_chunks");
    }
    slots_to_nodes<<<(n_nodes + 255) / 256, 256, 0, s>>>(frame_dev, (const float2 *)slots, scale, out, K, k, 0);
    D2IC_CHECK_LAUNCH("slots_to_nodes");
    return D2IC_OK;
}

extern "C" int d2ic_mixed_term_batch(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                                     const float *u, const float *dcoeff, int n_images, long long coeff_stride,
                                     float scale, float *slots, float *out, int K, int k0, void *stream) {
    D2IC_REQUIRE(frame_dev && u && dcoeff && slots && out && n_nodes >= 1 && node_chunk_k >= 1 && n_images >= 1 &&
                     n_images < 65536 && k0 >= 0 && k0 + n_images <= K && coeff_stride > 0,
                 "d2ic_mixed_term_batch: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t slot_stride = (size_t)node_chunk_k * n_nodes;   // float2 per image
    if (n_chunks > 0) {
        mixed_chunks<<<n_chunks, 256, 0, s>>>(frame_dev, (const float2 *)u, dcoeff, (float2 *)slots,
                                              (size_t)coeff_stride, slot_stride, n_images);
        D2IC_CHECK_LAUNCH("mixed_chunks");
    }
    slots_to_nodes<<<dim3((n_nodes + 255) / 256, n_images), 256, 0, s>>>(frame_dev, (const float2 *)slots, scale, out,
                                                                         K, k0, slot_stride);
    D2IC_CHECK_LAUNCH("slots_to_nodes");
    return D2IC_OK;
}

extern "C" int d2ic_mixed_term_T(const d2ic_frame_t *frame_dev, int n_chunks, const float *u, const float *lam,
                                 float scale, float *gcoeff, void *stream) {
    D2IC_REQUIRE(frame_dev && u && lam && gcoeff, "d2ic_mixed_term_T: bad arguments");
    if (n_chunks == 0) return D2IC_OK;
    mixed_T_scatter<<<(n_chunks * 32 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        frame_dev, (const float2 *)u, (const float2 *)lam, scale, gcoeff);
    D2IC_CHECK_LAUNCH("mixed_T_scatter");
    return D2IC_OK;
}

extern "C" int d2ic_bspline_prefilter_T(const float *gcoeff, int H, int W, int pad, int cpitch, float *tmp, float *gimg,
                                        void *stream) {
    D2IC_REQUIRE(gcoeff && tmp && gimg, "d2ic_bspline_prefilter_T: null pointer");
    D2IC_REQUIRE(H > 1 && W > 1 && pad >= KF_T && cpitch >= W + 2 * pad, "d2ic_bspline_prefilter_T: bad sizes");
    int st = ensure_fir_t();
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const int CW = W + 2 * pad;
    // transpose of the column pass: gcoeff (H + 2 pad rows) -> tmp (H rows), every column of the halo'd width
    fir_T<<<dim3((H + 127) / 128, CW), 128, 0, s>>>(gcoeff, H + 2 * pad, cpitch, 1, tmp, H, cpitch, 1, CW, pad);
    D2IC_CHECK_LAUNCH("prefilter_T cols");
    // transpose of the row pass: tmp (CW columns) -> gimg (W columns), every row
    fir_T<<<dim3((W + 127) / 128, H), 128, 0, s>>>(tmp, CW, 1, cpitch, gimg, W, 1, W, H, pad);
    D2IC_CHECK_LAUNCH("prefilter_T rows");
    return D2IC_OK;
}
