// Reference-domain discrepancy map I_def(x + u(x)) - I_ref(x), bilinear, per ROI pixel
// (d2ic/discrepancy.py:86-127 compute_discrepancy_map_ref).
//
// One warp per chunk of the element-major pixel list: the chunk's four nodal
// displacements are read once, each lane maps its pixels.  A sample is valid
// when its bilinear base (floor of the continuous coordinate) has a right and
// lower neighbour inside the image (the reference's `valid` test); invalid
// residuals are NaN in the map and left out of the RMS.  Every ROI pixel owns
// its own map entry, so the map is written without atomics; the RMS partials
// are per chunk (FP64 sum of r^2 and the valid count) and reduced by the host
// in chunk order.
#include "common.cuh"

namespace d2ic {

// bilinear value at a continuous coordinate (x - 0.5, y - 0.5 already applied); NaN when invalid
__device__ __forceinline__ float bilinear_valid(const float *img, int H, int W, float xc, float yc) {
    const float fj = floorf(xc), fi = floorf(yc);
    if (!(fj >= 0.f && fi >= 0.f && fj < (float)(W - 1) && fi < (float)(H - 1))) return __int_as_float(0x7fc00000);
    const int j0 = (int)fj, i0 = (int)fi;
    const float fx = xc - fj, fy = yc - fi;
    const float *r0 = img + (size_t)i0 * W + j0, *r1 = r0 + W;
    return r0[0] * (1.f - fx) * (1.f - fy) + r0[1] * fx * (1.f - fy) + r1[0] * (1.f - fx) * fy + r1[1] * fx * fy;
}

__global__ void __launch_bounds__(256) discrepancy_kernel(const d2ic_frame_t *__restrict__ F, const float *__restrict__ ref,
                                                          const float *__restrict__ def, const float2 *__restrict__ u,
                                                          float *__restrict__ map, double *__restrict__ sums,
                                                          int *__restrict__ counts) {
    const int lane = threadIdx.x & 31;
    const int W = F->W, H = F->H, nc = F->n_chunks;
    const uint4 *pix = reinterpret_cast<const uint4 *>(F->pix);
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nc; c += (gridDim.x * blockDim.x) >> 5) {
        float ux[4], uy[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const float2 v = u[__ldg(F->chunk_nodes + 4 * c + a)];
            ux[a] = v.x;
            uy[a] = v.y;
        }
        const int pb = __ldg(F->chunk_begin + c), pe = __ldg(F->chunk_begin + c + 1);
        double s = 0.0;
        int cnt = 0;
        for (int p = pb + lane; p < pe; p += 32) {
            const uint4 r4 = __ldg(pix + p);
            const int col = (int)(r4.x & 0xffffu), row = (int)(r4.x >> 16);
            const float xi = __uint_as_float(r4.z), eta = __uint_as_float(r4.w);
            const float a0 = 0.5f * (1.f - xi), a1 = 0.5f * (1.f + xi);
            const float b0 = 0.5f * (1.f - eta), b1 = 0.5f * (1.f + eta);
            const float N0 = a0 * b0, N1 = a1 * b0, N2 = a1 * b1, N3 = a0 * b1;
            const float dx = N0 * ux[0] + N1 * ux[1] + N2 * ux[2] + N3 * ux[3];
            const float dy = N0 * uy[0] + N1 * uy[1] + N2 * uy[2] + N3 * uy[3];
            // pixel centre (col + 0.5, row + 0.5): continuous coordinate (col, row) in the reference,
            // (col + dx, row + dy) in the deformed image
            const float iref = bilinear_valid(ref, H, W, (float)col, (float)row);
            const float idef = bilinear_valid(def, H, W, (float)col + dx, (float)row + dy);
            const float r = idef - iref;
            map[(size_t)row * W + col] = r;
            if (r == r) {
                s += (double)r * (double)r;
                ++cnt;
            }
        }
        s = warp_sum_d(s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (lane == 0) {
            sums[c] = s;
            counts[c] = cnt;
        }
    }
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_discrepancy_map(const d2ic_frame_t *frame_dev, int n_chunks, const float *ref, const float *def,
                                    const float *u, int H, int W, float *map, double *chunk_sums, int *chunk_counts,
                                    void *stream) {
    D2IC_REQUIRE(frame_dev && ref && def && u && map && chunk_sums && chunk_counts,
                 "d2ic_discrepancy_map: null pointer");
    D2IC_REQUIRE(H >= 1 && W >= 1 && n_chunks >= 0, "d2ic_discrepancy_map: bad sizes");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(map, 0xff, sizeof(float) * (size_t)H * W, s);   // all-ones words: NaN
    if (e != cudaSuccess) return cuda_status(e, "discrepancy map fill");
    if (n_chunks == 0) return D2IC_OK;
    const int warps_per_block = 8;
    int blocks = (n_chunks + warps_per_block - 1) / warps_per_block;
    if (blocks > 65535) blocks = 65535;
    discrepancy_kernel<<<blocks, 32 * warps_per_block, 0, s>>>(frame_dev, ref, def, (const float2 *)u, map, chunk_sums,
                                                                 chunk_counts);
    D2IC_CHECK_LAUNCH("discrepancy_kernel");
    return D2IC_OK;
}
