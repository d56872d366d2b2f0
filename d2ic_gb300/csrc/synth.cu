// Synthetic speckle frames on the device, for benchmark streams and tests.
//
// No counterpart in the reference, which reads camera images from disk.  A
// speckle pattern is a sum of Gaussian dots; a deformed frame evaluates the
// same dot field at the back-mapped pixel centre x = phi^-1(y) for an affine
// map phi, so that brightness constancy I2(phi(x)) = I1(x) holds up to noise.
// The dots are bucketed on the host into square cells at least as wide as the
// largest cut-off radius; a pixel visits the 3 x 3 cells around x and sums its
// dots in cell order (deterministic, no atomics).
//
// d2ic_speckle_finish scales the raw sum to grey levels, adds N(0, sigma^2)
// noise from a counter-based generator (SplitMix64 of seed and pixel index,
// Steele, Lea & Flood, OOPSLA 2014; Box-Muller transform, 1958) and writes
// float32 or 8-bit pixels (rounded, clamped to [0, 255]) like a camera.
#include "common.cuh"

namespace d2ic {

struct Affine6 {
    double m[6];   // x = m0 + m1 yx + m2 yy, y = m3 + m4 yx + m5 yy (pixel-centre coordinates)
};

__global__ void __launch_bounds__(256) render_speckle_kernel(const float4 *__restrict__ dots,
                                                             const int *__restrict__ cell_start, float cell_px,
                                                             int gw, int gh, float cut2, Affine6 A, int H, int W,
                                                             float *__restrict__ out) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * 8 + threadIdx.y;
    if (i >= H || j >= W) return;
    const double yx = j + 0.5, yy = i + 0.5;
    const float x = (float)(A.m[0] + A.m[1] * yx + A.m[2] * yy);
    const float y = (float)(A.m[3] + A.m[4] * yx + A.m[5] * yy);
    const int cx = (int)floorf(x / cell_px), cy = (int)floorf(y / cell_px);
    float acc = 0.f;
    for (int gy = cy - 1; gy <= cy + 1; ++gy) {
        if (gy < 0 || gy >= gh) continue;
        for (int gx = cx - 1; gx <= cx + 1; ++gx) {
            if (gx < 0 || gx >= gw) continue;
            const int c = gy * gw + gx;
            const int k1 = __ldg(cell_start + c + 1);
            for (int k = __ldg(cell_start + c); k < k1; ++k) {
                const float4 d = __ldg(dots + k);
                const float dx = x - d.x, dy = y - d.y;
                const float d2 = dx * dx + dy * dy, s2 = d.z * d.z;
                if (d2 <= cut2 * s2) acc += d.w * expf(-d2 / (2.f * s2));
            }
        }
    }
    out[(size_t)i * W + j] = acc;
}

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <class T>
__global__ void __launch_bounds__(256) speckle_finish_kernel(const float *__restrict__ raw, long long n, float lo,
                                                             float scale, float sigma, unsigned long long seed,
                                                             T *__restrict__ out) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float v = 20.f + (raw[p] - lo) * scale;
    if (sigma > 0.f) {
        const unsigned long long r = splitmix64(seed * 0x632BE59BD9B4E019ull + (unsigned long long)p);
        const float u1 = ((float)(r >> 40) + 1.f) * (1.f / 16777216.f);          // (0, 1]
        const float u2 = (float)((r >> 16) & 0xFFFFFFull) * (1.f / 16777216.f);    // [0, 1)
        v += sigma * sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
    }
    if constexpr (sizeof(T) == 1)
        out[p] = (T)fminf(fmaxf(rintf(v), 0.f), 255.f);
    else
        out[p] = v;
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_render_speckle(const float *dots, const int *cell_start, float cell_px, int gw, int gh,
                                   float cutoff_sigmas, const double *inv_affine, int H, int W, float *out,
                                   void *stream) {
    D2IC_REQUIRE(dots && cell_start && inv_affine && out, "d2ic_render_speckle: null pointer");
    D2IC_REQUIRE(H > 0 && W > 0 && gw > 0 && gh > 0 && cell_px > 0.f, "d2ic_render_speckle: bad sizes");
    Affine6 A;                                   // inv_affine is a host array; the map travels by value
    for (int k = 0; k < 6; ++k) A.m[k] = inv_affine[k];
    render_speckle_kernel<<<dim3((W + 31) / 32, (H + 7) / 8), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        (const float4 *)dots, cell_start, cell_px, gw, gh, cutoff_sigmas * cutoff_sigmas, A, H, W, out);
    D2IC_CHECK_LAUNCH("render_speckle");
    return D2IC_OK;
}

extern "C" int d2ic_speckle_finish(const float *raw, long long n, float lo, float scale, float sigma,
                                   unsigned long long seed, int out_u8, void *out, void *stream) {
    D2IC_REQUIRE(raw && out && n >= 0, "d2ic_speckle_finish: bad arguments");
    if (n == 0) return D2IC_OK;
    const unsigned nb = (unsigned)((n + 255) / 256);
    if (out_u8)
        speckle_finish_kernel<unsigned char><<<nb, 256, 0, (cudaStream_t)stream>>>(raw, n, lo, scale, sigma, seed,
                                                                                   (unsigned char *)out);
    else
        speckle_finish_kernel<float><<<nb, 256, 0, (cudaStream_t)stream>>>(raw, n, lo, scale, sigma, seed,
                                                                           (float *)out);
    D2IC_CHECK_LAUNCH("speckle_finish");
    return D2IC_OK;
}
