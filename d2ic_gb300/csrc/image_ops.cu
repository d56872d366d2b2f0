// Image preparation kernels: cubic B-spline prefilter, halo padding, point
// sampling and pixel-record packing.
//
// The prefilter computes the interpolating cubic B-spline coefficients of the
// edge-extended image.  The exact inverse of the sampled B-spline kernel
// (1, 4, 1)/6 has impulse response h[k] = sqrt(3) * z^|k|, z = sqrt(3) - 2
// (Unser, "B-spline signal processing", IEEE TSP 1993).  |z|^17 < 2e-10, so a
// 33-tap FIR (|k| <= 16) applied separably to the edge-replicated image gives
// the coefficients to FP32 precision with fully parallel, coalesced passes
// (instead of the sequential causal/anti-causal recursion).
#include "common.cuh"

namespace d2ic {

constexpr int KF = 16;                 // FIR half-length
__constant__ float c_fir[2 * KF + 1];
static bool g_fir_ready[64] = {false};

static int ensure_fir() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && g_fir_ready[dev]) return D2IC_OK;
    float h[2 * KF + 1];
    const double z = 1.7320508075688772 - 2.0;
    for (int k = -KF; k <= KF; ++k) {
        double v = 1.7320508075688772;
        for (int i = 0; i < (k < 0 ? -k : k); ++i) v *= z;
        h[k + KF] = (float)v;
    }
    cudaError_t e = cudaMemcpyToSymbol(c_fir, h, sizeof(h));
    if (e != cudaSuccess) return cuda_status(e, "prefilter constants");
    if (dev >= 0 && dev < 64) g_fir_ready[dev] = true;
    return D2IC_OK;
}

// rows: tmp[y][cx] = sum_k h[k] img[y][clamp(cx - pad + k)], cx in [0, W + 2 pad); image
// blockIdx.z of a batch (contiguous images and buffers).  T: float or 8-bit camera pixels.
template <class T>
__global__ void __launch_bounds__(256) prefilter_rows(const T *__restrict__ img, int H, int W, int pad,
                                                      int cpitch, float *__restrict__ tmp) {
    __shared__ float s[256 + 2 * KF];
    img += (size_t)blockIdx.z * H * W;
    tmp += (size_t)blockIdx.z * H * cpitch;
    const int y = blockIdx.y;
    const int cx0 = blockIdx.x * 256;
    const T *row = img + (size_t)y * W;
    for (int i = threadIdx.x; i < 256 + 2 * KF; i += 256) {
        const int src = clampi(cx0 - pad - KF + i, 0, W - 1);
        s[i] = (float)__ldg(row + src);
    }
    __syncthreads();
    const int cx = cx0 + threadIdx.x;
    if (cx < W + 2 * pad) {
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k <= 2 * KF; ++k) acc += c_fir[k] * s[threadIdx.x + k];
        tmp[(size_t)y * cpitch + cx] = acc;
    }
}

// columns: coeff[cy][cx] = sum_k h[k] tmp[clamp(cy - pad + k)][cx], cy in [0, H + 2 pad)
constexpr int CT_W = 32, CT_H = 64;
__global__ void __launch_bounds__(256) prefilter_cols(const float *__restrict__ tmp, int H, int W, int pad,
                                                      int cpitch, float *__restrict__ coeff) {
    __shared__ float s[CT_H + 2 * KF][CT_W + 1];
    tmp += (size_t)blockIdx.z * H * cpitch;
    coeff += (size_t)blockIdx.z * (H + 2 * pad) * cpitch;
    const int cx = blockIdx.x * CT_W + threadIdx.x;
    const int cy0 = blockIdx.y * CT_H;
    const int CW = W + 2 * pad;
    for (int r = threadIdx.y; r < CT_H + 2 * KF; r += 8) {
        const int src = clampi(cy0 - pad - KF + r, 0, H - 1);
        s[r][threadIdx.x] = (cx < CW) ? tmp[(size_t)src * cpitch + cx] : 0.f;
    }
    __syncthreads();
    if (cx >= CW) return;
    for (int r = threadIdx.y; r < CT_H; r += 8) {
        const int cy = cy0 + r;
        if (cy >= H + 2 * pad) break;
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k <= 2 * KF; ++k) acc += c_fir[k] * s[r + k][threadIdx.x];
        coeff[(size_t)cy * cpitch + cx] = acc;
    }
}

template <class T>
__global__ void pad_image_kernel(const T *__restrict__ img, int H, int W, int pad, int cpitch,
                                 float *__restrict__ out) {
    const int cx = blockIdx.x * blockDim.x + threadIdx.x;
    const int cy = blockIdx.y;
    if (cx >= W + 2 * pad) return;
    const int sy = clampi(cy - pad, 0, H - 1), sx = clampi(cx - pad, 0, W - 1);
    out[(size_t)cy * cpitch + cx] = (float)__ldg(img + (size_t)sy * W + sx);
}

template <class T>
static int prefilter_one(const T *img, int H, int W, int pad, int cpitch, float *tmp, float *coeff, cudaStream_t s,
                         const char *name) {
    D2IC_REQUIRE(img && tmp && coeff, "%s: null pointer", name);
    D2IC_REQUIRE(H > 0 && W > 0 && H < 65536 && W < 65536, "%s: bad image size %dx%d", name, H, W);
    D2IC_REQUIRE(pad >= KF && cpitch >= W + 2 * pad, "%s: need pad >= %d and cpitch >= W + 2 pad", name, KF);
    int st = ensure_fir();
    if (st) return st;
    const int CW = W + 2 * pad;
    prefilter_rows<T><<<dim3((CW + 255) / 256, H), 256, 0, s>>>(img, H, W, pad, cpitch, tmp);
    D2IC_CHECK_LAUNCH("prefilter_rows");
    prefilter_cols<<<dim3((CW + CT_W - 1) / CT_W, (H + 2 * pad + CT_H - 1) / CT_H), dim3(CT_W, 8), 0, s>>>(
        tmp, H, W, pad, cpitch, coeff);
    D2IC_CHECK_LAUNCH("prefilter_cols");
    return D2IC_OK;
}

template <class T>
static int pad_one(const T *img, int H, int W, int pad, int cpitch, float *out, cudaStream_t s, const char *name) {
    D2IC_REQUIRE(img && out, "%s: null pointer", name);
    D2IC_REQUIRE(H > 0 && W > 0 && H < 65536 && W < 65536, "%s: bad image size %dx%d", name, H, W);
    D2IC_REQUIRE(pad >= 0 && cpitch >= W + 2 * pad, "%s: need cpitch >= W + 2 pad", name);
    const int CW = W + 2 * pad;
    pad_image_kernel<T><<<dim3((CW + 255) / 256, H + 2 * pad), 256, 0, s>>>(img, H, W, pad, cpitch, out);
    D2IC_CHECK_LAUNCH("pad_image");
    return D2IC_OK;
}

template <int KIND>
__global__ void sample_points_kernel(Img im, const float2 *__restrict__ xy, int n, float *val, float *gx,
                                     float *gy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 p = xy[i];
    const float fx = safe_floor(p.x), fy = safe_floor(p.y);
    float a, b;
    const float v = sample<KIND>(im, (int)fx, (int)fy, p.x - fx, p.y - fy, a, b);
    val[i] = v;
    if (gx) gx[i] = a;
    if (gy) gy[i] = b;
}

template <int KIND>
__global__ void pack_pixels_kernel(const int2 *__restrict__ colrow, const float2 *__restrict__ xieta, int n,
                                   Img im, uint4 *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 cr = colrow[i];
    const float2 xe = xieta[i];
    float a, b;
    const float I1 = sample<KIND>(im, cr.x, cr.y, 0.f, 0.f, a, b);
    out[i] = make_uint4((uint32_t)cr.x | ((uint32_t)cr.y << 16), __float_as_uint(I1), __float_as_uint(xe.x),
                        __float_as_uint(xe.y));
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_bspline_prefilter_batch(const float *img, int n_images, int H, int W, int pad, int cpitch,
                                            float *tmp, float *coeff, void *stream) {
    D2IC_REQUIRE(img && tmp && coeff, "d2ic_bspline_prefilter_batch: null pointer");
    D2IC_REQUIRE(n_images >= 1 && n_images < 65536, "d2ic_bspline_prefilter_batch: bad image count %d", n_images);
    D2IC_REQUIRE(H > 0 && W > 0 && H < 65536 && W < 65536, "d2ic_bspline_prefilter_batch: bad image size %dx%d", H, W);
    D2IC_REQUIRE(pad >= KF && cpitch >= W + 2 * pad,
                 "d2ic_bspline_prefilter_batch: need pad >= %d and cpitch >= W + 2 pad", KF);
    int st = ensure_fir();
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const int CW = W + 2 * pad;
    prefilter_rows<float><<<dim3((CW + 255) / 256, H, n_images), 256, 0, s>>>(img, H, W, pad, cpitch, tmp);
    D2IC_CHECK_LAUNCH("prefilter_rows");
    prefilter_cols<<<dim3((CW + CT_W - 1) / CT_W, (H + 2 * pad + CT_H - 1) / CT_H, n_images), dim3(CT_W, 8), 0, s>>>(
        tmp, H, W, pad, cpitch, coeff);
    D2IC_CHECK_LAUNCH("prefilter_cols");
    return D2IC_OK;
}

extern "C" int d2ic_bspline_prefilter(const float *img, int H, int W, int pad, int cpitch, float *tmp,
                                      float *coeff, void *stream) {
    return prefilter_one(img, H, W, pad, cpitch, tmp, coeff, (cudaStream_t)stream, "d2ic_bspline_prefilter");
}

extern "C" int d2ic_bspline_prefilter_u8(const unsigned char *img, int H, int W, int pad, int cpitch, float *tmp,
                                         float *coeff, void *stream) {
    return prefilter_one(img, H, W, pad, cpitch, tmp, coeff, (cudaStream_t)stream, "d2ic_bspline_prefilter_u8");
}

extern "C" int d2ic_pad_image(const float *img, int H, int W, int pad, int cpitch, float *out, void *stream) {
    return pad_one(img, H, W, pad, cpitch, out, (cudaStream_t)stream, "d2ic_pad_image");
}

extern "C" int d2ic_pad_image_u8(const unsigned char *img, int H, int W, int pad, int cpitch, float *out,
                                 void *stream) {
    return pad_one(img, H, W, pad, cpitch, out, (cudaStream_t)stream, "d2ic_pad_image_u8");
}

extern "C" int d2ic_sample_points(const float *coeff, int H, int W, int pad, int cpitch, int kind, const float *xy,
                                  int n, float *val, float *gx, float *gy, void *stream) {
    D2IC_REQUIRE(coeff && xy && val, "d2ic_sample_points: null pointer");
    D2IC_REQUIRE(n >= 0 && H > 0 && W > 0 && pad >= 0 && cpitch >= W + 2 * pad, "d2ic_sample_points: bad sizes");
    D2IC_REQUIRE(kind == D2IC_INTERP_CUBIC || kind == D2IC_INTERP_LINEAR, "d2ic_sample_points: unknown kind %d", kind);
    if (n == 0) return D2IC_OK;
    Img im{coeff, W, H, cpitch, pad};
    const int nb = (n + 255) / 256;
    if (kind == D2IC_INTERP_CUBIC)
        sample_points_kernel<D2IC_INTERP_CUBIC><<<nb, 256, 0, (cudaStream_t)stream>>>(im, (const float2 *)xy, n, val, gx, gy);
    else
        sample_points_kernel<D2IC_INTERP_LINEAR><<<nb, 256, 0, (cudaStream_t)stream>>>(im, (const float2 *)xy, n, val, gx, gy);
    D2IC_CHECK_LAUNCH("sample_points");
    return D2IC_OK;
}

extern "C" int d2ic_pack_pixels(const int *colrow, const float *xieta, int n, const float *coeff1, int H, int W,
                                int pad, int cpitch, int kind, d2ic_pixrec_t *out, void *stream) {
    D2IC_REQUIRE(colrow && xieta && coeff1 && out, "d2ic_pack_pixels: null pointer");
    D2IC_REQUIRE(n >= 0 && H > 0 && W > 0 && H < 65536 && W < 65536 && cpitch >= W + 2 * pad,
                 "d2ic_pack_pixels: bad sizes");
    D2IC_REQUIRE(kind == D2IC_INTERP_CUBIC || kind == D2IC_INTERP_LINEAR, "d2ic_pack_pixels: unknown kind %d", kind);
    if (n == 0) return D2IC_OK;
    Img im{coeff1, W, H, cpitch, pad};
    const int nb = (n + 255) / 256;
    if (kind == D2IC_INTERP_CUBIC)
        pack_pixels_kernel<D2IC_INTERP_CUBIC><<<nb, 256, 0, (cudaStream_t)stream>>>((const int2 *)colrow, (const float2 *)xieta, n, im, (uint4 *)out);
    else
        pack_pixels_kernel<D2IC_INTERP_LINEAR><<<nb, 256, 0, (cudaStream_t)stream>>>((const int2 *)colrow, (const float2 *)xieta, n, im, (uint4 *)out);
    D2IC_CHECK_LAUNCH("pack_pixels");
    return D2IC_OK;
}
