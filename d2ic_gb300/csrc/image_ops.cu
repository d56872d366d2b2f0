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
// blockIdx.z of a batch (contiguous images and buffers).  T: float or 8-bit camera pixels.  A block
// takes an even share (at most RT_OUT outputs, a multiple of 4) of one row, its edge-extended
// segment staged once in shared memory; a thread makes 4 consecutive outputs from 10 float4 reads
// of the segment (each output's taps still summed in order k = 0 .. 2 KF).  The host sizes the
// block to the share (rows_launch), so that no warp idles on 1024- or 2048-pixel rows.
constexpr int RT_OUT = 4096;
template <class T>
__global__ void __launch_bounds__(1024) prefilter_rows(const T *__restrict__ img, int H, int W, int pad,
                                                      int cpitch, float *__restrict__ tmp) {
    __shared__ __align__(16) float s[RT_OUT + 2 * KF + 4];
    img += (size_t)blockIdx.z * H * W;
    tmp += (size_t)blockIdx.z * H * cpitch;
    const int y = blockIdx.y;
    const int CW = W + 2 * pad;
    const int per = (((CW + gridDim.x - 1) / gridDim.x) + 3) & ~3;   // <= RT_OUT
    const int cx0 = blockIdx.x * per;
    const int n_out = min(per, CW - cx0);
    const T *row = img + (size_t)y * W;
    for (int i = threadIdx.x; i < ((n_out + 3) & ~3) + 2 * KF + 4; i += blockDim.x) {
        const int src = clampi(cx0 - pad - KF + i, 0, W - 1);
        s[i] = (float)__ldg(row + src);
    }
    __syncthreads();
    const int o0 = 4 * threadIdx.x;
    if (o0 >= n_out) return;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const float4 *s4 = reinterpret_cast<const float4 *>(s) + threadIdx.x;
#pragma unroll
    for (int m = 0; m < (2 * KF + 4) / 4 + 1; ++m) {
        const float4 q = s4[m];
        const float v[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int e = 0; e < 4; ++e)
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const int k = 4 * m + e - o;
                if (k >= 0 && k <= 2 * KF) acc[o] += c_fir[k] * v[e];
            }
    }
    float *out = tmp + (size_t)y * cpitch + cx0 + o0;
#pragma unroll
    for (int o = 0; o < 4; ++o)
        if (o0 + o < n_out) out[o] = acc[o];
}

// columns: coeff[cy][cx] = sum_k h[k] tmp[clamp(cy - pad + k)][cx], cy in [0, H + 2 pad).  A block
// takes CT_W columns x CT_H rows; thread (x, y) makes the CT_R consecutive rows y CT_R .. of column x
// from CT_R + 2 KF shared-memory reads (sliding window, taps in order k = 0 .. 2 KF per output).
constexpr int CT_W = 32, CT_H = 128, CT_R = CT_H / 8;
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
    const int r0 = threadIdx.y * CT_R;
    float acc[CT_R];
#pragma unroll
    for (int o = 0; o < CT_R; ++o) acc[o] = 0.f;
#pragma unroll
    for (int j = 0; j < CT_R + 2 * KF; ++j) {
        const float v = s[r0 + j][threadIdx.x];
#pragma unroll
        for (int o = 0; o < CT_R; ++o) {
            const int k = j - o;
            if (k >= 0 && k <= 2 * KF) acc[o] += c_fir[k] * v;
        }
    }
#pragma unroll
    for (int o = 0; o < CT_R; ++o) {
        const int cy = cy0 + r0 + o;
        if (cy < H + 2 * pad) coeff[(size_t)cy * cpitch + cx] = acc[o];
    }
}

// blocks per row and threads per block of prefilter_rows for rows of CW outputs: the fewest blocks
// of at most RT_OUT outputs, and one thread per 4 outputs of the (even, 4-aligned) share
struct RowsLaunch {
    unsigned blocks, threads;
};
static RowsLaunch rows_launch(int CW) {
    const int blocks = (CW + RT_OUT - 1) / RT_OUT;
    const int per = (((CW + blocks - 1) / blocks) + 3) & ~3;
    const int quads = per / 4;
    return RowsLaunch{(unsigned)blocks, (unsigned)(((quads + 31) / 32) * 32)};
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
    const RowsLaunch rl = rows_launch(CW);
    prefilter_rows<T><<<dim3(rl.blocks, H), rl.threads, 0, s>>>(img, H, W, pad, cpitch, tmp);
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
    const RowsLaunch rl = rows_launch(CW);
    prefilter_rows<float><<<dim3(rl.blocks, H, n_images), rl.threads, 0, s>>>(img, H, W, pad, cpitch, tmp);
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
