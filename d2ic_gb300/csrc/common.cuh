// Shared device helpers of the d2ic_gb300 library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/d2ic_gb300.h"

namespace d2ic {

// ---- error reporting (thread-local message behind d2ic_last_error_string) ----
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *what);

#define D2IC_CHECK_LAUNCH(what)                                       \
    do {                                                              \
        cudaError_t _e = cudaGetLastError();                          \
        if (_e != cudaSuccess) return ::d2ic::cuda_status(_e, what);  \
    } while (0)

#define D2IC_REQUIRE(cond, ...)                 \
    do {                                        \
        if (!(cond)) {                          \
            ::d2ic::set_error(__VA_ARGS__);     \
            return D2IC_BAD_ARG;                \
        }                                       \
    } while (0)

// ---- cubic B-spline weights for taps -1..2 at fractional offset t in [0,1) ----
__device__ __forceinline__ void bspline_w(float t, float w[4], float dw[4]) {
    const float t2 = t * t, t3 = t2 * t, o = 1.0f - t;
    const float s = 1.0f / 6.0f;
    w[0] = o * o * o * s;
    w[1] = (3.0f * t3 - 6.0f * t2 + 4.0f) * s;
    w[2] = (-3.0f * t3 + 3.0f * t2 + 3.0f * t + 1.0f) * s;
    w[3] = t3 * s;
    dw[0] = -0.5f * o * o;
    dw[1] = 1.5f * t2 - 2.0f * t;
    dw[2] = -1.5f * t2 + t + 0.5f;
    dw[3] = 0.5f * t2;
}

struct Img {
    const float *c;   // halo'd array
    int W, H, cp, pad;
    __device__ __forceinline__ float at(int r, int col) const {   // r, col: pixel indices (may be in the halo)
        return __ldg(c + (size_t)(r + pad) * cp + (col + pad));
    }
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

// The 4x4 tap arithmetic of the cubic B-spline, shared by every source of
// coefficients (global memory, clamped global, shared-memory tile) so that all
// paths produce identical bits.  Taps c[a][b]: row iy - 1 + a, column ix - 1 + b.
__device__ __forceinline__ float cubic_taps(const float c[4][4], float tx, float ty, float &gx, float &gy) {
    float wx[4], dwx[4], wy[4], dwy[4];
    bspline_w(tx, wx, dwx);
    bspline_w(ty, wy, dwy);
    float v = 0.f, ax = 0.f, ay = 0.f;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const float rv = __fmaf_rn(wx[3], c[a][3], __fmaf_rn(wx[2], c[a][2], __fmaf_rn(wx[1], c[a][1], wx[0] * c[a][0])));
        const float rd = __fmaf_rn(dwx[3], c[a][3], __fmaf_rn(dwx[2], c[a][2], __fmaf_rn(dwx[1], c[a][1], dwx[0] * c[a][0])));
        v = __fmaf_rn(wy[a], rv, v);
        ax = __fmaf_rn(wy[a], rd, ax);
        ay = __fmaf_rn(dwy[a], rv, ay);
    }
    gx = ax;
    gy = ay;
    return v;
}

// Cubic B-spline value and gradient at pixel (ix + tx, iy + ty), with integer
// base (ix, iy) and fractional parts tx, ty in [0, 1).  Taps outside the halo'd
// array clamp to its border, where the coefficients equal the edge value.
__device__ __forceinline__ float sample_cubic(const Img &im, int ix, int iy, float tx, float ty,
                                              float &gx, float &gy) {
    float c[4][4];
    const int x0 = ix - 1, y0 = iy - 1;
    if (x0 >= -im.pad && x0 + 3 < im.W + im.pad && y0 >= -im.pad && y0 + 3 < im.H + im.pad) {
        const float *base = im.c + (size_t)(y0 + im.pad) * im.cp + (x0 + im.pad);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) c[a][b] = __ldg(base + (size_t)a * im.cp + b);
    } else {
        int cx[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) cx[b] = clampi(x0 + b, -im.pad, im.W - 1 + im.pad);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int r = clampi(y0 + a, -im.pad, im.H - 1 + im.pad);
#pragma unroll
            for (int b = 0; b < 4; ++b) c[a][b] = im.at(r, cx[b]);
        }
    }
    return cubic_taps(c, tx, ty, gx, gy);
}

// Same, with the taps read from a shared-memory tile whose element (0, 0) is the
// tap at (row ly, column lx) relative to the tile; the caller guarantees
// 0 <= lx <= tw - 4 and 0 <= ly <= th - 4.
__device__ __forceinline__ float sample_cubic_tile(const float *tile, int tw, int lx, int ly, float tx, float ty,
                                                   float &gx, float &gy) {
    float c[4][4];
    const float *base = tile + ly * tw + lx;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) c[a][b] = base[a * tw + b];
    return cubic_taps(c, tx, ty, gx, gy);
}

// Bilinear value and gradient at pixel (ix + tx, iy + ty); taps clamped into the image.
__device__ __forceinline__ float sample_linear(const Img &im, int ix, int iy, float tx, float ty,
                                               float &gx, float &gy) {
    const int x0 = clampi(ix, 0, im.W - 1), x1 = clampi(ix + 1, 0, im.W - 1);
    const int y0 = clampi(iy, 0, im.H - 1), y1 = clampi(iy + 1, 0, im.H - 1);
    const float i00 = im.at(y0, x0), i10 = im.at(y0, x1), i01 = im.at(y1, x0), i11 = im.at(y1, x1);
    gx = (1.f - ty) * (i10 - i00) + ty * (i11 - i01);
    gy = (1.f - tx) * (i01 - i00) + tx * (i11 - i10);
    return (1.f - tx) * (1.f - ty) * i00 + tx * (1.f - ty) * i10 + (1.f - tx) * ty * i01 + tx * ty * i11;
}

template <int KIND>
__device__ __forceinline__ float sample(const Img &im, int ix, int iy, float tx, float ty, float &gx, float &gy) {
    if (KIND == D2IC_INTERP_LINEAR) return sample_linear(im, ix, iy, tx, ty, gx, gy);
    return sample_cubic(im, ix, iy, tx, ty, gx, gy);
}

// floor(d) clamped to +-2^24 before the integer conversion, so that huge or
// NaN coordinates give a far-outside (clamped) tap instead of a saturated
// integer that could overflow the bounds arithmetic.  NaN propagates through
// the fraction, never through an index.
__device__ __forceinline__ float safe_floor(float d) {
    return fminf(fmaxf(floorf(d), -16777216.0f), 16777216.0f);
}

// Split an image-index coordinate x = i + d (i integer pixel, d small
// displacement) into integer base and fraction in [0,1) without forming the
// rounded sum i + d.
__device__ __forceinline__ void split_coord(int i, float d, int &ib, float &t) {
    const float fl = safe_floor(d);
    ib = i + (int)fl;
    t = d - fl;
}

// Double-float ("hi + lo") accumulation: TwoSum / TwoProduct are error-free
// transformations in FP32 (Knuth; Ogita, Rump & Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 2005), giving ~48-bit sums at FP32 issue
// rate.  GB300's FP64 pipe runs at a small fraction of FP32, so the inner
// products of the CG control are accumulated this way and converted to FP64
// once per group.  df_add is commutative bit for bit, so xor-butterfly warp
// reductions leave every lane with the same value.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
    const DF s = df_two_sum(x.hi, y.hi);
    const float e = s.lo + (x.lo + y.lo);
    const float h = s.hi + e;
    return {h, e - (h - s.hi)};
}
__device__ __forceinline__ DF df_prod(float a, float b) {
    const float p = a * b;
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ DF df_warp_sum(DF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const DF w = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = df_add(v, w);
    }
    return v;
}
__device__ __forceinline__ double df_to_double(DF v) { return (double)v.hi + (double)v.lo; }

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace d2ic
