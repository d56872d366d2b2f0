// Pixel-asset setup on the device: the element of every pixel on a tensor-grid
// mesh (d2ic/pixel_assets.py:135-237 for the grids mask_to_mesh builds), and the
// local (xi, eta) coordinates of every pixel in its Q4 element by Newton's method
// (d2ic/pixel_assets.py:277-294, the reference's _newton_quadrature), in FP64.
//
// Each step is the host restatement's operation sequence with correctly rounded
// FP64 intrinsics (no contraction into FMAs): shape functions and derivatives,
// residual and Jacobian as left-to-right sums of products, the 2x2 solve by LU
// with partial pivoting, and the update.  A pixel whose update is exactly zero
// keeps its coordinates for every later step, so it stops there.  The results
// are therefore bit-identical to the host restatement.
#include "common.cuh"

namespace d2ic {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

__global__ void __launch_bounds__(256) local_coords_kernel(const double *__restrict__ pc, const int *__restrict__ pn,
                                                           const double *__restrict__ nodes, long long n, int iters,
                                                           double *__restrict__ xi_out, double *__restrict__ eta_out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        double X[4], Y[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int k = pn[4 * p + a];
            X[a] = nodes[2 * (long long)k];
            Y[a] = nodes[2 * (long long)k + 1];
        }
        const double px = pc[2 * p], py = pc[2 * p + 1];
        double xi = 0.0, eta = 0.0;
        for (int it = 0; it < iters; ++it) {
            const double om_x = sub(1.0, xi), op_x = add(1.0, xi), om_e = sub(1.0, eta), op_e = add(1.0, eta);
            const double n0 = mul(mul(0.25, om_x), om_e), n1 = mul(mul(0.25, op_x), om_e);
            const double n2 = mul(mul(0.25, op_x), op_e), n3 = mul(mul(0.25, om_x), op_e);
            const double dx0 = mul(-0.25, om_e), dx1 = mul(0.25, om_e), dx2 = mul(0.25, op_e), dx3 = mul(-0.25, op_e);
            const double de0 = mul(-0.25, om_x), de1 = mul(-0.25, op_x), de2 = mul(0.25, op_x), de3 = mul(0.25, om_x);
            const double fx = sub(add(add(add(mul(n0, X[0]), mul(n1, X[1])), mul(n2, X[2])), mul(n3, X[3])), px);
            const double fy = sub(add(add(add(mul(n0, Y[0]), mul(n1, Y[1])), mul(n2, Y[2])), mul(n3, Y[3])), py);
            const double j11 = add(add(add(mul(dx0, X[0]), mul(dx1, X[1])), mul(dx2, X[2])), mul(dx3, X[3]));
            const double j21 = add(add(add(mul(dx0, Y[0]), mul(dx1, Y[1])), mul(dx2, Y[2])), mul(dx3, Y[3]));
            const double j12 = add(add(add(mul(de0, X[0]), mul(de1, X[1])), mul(de2, X[2])), mul(de3, X[3]));
            const double j22 = add(add(add(mul(de0, Y[0]), mul(de1, Y[1])), mul(de2, Y[2])), mul(de3, Y[3]));
            // LU with partial pivoting: rows swapped when |a21| > |a11|
            const bool swap = fabs(j21) > fabs(j11);
            const double p11 = swap ? j21 : j11, p12 = swap ? j22 : j12, p21 = swap ? j11 : j21, p22 = swap ? j12 : j22;
            const double q1 = swap ? fy : fx, q2 = swap ? fx : fy;
            const double l21 = dvd(p21, p11);
            const double d2 = dvd(sub(q2, mul(l21, q1)), sub(p22, mul(l21, p12)));
            const double d1 = dvd(sub(q1, mul(p12, d2)), p11);
            xi = sub(xi, d1);
            eta = sub(eta, d2);
            const bool moving = d1 != 0.0 || d2 != 0.0 || !isfinite(d1) || !isfinite(d2);
            if (!moving) break;
        }
        xi_out[p] = xi;
        eta_out[p] = eta;
    }
}

// number of entries of the ascending array g[0..n) that are <= x (searchsorted, side "right")
__device__ __forceinline__ int count_le(const double *g, int n, double x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (g[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// The four cells around the pixel whose closed rectangles can hold it (the last grid line <= x
// and the one before, likewise in y); the lowest element index among those that do.
__global__ void __launch_bounds__(256) structured_assign_kernel(const double *__restrict__ pc, long long n,
                                                                const double *__restrict__ gx, int nx,
                                                                const double *__restrict__ gy, int ny,
                                                                const long long *__restrict__ cell,
                                                                long long *__restrict__ elts) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const double x = pc[2 * p], y = pc[2 * p + 1];
        const int ixr = count_le(gx, nx, x) - 1, iyr = count_le(gy, ny, y) - 1;
        long long best = -1;
        for (int dx = 0; dx < 2; ++dx) {
            const int cx = ixr - dx;
            if (cx < 0 || cx > nx - 2 || !(gx[cx] <= x && x <= gx[cx + 1])) continue;
            for (int dy = 0; dy < 2; ++dy) {
                const int cy = iyr - dy;
                if (cy < 0 || cy > ny - 2 || !(gy[cy] <= y && y <= gy[cy + 1])) continue;
                const long long e = cell[(long long)cy * (nx - 1) + cx];
                if (e >= 0 && (best < 0 || e < best)) best = e;
            }
        }
        elts[p] = best;
    }
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_structured_assign(const double *pixel_coords, long long n_pix, const double *gx, int nx,
                                      const double *gy, int ny, const long long *cell, long long *elts,
                                      void *stream) {
    D2IC_REQUIRE(n_pix >= 0 && nx >= 2 && ny >= 2, "d2ic_structured_assign: bad sizes");
    if (n_pix == 0) return D2IC_OK;
    D2IC_REQUIRE(pixel_coords && gx && gy && cell && elts, "d2ic_structured_assign: null pointer");
    long long blocks = (n_pix + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    structured_assign_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(pixel_coords, n_pix, gx, nx, gy, ny, cell,
                                                                            elts);
    D2IC_CHECK_LAUNCH("structured_assign_kernel");
    return D2IC_OK;
}

extern "C" int d2ic_local_coordinates(const double *pixel_coords, const int *pixel_nodes, const double *nodes,
                                      long long n_pix, int iters, double *xi, double *eta, void *stream) {
    D2IC_REQUIRE(n_pix >= 0 && iters >= 0, "d2ic_local_coordinates: bad sizes");
    if (n_pix == 0) return D2IC_OK;
    D2IC_REQUIRE(pixel_coords && pixel_nodes && nodes && xi && eta, "d2ic_local_coordinates: null pointer");
    long long blocks = (n_pix + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    local_coords_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(pixel_coords, pixel_nodes, nodes, n_pix, iters,
                                                                       xi, eta);
    D2IC_CHECK_LAUNCH("local_coords_kernel");
    return D2IC_OK;
}
