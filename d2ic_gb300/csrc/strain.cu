// Nodal Green-Lagrange strain by weighted least squares over the node's
// neighbours (d2ic/strain.py:11-114): per node, grad u from the 2x2 normal
// equations (sum w dX dX^T + eps I), F = I + grad u, E = (F^T F - I) / 2,
// Voigt [E11, E22, E12].  One thread per node, FP64 accumulation.
#include "common.cuh"

namespace d2ic {

__global__ void strain_kernel(const float2 *__restrict__ u, const float2 *__restrict__ X, const int *__restrict__ idx,
                              const int *__restrict__ deg, int n, int md, float L, float eps, float *__restrict__ voigt,
                              float *__restrict__ Fout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 xi = X[i], ui = u[i];
    const int d = deg[i];
    double a11 = 0, a12 = 0, a22 = 0, b0x = 0, b0y = 0, b1x = 0, b1y = 0;
    for (int k = 0; k < md; ++k) {
        // entries beyond the degree get weight 0 (their index is replaced by 0 in the reference)
        if (k >= d) break;
        const int j = idx[(size_t)i * md + k];
        if (j < 0 || j >= n) continue;   // malformed table entry: contributes nothing
        const double dx = (double)X[j].x - xi.x, dy = (double)X[j].y - xi.y;
        const double dux = (double)u[j].x - ui.x, duy = (double)u[j].y - ui.y;
        double w = 1.0;
        if (L > 0.f) {
            const double r = sqrt(dx * dx + dy * dy) / ((double)L + 1e-12);
            w = exp(-r * r);
        }
        a11 += w * dx * dx;
        a12 += w * dx * dy;
        a22 += w * dy * dy;
        b0x += w * dx * dux;
        b0y += w * dy * dux;
        b1x += w * dx * duy;
        b1y += w * dy * duy;
    }
    a11 += eps;
    a22 += eps;
    const double det = a11 * a22 - a12 * a12;
    const double g00 = (a22 * b0x - a12 * b0y) / det, g01 = (a11 * b0y - a12 * b0x) / det;   // d ux / d(x, y)
    const double g10 = (a22 * b1x - a12 * b1y) / det, g11 = (a11 * b1y - a12 * b1x) / det;   // d uy / d(x, y)
    const double F00 = 1.0 + g00, F01 = g01, F10 = g10, F11 = 1.0 + g11;
    const double C00 = F00 * F00 + F10 * F10, C11 = F01 * F01 + F11 * F11, C01 = F00 * F01 + F10 * F11;
    voigt[3 * i + 0] = (float)(0.5 * (C00 - 1.0));
    voigt[3 * i + 1] = (float)(0.5 * (C11 - 1.0));
    voigt[3 * i + 2] = (float)(0.5 * C01);
    if (Fout) {
        Fout[4 * i + 0] = (float)F00;
        Fout[4 * i + 1] = (float)F01;
        Fout[4 * i + 2] = (float)F10;
        Fout[4 * i + 3] = (float)F11;
    }
}

// Linearised strain for many displacement directions (the strain sensitivity of the implicit
// adjoint): with G(v) = A^-1 B(v) the least-squares gradient of a nodal field v (G[c][i] = d v_c /
// d x_i, A = sum w dX dX^T + eps I, B(v) = sum w dX dv^T), F = I + G(u) and dG = G(du),
// dE = (dG^T F + F^T dG) / 2 in Voigt form [dE00, dE11, (dE01 + dE10) / 2].  FP64 throughout.
// strain_geom: per node A^-1 and F (work[8 i ..]) and the neighbour weights (wk[i * md + k]);
// strain_jvp: one thread per (direction, node).
__global__ void strain_geom_kernel(const double *__restrict__ u, const double2 *__restrict__ X,
                                   const int *__restrict__ idx, const int *__restrict__ deg, int n, int md, double L,
                                   double eps, double *__restrict__ work, double *__restrict__ wk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 xi = X[i];
    const double uix = u[2 * i], uiy = u[2 * i + 1];
    const int d = deg[i];
    double a00 = 0, a01 = 0, a11 = 0, b00 = 0, b01 = 0, b10 = 0, b11 = 0;   // b[j][c] = sum w dX_j dv_c
    for (int k = 0; k < md; ++k) {
        double w = 0.0;
        const int j = k < d ? idx[(size_t)i * md + k] : -1;
        if (j >= 0 && j < n) {
            const double dx = X[j].x - xi.x, dy = X[j].y - xi.y;
            w = 1.0;
            if (L > 0.0) {
                const double r = sqrt(dx * dx + dy * dy) / (L + 1e-12);
                w = exp(-r * r);
            }
            const double dux = u[2 * j] - uix, duy = u[2 * j + 1] - uiy;
            a00 += w * dx * dx;
            a01 += w * dx * dy;
            a11 += w * dy * dy;
            b00 += w * dx * dux;
            b01 += w * dx * duy;
            b10 += w * dy * dux;
            b11 += w * dy * duy;
        }
        wk[(size_t)i * md + k] = w;
    }
    a00 += eps;
    a11 += eps;
    const double det = a00 * a11 - a01 * a01;
    const double i00 = a11 / det, i01 = -a01 / det, i11 = a00 / det;
    // G[c][i'] = sum_j Ainv[i'][j] b[j][c]
    const double G00 = i00 * b00 + i01 * b10, G01 = i01 * b00 + i11 * b10;
    const double G10 = i00 * b01 + i01 * b11, G11 = i01 * b01 + i11 * b11;
    double *o = work + 8 * (size_t)i;
    o[0] = i00;
    o[1] = i01;
    o[2] = i01;
    o[3] = i11;
    o[4] = 1.0 + G00;
    o[5] = G01;
    o[6] = G10;
    o[7] = 1.0 + G11;
}

__global__ void strain_jvp_kernel(const double *__restrict__ du, int K, const double2 *__restrict__ X,
                                  const int *__restrict__ idx, const int *__restrict__ deg, int n, int md,
                                  const double *__restrict__ work, const double *__restrict__ wk,
                                  double *__restrict__ dvoigt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int kk = blockIdx.y;
    if (i >= n || kk >= K) return;
    const double *v = du + (size_t)kk * n * 2;
    const double2 xi = X[i];
    const double vix = v[2 * i], viy = v[2 * i + 1];
    const int d = deg[i];
    double b00 = 0, b01 = 0, b10 = 0, b11 = 0;
    for (int k = 0; k < d && k < md; ++k) {
        const int j = idx[(size_t)i * md + k];
        if (j < 0 || j >= n) continue;
        const double w = wk[(size_t)i * md + k];
        const double dx = X[j].x - xi.x, dy = X[j].y - xi.y;
        const double dvx = v[2 * j] - vix, dvy = v[2 * j + 1] - viy;
        b00 += w * dx * dvx;
        b01 += w * dx * dvy;
        b10 += w * dy * dvx;
        b11 += w * dy * dvy;
    }
    const double *g = work + 8 * (size_t)i;
    const double i00 = g[0], i01 = g[1], i11 = g[3];
    const double F00 = g[4], F01 = g[5], F10 = g[6], F11 = g[7];
    const double D00 = i00 * b00 + i01 * b10, D01 = i01 * b00 + i11 * b10;   // dG[c][i']
    const double D10 = i00 * b01 + i01 * b11, D11 = i01 * b01 + i11 * b11;
    // (dG^T F)[a][b] = sum_c dG[c][a] F[c][b]
    const double P00 = D00 * F00 + D10 * F10, P01 = D00 * F01 + D10 * F11;
    const double P10 = D01 * F00 + D11 * F10, P11 = D01 * F01 + D11 * F11;
    double *o = dvoigt + ((size_t)kk * n + i) * 3;
    o[0] = P00;                       // (P + P^T) / 2 on the diagonal
    o[1] = P11;
    o[2] = 0.5 * (P01 + P10);         // ((P + P^T)_01 + (P + P^T)_10) / 4
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_strain_gl(const float *u, const float *nodes, const int *nbr_index, const int *nbr_degree,
                              int n_nodes, int max_deg, float gauge_length, float eps, float *voigt_out, float *F_out,
                              void *stream) {
    D2IC_REQUIRE(u && nodes && nbr_degree && voigt_out && (nbr_index || max_deg == 0), "d2ic_strain_gl: null pointer");
    D2IC_REQUIRE(n_nodes >= 0 && max_deg >= 0, "d2ic_strain_gl: bad sizes");
    if (n_nodes == 0) return D2IC_OK;
    strain_kernel<<<(n_nodes + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        (const float2 *)u, (const float2 *)nodes, nbr_index, nbr_degree, n_nodes, max_deg, gauge_length, eps,
        voigt_out, F_out);
    D2IC_CHECK_LAUNCH("strain_kernel");
    return D2IC_OK;
}

extern "C" int d2ic_strain_gl_jvp(const double *u, const double *du, int K, const double *nodes, const int *nbr_index,
                                  const int *nbr_degree, int n_nodes, int max_deg, double gauge_length, double eps,
                                  double *work, double *dvoigt_out, void *stream) {
    D2IC_REQUIRE(u && du && nodes && nbr_degree && work && dvoigt_out && (nbr_index || max_deg == 0),
                 "d2ic_strain_gl_jvp: null pointer");
    D2IC_REQUIRE(n_nodes >= 0 && max_deg >= 0 && K >= 0 && K < 65536, "d2ic_strain_gl_jvp: bad sizes");
    if (n_nodes == 0 || K == 0) return D2IC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    double *wk = work + 8 * (size_t)n_nodes;
    strain_geom_kernel<<<(n_nodes + 255) / 256, 256, 0, s>>>(u, (const double2 *)nodes, nbr_index, nbr_degree, n_nodes,
                                                             max_deg, gauge_length, eps, work, wk);
    D2IC_CHECK_LAUNCH("strain_geom_kernel");
    strain_jvp_kernel<<<dim3((n_nodes + 255) / 256, K), 256, 0, s>>>(du, K, (const double2 *)nodes, nbr_index,
                                                                     nbr_degree, n_nodes, max_deg, work, wk,
                                                                     dvoigt_out);
    D2IC_CHECK_LAUNCH("strain_jvp_kernel");
    return D2IC_OK;
}

extern "C" size_t d2ic_strain_gl_jvp_work_doubles(int n_nodes, int max_deg) {
    return (size_t)(n_nodes > 0 ? n_nodes : 0) * (size_t)(8 + (max_deg > 0 ? max_deg : 0));
}
