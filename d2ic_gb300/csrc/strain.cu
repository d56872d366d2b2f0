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
