/*
 * FP64 pixel term of the D2IC global objective, in C for speed.
 *
 * Test infrastructure only: called by the oracle (oracle/fast.py) to run the
 * reference's nonlinear CG at full benchmark sizes.  Never linked into the
 * product library.
 *
 * Restates residuals_pixelwise_core / J_pixelwise_core and their gradient
 * (d2ic/solver_global_cg.py:205-258) with the oracle's cubic definition: the
 * interpolating cubic B-spline with edge-replicating boundary, evaluated on a
 * coefficient array that carries a `pad`-wide halo (oracle/cubic.py).
 *
 * Build: see oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline void bsw(double t, double w[4], double dw[4]) {
    double t2 = t * t, t3 = t2 * t, o = 1.0 - t;
    w[0] = o * o * o / 6.0;
    w[1] = (3.0 * t3 - 6.0 * t2 + 4.0) / 6.0;
    w[2] = (-3.0 * t3 + 3.0 * t2 + 3.0 * t + 1.0) / 6.0;
    w[3] = t3 / 6.0;
    dw[0] = -0.5 * o * o;
    dw[1] = 1.5 * t2 - 2.0 * t;
    dw[2] = -1.5 * t2 + t + 0.5;
    dw[3] = 0.5 * t2;
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* value and gradient of the spline at image-index coordinates (x = col, y = row) */
static inline double sample(const double *c, int Hc, int Wc, int pad, double x, double y,
                            double *gx, double *gy) {
    double fx = floor(x), fy = floor(y);
    int ix = (int)fx, iy = (int)fy;
    double wx[4], dwx[4], wy[4], dwy[4];
    bsw(x - fx, wx, dwx);
    bsw(y - fy, wy, dwy);
    double v = 0.0, ax = 0.0, ay = 0.0;
    for (int a = 0; a < 4; ++a) {
        int r = clampi(iy - 1 + a + pad, 0, Hc - 1);
        const double *row = c + (size_t)r * Wc;
        double rv = 0.0, rd = 0.0;
        for (int b = 0; b < 4; ++b) {
            double cv = row[clampi(ix - 1 + b + pad, 0, Wc - 1)];
            rv += wx[b] * cv;
            rd += dwx[b] * cv;
        }
        v += wy[a] * rv;
        ax += wy[a] * rd;
        ay += dwy[a] * rv;
    }
    *gx = ax;
    *gy = ay;
    return v;
}

/*
 * sum_r2 = sum_p r_p^2 with r_p = I2(x_p + sum_a N_pa u_{n_pa}) - I1_p.
 * If grad != NULL: grad[n] += scale * sum_{p,a: n_pa = n} r_p N_pa dI2/dx.
 * Per-thread private gradient buffers, static schedule: deterministic for a
 * fixed thread count.
 */
void oracle_pixel_terms(const double *coeff, int Hc, int Wc, int pad,
                        const double *coords, const int *pnodes, const double *N,
                        const double *I1, int Np, const double *u, int Nn,
                        double scale, double *sum_r2, double *grad, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    double total = 0.0;
    double *priv = NULL;
    if (grad) {
        priv = (double *)calloc((size_t)nthreads * Nn * 2, sizeof(double));
    }
    double *parts = (double *)calloc((size_t)nthreads, sizeof(double));
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        long lo = (long)Np * tid / nt, hi = (long)Np * (tid + 1) / nt;
        double acc = 0.0;
        double *g = grad ? priv + (size_t)tid * Nn * 2 : NULL;
        for (long p = lo; p < hi; ++p) {
            const int *nd = pnodes + 4 * p;
            const double *w = N + 4 * p;
            double ux = 0.0, uy = 0.0;
            for (int a = 0; a < 4; ++a) {
                ux += w[a] * u[2 * nd[a]];
                uy += w[a] * u[2 * nd[a] + 1];
            }
            double xd = coords[2 * p] + ux - 0.5;
            double yd = coords[2 * p + 1] + uy - 0.5;
            double gx, gy;
            double r = sample(coeff, Hc, Wc, pad, xd, yd, &gx, &gy) - I1[p];
            acc += r * r;
            if (g) {
                double s = scale * r;
                for (int a = 0; a < 4; ++a) {
                    g[2 * nd[a]] += s * w[a] * gx;
                    g[2 * nd[a] + 1] += s * w[a] * gy;
                }
            }
        }
        parts[tid] = acc;
    }
    for (int t = 0; t < nthreads; ++t) total += parts[t];
    if (grad) {
        for (int t = 0; t < nthreads; ++t) {
            const double *g = priv + (size_t)t * Nn * 2;
            for (long i = 0; i < 2L * Nn; ++i) grad[i] += g[i];
        }
        free(priv);
    }
    free(parts);
    *sum_r2 = total;
}
