/*
 * Body of the oracle's pixel term, written once for a REAL type and
 * instantiated by objective_c.c for double (the FP64 oracle) and for float
 * (an x32-equivalent CPU timing: the reference runs JAX in float32 unless x64
 * is enabled).  FN(name) names each instantiation.
 *
 * Test infrastructure only; see objective_c.c.
 */

static inline void FN(bsw)(REAL t, REAL w[4], REAL dw[4]) {
    const REAL t2 = t * t, t3 = t2 * t, o = (REAL)1 - t;
    w[0] = o * o * o / (REAL)6;
    w[1] = ((REAL)3 * t3 - (REAL)6 * t2 + (REAL)4) / (REAL)6;
    w[2] = ((REAL)-3 * t3 + (REAL)3 * t2 + (REAL)3 * t + (REAL)1) / (REAL)6;
    w[3] = t3 / (REAL)6;
    dw[0] = (REAL)-0.5 * o * o;
    dw[1] = (REAL)1.5 * t2 - (REAL)2 * t;
    dw[2] = (REAL)-1.5 * t2 + t + (REAL)0.5;
    dw[3] = (REAL)0.5 * t2;
}

/* value and gradient of the spline at image-index coordinates (x = col, y = row) */
static inline REAL FN(sample)(const REAL *c, int Hc, int Wc, int pad, REAL x, REAL y, REAL *gx, REAL *gy) {
    const REAL fx = (REAL)floor((double)x), fy = (REAL)floor((double)y);
    const int ix = (int)fx, iy = (int)fy;
    REAL wx[4], dwx[4], wy[4], dwy[4];
    FN(bsw)(x - fx, wx, dwx);
    FN(bsw)(y - fy, wy, dwy);
    REAL v = 0, ax = 0, ay = 0;
    for (int a = 0; a < 4; ++a) {
        const int r = clampi(iy - 1 + a + pad, 0, Hc - 1);
        const REAL *row = c + (size_t)r * Wc;
        REAL rv = 0, rd = 0;
        for (int b = 0; b < 4; ++b) {
            const REAL cv = row[clampi(ix - 1 + b + pad, 0, Wc - 1)];
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
void FN(oracle_pixel_terms)(const REAL *coeff, int Hc, int Wc, int pad, const REAL *coords, const int *pnodes,
                            const REAL *N, const REAL *I1, int Np, const REAL *u, int Nn, REAL scale,
                            double *sum_r2, REAL *grad, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    double total = 0.0;
    REAL *priv = NULL;
    if (grad) priv = (REAL *)calloc((size_t)nthreads * Nn * 2, sizeof(REAL));
    REAL *parts = (REAL *)calloc((size_t)nthreads, sizeof(REAL));
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        const long lo = (long)Np * tid / nt, hi = (long)Np * (tid + 1) / nt;
        REAL acc = 0;
        REAL *g = grad ? priv + (size_t)tid * Nn * 2 : NULL;
        for (long p = lo; p < hi; ++p) {
            const int *nd = pnodes + 4 * p;
            const REAL *w = N + 4 * p;
            REAL ux = 0, uy = 0;
            for (int a = 0; a < 4; ++a) {
                ux += w[a] * u[2 * nd[a]];
                uy += w[a] * u[2 * nd[a] + 1];
            }
            const REAL xd = coords[2 * p] + ux - (REAL)0.5;
            const REAL yd = coords[2 * p + 1] + uy - (REAL)0.5;
            REAL gx, gy;
            const REAL r = FN(sample)(coeff, Hc, Wc, pad, xd, yd, &gx, &gy) - I1[p];
            acc += r * r;
            if (g) {
                const REAL s = scale * r;
                for (int a = 0; a < 4; ++a) {
                    g[2 * nd[a]] += s * w[a] * gx;
                    g[2 * nd[a] + 1] += s * w[a] * gy;
                }
            }
        }
        parts[tid] = acc;
    }
    for (int t = 0; t < nthreads; ++t) total += (double)parts[t];
    if (grad) {
        for (int t = 0; t < nthreads; ++t) {
            const REAL *g = priv + (size_t)t * Nn * 2;
            for (long i = 0; i < 2L * Nn; ++i) grad[i] += g[i];
        }
        free(priv);
    }
    free(parts);
    *sum_r2 = total;
}
