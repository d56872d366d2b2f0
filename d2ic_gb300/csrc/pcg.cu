// Block-Jacobi preconditioned CG on the exact Hessian of the converged frame,
// for K right-hand sides in lock step (the linear solves of the implicit
// adjoint: H X = B).  Vectors are (n_nodes, 2, K) FP64 with the column index
// fastest; H is applied in FP32 by d2ic_hessian_matvec; the 2x2 diagonal blocks'
// inverses (Minv) and the active-dof mask come from the host.
//
// Per iteration: AP = H P (masked), pap = P.AP, a = rz / pap, X += a P,
// R -= a AP, Z = Minv R, rr = R.R, rz' = R.Z, P = Z + (rz' / rz) P.  Every
// column reduction is a per-block partial followed by a fixed-order sum over
// blocks, so the solve is deterministic.  The host checks ||R|| <= rtol ||B||
// for all columns after each iteration.
#include <stdlib.h>
#include <string.h>

#include "common.cuh"

namespace d2ic {

constexpr int PT = 256;          // threads per block; thread t owns columns t, t + PT, ...

// nodes [n0, n1) of block b
__device__ __forceinline__ void node_range(int n_nodes, int &n0, int &n1) {
    const int per = (n_nodes + gridDim.x - 1) / gridDim.x;
    n0 = min((int)blockIdx.x * per, n_nodes);
    n1 = min(n0 + per, n_nodes);
}

__global__ void __launch_bounds__(PT) pcg_init(int n_nodes, int K, const double *__restrict__ B,
                                               const unsigned char *__restrict__ act, const double *__restrict__ Minv,
                                               double *__restrict__ X, double *__restrict__ R, double *__restrict__ Z,
                                               double *__restrict__ P, float *__restrict__ Pf,
                                               double *__restrict__ part_rz, double *__restrict__ part_bb) {
    int n0, n1;
    node_range(n_nodes, n0, n1);
    for (int k = threadIdx.x; k < K; k += PT) {
        double rz = 0.0, bb = 0.0;
        for (int n = n0; n < n1; ++n) {
            const double m = act[n] ? 1.0 : 0.0;
            const size_t i0 = ((size_t)n * 2) * K + k, i1 = i0 + K;
            const double b0 = B[i0] * m, b1 = B[i1] * m;
            const double *M = Minv + 4 * (size_t)n;
            const double z0 = M[0] * b0 + M[1] * b1, z1 = M[2] * b0 + M[3] * b1;
            X[i0] = 0.0;
            X[i1] = 0.0;
            R[i0] = b0;
            R[i1] = b1;
            Z[i0] = z0;
            Z[i1] = z1;
            P[i0] = z0;
            P[i1] = z1;
            Pf[i0] = (float)z0;
            Pf[i1] = (float)z1;
            rz += b0 * z0 + b1 * z1;
            bb += b0 * b0 + b1 * b1;
        }
        part_rz[(size_t)blockIdx.x * K + k] = rz;
        part_bb[(size_t)blockIdx.x * K + k] = bb;
    }
}

__global__ void __launch_bounds__(PT) pcg_pap(int n_nodes, int K, const double *__restrict__ P, const float *__restrict__ AP,
                                              const unsigned char *__restrict__ act, double *__restrict__ part) {
    int n0, n1;
    node_range(n_nodes, n0, n1);
    for (int k = threadIdx.x; k < K; k += PT) {
        double s = 0.0;
        for (int n = n0; n < n1; ++n) {
            if (!act[n]) continue;
            const size_t i0 = ((size_t)n * 2) * K + k, i1 = i0 + K;
            s += P[i0] * (double)AP[i0] + P[i1] * (double)AP[i1];
        }
        part[(size_t)blockIdx.x * K + k] = s;
    }
}

__global__ void __launch_bounds__(PT) pcg_step(int n_nodes, int K, const double *__restrict__ rz,
                                               const double *__restrict__ pap, const unsigned char *__restrict__ act,
                                               const double *__restrict__ Minv, double *__restrict__ X,
                                               double *__restrict__ R, double *__restrict__ Z,
                                               const double *__restrict__ P, const float *__restrict__ AP,
                                               double *__restrict__ part_rr, double *__restrict__ part_rz) {
    int n0, n1;
    node_range(n_nodes, n0, n1);
    for (int k = threadIdx.x; k < K; k += PT) {
        const double a = pap[k] > 0.0 ? rz[k] / pap[k] : 0.0;
        double rr = 0.0, rzn = 0.0;
        for (int n = n0; n < n1; ++n) {
            const double m = act[n] ? 1.0 : 0.0;
            const size_t i0 = ((size_t)n * 2) * K + k, i1 = i0 + K;
            X[i0] += a * P[i0];
            X[i1] += a * P[i1];
            const double r0 = R[i0] - a * ((double)AP[i0] * m), r1 = R[i1] - a * ((double)AP[i1] * m);
            R[i0] = r0;
            R[i1] = r1;
            const double *M = Minv + 4 * (size_t)n;
            const double z0 = M[0] * r0 + M[1] * r1, z1 = M[2] * r0 + M[3] * r1;
            Z[i0] = z0;
            Z[i1] = z1;
            rr += r0 * r0 + r1 * r1;
            rzn += r0 * z0 + r1 * z1;
        }
        part_rr[(size_t)blockIdx.x * K + k] = rr;
        part_rz[(size_t)blockIdx.x * K + k] = rzn;
    }
}

__global__ void __launch_bounds__(PT) pcg_dir(int n_nodes, int K, const double *__restrict__ rz_old,
                                              const double *__restrict__ rz_new, const double *__restrict__ Z,
                                              double *__restrict__ P, float *__restrict__ Pf) {
    int n0, n1;
    node_range(n_nodes, n0, n1);
    for (int k = threadIdx.x; k < K; k += PT) {
        const double beta = rz_old[k] > 0.0 ? rz_new[k] / rz_old[k] : 0.0;
        for (int n = n0; n < n1; ++n) {
            const size_t i0 = ((size_t)n * 2) * K + k, i1 = i0 + K;
            const double p0 = Z[i0] + beta * P[i0], p1 = Z[i1] + beta * P[i1];
            P[i0] = p0;
            P[i1] = p1;
            Pf[i0] = (float)p0;
            Pf[i1] = (float)p1;
        }
    }
}

// out[k] = sum over blocks of part[b][k]: one warp per column, lane l sums blocks l, l + 32, ...
// in order, then a fixed shuffle tree (deterministic)
__global__ void pcg_reduce(int nb, int K, const double *__restrict__ part, double *__restrict__ out) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= K) return;
    double s = 0.0;
    for (int b = lane; b < nb; b += 32) s += part[(size_t)b * K + k];
    s = warp_sum_d(s);
    if (lane == 0) out[k] = s;
}

struct PcgWork {
    double *R, *Z, *P, *part_a, *part_b, *rz, *rz2, *pap, *rr, *bb;
    float *Pf, *AP, *slots;
};

static size_t carve(int n_nodes, int K, int node_chunk_k, int nb, char *base, PcgWork *w) {
    const size_t v = (size_t)n_nodes * 2 * K;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    w->R = (double *)take(sizeof(double) * v);
    w->Z = (double *)take(sizeof(double) * v);
    w->P = (double *)take(sizeof(double) * v);
    w->Pf = (float *)take(sizeof(float) * v);
    w->AP = (float *)take(sizeof(float) * v);
    w->slots = (float *)take(sizeof(float) * (size_t)node_chunk_k * v);
    w->part_a = (double *)take(sizeof(double) * (size_t)nb * K);
    w->part_b = (double *)take(sizeof(double) * (size_t)nb * K);
    w->rz = (double *)take(sizeof(double) * K);
    w->rz2 = (double *)take(sizeof(double) * K);
    w->pap = (double *)take(sizeof(double) * K);
    w->rr = (double *)take(sizeof(double) * K);
    w->bb = (double *)take(sizeof(double) * K);
    return off;
}

static int pcg_blocks(int n_nodes) {
    int nb = (n_nodes + 15) / 16;                 // >= 16 nodes per block
    return nb < 1 ? 1 : (nb > 1024 ? 1024 : nb);
}

}  // namespace d2ic

using namespace d2ic;

extern "C" size_t d2ic_pcg_work_bytes(int n_nodes, int K, int node_chunk_k) {
    PcgWork w;
    if (n_nodes < 1) n_nodes = 1;
    if (K < 1) K = 1;
    if (node_chunk_k < 1) node_chunk_k = 1;
    return carve(n_nodes, K, node_chunk_k, pcg_blocks(n_nodes), nullptr, &w);
}

extern "C" int d2ic_pcg_solve(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                              const float *chunk_hess, float inv_np, float alpha_reg, const double *Minv,
                              const unsigned char *active, const double *B, double *X, int K, double rtol,
                              int max_iter, void *work, size_t work_bytes, int *iters_out, void *stream) {
    D2IC_REQUIRE(frame_dev && chunk_hess && Minv && active && B && X && work && K >= 1 && n_nodes >= 1 &&
                     node_chunk_k >= 1 && max_iter >= 0,
                 "d2ic_pcg_solve: bad arguments");
    D2IC_REQUIRE(((uintptr_t)work & 255) == 0, "d2ic_pcg_solve: work must be 256-byte aligned");
    const int nb = pcg_blocks(n_nodes);
    PcgWork w;
    const size_t need = carve(n_nodes, K, node_chunk_k, nb, (char *)work, &w);
    D2IC_REQUIRE(work_bytes >= need, "d2ic_pcg_solve: work %zu bytes < %zu needed", work_bytes, need);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t v = (size_t)n_nodes * 2 * K;
    // slots that no chunk owns must read as 0; owned ones are rewritten by every matvec
    cudaError_t e = cudaMemsetAsync(w.slots, 0, sizeof(float) * (size_t)node_chunk_k * v, s);
    if (e != cudaSuccess) return cuda_status(e, "pcg slots");
    const int rb = (K + 7) / 8;                    // pcg_reduce: 8 warps (columns) per block
    pcg_init<<<nb, PT, 0, s>>>(n_nodes, K, B, active, Minv, X, w.R, w.Z, w.P, w.Pf, w.part_a, w.part_b);
    pcg_reduce<<<rb, 256, 0, s>>>(nb, K, w.part_a, w.rz);
    pcg_reduce<<<rb, 256, 0, s>>>(nb, K, w.part_b, w.bb);
    D2IC_CHECK_LAUNCH("pcg init");
    double *host = (double *)malloc(sizeof(double) * 2 * K);
    if (!host) {
        set_error("d2ic_pcg_solve: host allocation failed");
        return D2IC_OOM;
    }
    double *h_rr = host, *h_bb = host + K;
    e = cudaMemcpyAsync(h_bb, w.bb, sizeof(double) * K, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        free(host);
        return cuda_status(e, "pcg norms");
    }
    int it = 0, st = D2IC_OK;
    double *rz = w.rz, *rz_new = w.rz2;
    for (it = 1; it <= max_iter; ++it) {
        st = d2ic_hessian_matvec(frame_dev, n_chunks, n_nodes, chunk_hess, w.Pf, K, inv_np, alpha_reg, w.slots, w.AP,
                                 stream);
        if (st) break;
        pcg_pap<<<nb, PT, 0, s>>>(n_nodes, K, w.P, w.AP, active, w.part_a);
        pcg_reduce<<<rb, 256, 0, s>>>(nb, K, w.part_a, w.pap);
        pcg_step<<<nb, PT, 0, s>>>(n_nodes, K, rz, w.pap, active, Minv, X, w.R, w.Z, w.P, w.AP, w.part_a, w.part_b);
        pcg_reduce<<<rb, 256, 0, s>>>(nb, K, w.part_a, w.rr);
        pcg_reduce<<<rb, 256, 0, s>>>(nb, K, w.part_b, rz_new);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_rr, w.rr, sizeof(double) * K, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            st = cuda_status(e, "pcg iteration");
            break;
        }
        bool done = true;
        for (int k = 0; k < K && done; ++k) {
            const double bn = sqrt(h_bb[k]) > 1e-300 ? sqrt(h_bb[k]) : 1e-300;
            done = sqrt(h_rr[k]) <= rtol * bn;
        }
        if (done) break;
        pcg_dir<<<nb, PT, 0, s>>>(n_nodes, K, rz, rz_new, w.Z, w.P, w.Pf);
        double *t = rz;
        rz = rz_new;
        rz_new = t;
    }
    free(host);
    if (iters_out) *iters_out = it > max_iter ? max_iter : it;
    if (st) return st;
    D2IC_CHECK_LAUNCH("pcg loop");
    return D2IC_OK;
}
