// The Hessian of the converged frame as an assembled node operator, and the
// block-Jacobi preconditioned CG that solves H X = B for K right-hand sides in
// lock step (the linear solves of the implicit adjoint).
//
// Assembly (once per linearisation point): the per-chunk element blocks
// (d2ic_hessian_chunks: 10 symmetric 2x2 blocks per chunk) are scattered into
// per-node slots (each chunk owns one slot of each of its nodes, so no atomics),
// then one warp per node merges its slots and its springs into at most
// D2IC_HOP_MAX (column node, symmetric 2x2 block) entries, in slot order:
//     H_nj = (1/Np) sum_{chunks c at n, j} K^c_nj  +  alpha * springs.
// Apply: Y = H V, one warp per node and 32 right-hand sides (lane = column),
// V and Y laid out (node, component, k) with k fastest, so every neighbour read
// is one coalesced 128-byte row; the entries of a node are read once for all
// columns.  This replaces the chunk -> node-slot -> node pass per product (one
// write and one read of node_chunk_k * Nn * 2 * K floats per product).
//
// PCG: per iteration AP = H P with the block partials of P.AP, their column sums,
// the update of X, R, Z with the partials of R.R and R.Z, their column sums (one
// warp per column, blocks summed in a fixed order: deterministic) and the new
// direction.  The last block of the second column sum decides convergence
// (||R|| <= rtol ||B|| for every column) into a device flag that makes the later
// kernels return at once, so the host launches iterations in batches and reads
// the flag once per batch instead of synchronising every iteration.
#include <stdlib.h>
#include <string.h>

#include "common.cuh"

namespace d2ic {

constexpr int HOP = D2IC_HOP_MAX;   // operator entries per node
static_assert(HOP <= 32, "one lane per operator entry");
constexpr int PT = 256;             // threads per block of the node-range kernels

__device__ __forceinline__ int hop_pair(int a, int b) {   // a <= b: index of the pair in 0..9
    return a * 4 - (a * (a - 1)) / 2 + (b - a);
}

// operator storage inside the caller's buffer
struct HopView {
    float4 *blk;     // Nn * HOP: (xx, xy, yy, 0) of entry q of node n at n * HOP + q
    int *idx;        // Nn * HOP: column node, -1 after the last entry
    int *err;        // 1 int: set when a node has more than HOP distinct columns
    int *sids;       // assembly scratch: node_chunk_k * Nn * 4 column nodes (-1: slot not owned)
    float4 *sblk;    // node_chunk_k * Nn * 4 blocks
};

__host__ __device__ inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

__host__ __device__ inline size_t hop_layout(int n_nodes, int node_chunk_k, char *base, HopView *v) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += al256(bytes);
        return p;
    };
    v->blk = (float4 *)take(sizeof(float4) * (size_t)n_nodes * HOP);
    v->idx = (int *)take(sizeof(int) * (size_t)n_nodes * HOP);
    v->err = (int *)take(sizeof(int));
    v->sids = (int *)take(sizeof(int) * (size_t)node_chunk_k * n_nodes * 4);
    v->sblk = (float4 *)take(sizeof(float4) * (size_t)node_chunk_k * n_nodes * 4);
    return off;
}

// chunk pass: thread (c, a) writes row a of chunk c's element matrix into slot rank_a(c) of node n_a
__global__ void __launch_bounds__(256) hop_scatter(const d2ic_frame_t *__restrict__ fp, const float *__restrict__ hess,
                                                   int *__restrict__ sids, float4 *__restrict__ sblk) {
    const d2ic_frame_t &F = *fp;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = t >> 2, a = t & 3;
    if (c >= F.n_chunks) return;
    const int n = __ldg(F.chunk_nodes + 4 * c + a);
    const int s = (int)(((unsigned)__ldg(F.chunk_slot + c) >> (8 * a)) & 0xffu);
    const size_t e = ((size_t)s * F.n_nodes + n) * 4;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int p = 3 * hop_pair(min(a, b), max(a, b));
        sids[e + b] = __ldg(F.chunk_nodes + 4 * c + b);
        sblk[e + b] = make_float4(__ldg(hess + 32 * (size_t)c + p), __ldg(hess + 32 * (size_t)c + p + 1),
                                  __ldg(hess + 32 * (size_t)c + p + 2), 0.f);
    }
}

// add (xx, xy, yy) to the entry of column j, appending it if new (whole warp; lane q holds entry q)
__device__ __forceinline__ void hop_add(int &my_idx, float4 &my_blk, int &count, int &overflow, int j, float xx,
                                        float xy, float yy, int lane) {
    const unsigned hit = __ballot_sync(0xffffffffu, my_idx == j);
    int q;
    if (hit) {
        q = __ffs(hit) - 1;
    } else {
        q = count;
        if (q >= HOP) {
            overflow = 1;
            return;
        }
        ++count;
        if (lane == q) my_idx = j;
    }
    if (lane == q) {
        my_blk.x += xx;
        my_blk.y += xy;
        my_blk.z += yy;
    }
}

// node pass: one warp per node merges its slots (slot order, row order) and its springs
__global__ void __launch_bounds__(256) hop_merge(const d2ic_frame_t *__restrict__ fp, const int *__restrict__ sids,
                                                 const float4 *__restrict__ sblk, float inv_np, float alpha,
                                                 int *__restrict__ idx, float4 *__restrict__ blk, int *__restrict__ err) {
    const d2ic_frame_t &F = *fp;
    const int lane = threadIdx.x & 31;
    const int n = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (n >= F.n_nodes) return;
    const size_t Nn = F.n_nodes;
    int my_idx = -1, count = 0, overflow = 0;
    float4 my_blk = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int s = 0; s < F.node_chunk_k; ++s) {
        const size_t e = ((size_t)s * Nn + n) * 4;
        const int jl = lane < 4 ? __ldg(sids + e + lane) : -1;
        const float4 bl = lane < 4 ? __ldg(sblk + e + lane) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int b = 0; b < 4; ++b) {
            const int j = __shfl_sync(0xffffffffu, jl, b);
            if (j < 0) break;   // slot not owned by a chunk (uniform)
            hop_add(my_idx, my_blk, count, overflow, j, inv_np * __shfl_sync(0xffffffffu, bl.x, b),
                    inv_np * __shfl_sync(0xffffffffu, bl.y, b), inv_np * __shfl_sync(0xffffffffu, bl.z, b), lane);
        }
    }
    for (int q = 0; q < F.max_deg; ++q) {                 // springs: alpha * w on the diagonal, -alpha * w off it
        const int j = __ldg(F.nbr_index + (size_t)q * Nn + n);
        if (j < 0) break;
        const float w = alpha * __ldg(F.nbr_weight + (size_t)q * Nn + n);
        hop_add(my_idx, my_blk, count, overflow, n, w, 0.f, w, lane);
        hop_add(my_idx, my_blk, count, overflow, j, -w, 0.f, -w, lane);
    }
    if (lane < HOP) {
        idx[(size_t)n * HOP + lane] = my_idx;
        blk[(size_t)n * HOP + lane] = my_blk;
    }
    if (overflow && lane == 0) atomicExch(err, 1);
}

// one node (warp) x 32 columns (lanes): y = sum_q blk_q v_{idx_q}
__device__ __forceinline__ void hop_row(const int *__restrict__ idx, const float4 *__restrict__ blk, int n, int K, int k,
                                        const float *__restrict__ V, int lane, float &yx, float &yy) {
    const int my_idx = lane < HOP ? __ldg(idx + (size_t)n * HOP + lane) : -1;
    const float4 my_blk = lane < HOP ? __ldg(blk + (size_t)n * HOP + lane) : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned live = __ballot_sync(0xffffffffu, my_idx >= 0);
    const int cnt = __popc(live);                          // entries are packed from lane 0
    yx = 0.f;
    yy = 0.f;
    constexpr int UB = 8;
    for (int q0 = 0; q0 < cnt; q0 += UB) {
        float vx[UB], vy[UB];
        int jj[UB];
#pragma unroll
        for (int u = 0; u < UB; ++u) {
            jj[u] = __shfl_sync(0xffffffffu, my_idx, (q0 + u) & 31);
            const bool ok = q0 + u < cnt && k < K;
            vx[u] = ok ? __ldg(V + ((size_t)jj[u] * 2) * K + k) : 0.f;
            vy[u] = ok ? __ldg(V + ((size_t)jj[u] * 2 + 1) * K + k) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < UB; ++u) {
            const int q = (q0 + u) & 31;
            const float bx = __shfl_sync(0xffffffffu, my_blk.x, q), by = __shfl_sync(0xffffffffu, my_blk.y, q),
                        bz = __shfl_sync(0xffffffffu, my_blk.z, q);
            if (q0 + u < cnt) {
                yx = __fmaf_rn(bx, vx[u], __fmaf_rn(by, vy[u], yx));
                yy = __fmaf_rn(by, vx[u], __fmaf_rn(bz, vy[u], yy));
            }
        }
    }
}

// Y = H V: block = 8 nodes (warps) x 32 columns
__global__ void __launch_bounds__(256) hop_apply(const int *__restrict__ idx, const float4 *__restrict__ blk,
                                                 int n_nodes, const float *__restrict__ V, int K, float *__restrict__ Y) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = blockIdx.x * 8 + w, k = blockIdx.y * 32 + lane;
    if (n >= n_nodes) return;
    float yx, yy;
    hop_row(idx, blk, n, K, k, V, lane, yx, yy);
    if (k < K) {
        Y[((size_t)n * 2) * K + k] = yx;
        Y[((size_t)n * 2 + 1) * K + k] = yy;
    }
}

// The entries of a block's 8 nodes, staged in shared memory and read as broadcasts.
struct HopTile {
    int idx[8][HOP];
    float4 blk[8][HOP];
    int cnt[8];
};

__device__ __forceinline__ void hop_stage(const int *__restrict__ idx, const float4 *__restrict__ blk, int n_nodes,
                                          HopTile &T) {
    static_assert(8 * HOP <= 256, "one thread per staged entry");
    const int t = threadIdx.x;
    if (t < 8 * HOP) {
        const int w = t / HOP, q = t % HOP, n = blockIdx.x * 8 + w;
        int j = -1;
        float4 b = make_float4(0.f, 0.f, 0.f, 0.f);
        if (n < n_nodes) {
            j = __ldg(idx + (size_t)n * HOP + q);
            b = __ldg(blk + (size_t)n * HOP + q);
        }
        T.idx[w][q] = j;
        T.blk[w][q] = b;
    }
    __syncthreads();
    if (t < 8) {
        int c = 0;
        while (c < HOP && T.idx[t][c] >= 0) ++c;   // entries are packed from the first
        T.cnt[t] = c;
    }
    __syncthreads();
}

// node w of the tile x 4 consecutive columns k0 .. k0 + 3 (K a multiple of 4): the same operations per
// column, in the same order, as hop_row
__device__ __forceinline__ void hop_row4(const HopTile &T, int w, int K, int k0, const float *__restrict__ V,
                                         float4 &yx, float4 &yy) {
    yx = make_float4(0.f, 0.f, 0.f, 0.f);
    yy = yx;
    const int cnt = T.cnt[w];
#pragma unroll 3
    for (int q = 0; q < cnt; ++q) {
        const int j = T.idx[w][q];
        const float4 b = T.blk[w][q];
        const float4 vx = __ldg(reinterpret_cast<const float4 *>(V + ((size_t)j * 2) * K + k0));
        const float4 vy = __ldg(reinterpret_cast<const float4 *>(V + ((size_t)j * 2 + 1) * K + k0));
        yx.x = __fmaf_rn(b.x, vx.x, __fmaf_rn(b.y, vy.x, yx.x));
        yx.y = __fmaf_rn(b.x, vx.y, __fmaf_rn(b.y, vy.y, yx.y));
        yx.z = __fmaf_rn(b.x, vx.z, __fmaf_rn(b.y, vy.z, yx.z));
        yx.w = __fmaf_rn(b.x, vx.w, __fmaf_rn(b.y, vy.w, yx.w));
        yy.x = __fmaf_rn(b.y, vx.x, __fmaf_rn(b.z, vy.x, yy.x));
        yy.y = __fmaf_rn(b.y, vx.y, __fmaf_rn(b.z, vy.y, yy.y));
        yy.z = __fmaf_rn(b.y, vx.z, __fmaf_rn(b.z, vy.z, yy.z));
        yy.w = __fmaf_rn(b.y, vx.w, __fmaf_rn(b.z, vy.w, yy.w));
    }
}

// Y = H V for K a multiple of 4: one warp per node (8 per block), lane l on columns 4 l .. 4 l + 3 of
// each 128-column pass over K.  The node's entries are staged once per warp in shared memory (no
// block-wide barrier) and read as broadcasts; per column the operations are those of hop_row.  At
// 32 registers 64 warps fit on an SM, so a frame's nodes (one warp each) run in a single wave on
// 152 SMs up to 9,728 nodes instead of queueing a second, mostly empty wave of blocks.
__global__ void __launch_bounds__(256, 8) hop_apply4(const int *__restrict__ idx, const float4 *__restrict__ blk,
                                                     int n_nodes, const float *__restrict__ V, int K,
                                                     float *__restrict__ Y) {
    __shared__ int s_j[8][HOP];
    __shared__ float4 s_b[8][HOP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = blockIdx.x * 8 + w;
    if (n >= n_nodes) return;                  // the whole warp: nothing below waits on the block
    int j = -1;
    if (lane < HOP) {
        j = __ldg(idx + (size_t)n * HOP + lane);
        s_j[w][lane] = j;
        s_b[w][lane] = __ldg(blk + (size_t)n * HOP + lane);
    }
    const int cnt = __popc(__ballot_sync(0xffffffffu, j >= 0));   // entries are packed from the first
    __syncwarp();
    // float4 offsets within 32 bits (the host checks n_nodes * 2 * K < 2^31): row 2 j at j * K / 2
    const int h = K >> 1, q4 = K >> 2;
    const float4 *V4 = reinterpret_cast<const float4 *>(V);
    float4 *Y4 = reinterpret_cast<float4 *>(Y) + n * h;
    for (int c = lane; c < q4; c += 32) {
        float4 yx = make_float4(0.f, 0.f, 0.f, 0.f), yy = yx;
#pragma unroll 1
        for (int q = 0; q < cnt; ++q) {
            const int r = s_j[w][q] * h + c;
            const float4 b = s_b[w][q];
            const float4 vx = __ldg(V4 + r);
            const float4 vy = __ldg(V4 + r + q4);
            yx.x = __fmaf_rn(b.x, vx.x, __fmaf_rn(b.y, vy.x, yx.x));
            yx.y = __fmaf_rn(b.x, vx.y, __fmaf_rn(b.y, vy.y, yx.y));
            yx.z = __fmaf_rn(b.x, vx.z, __fmaf_rn(b.y, vy.z, yx.z));
            yx.w = __fmaf_rn(b.x, vx.w, __fmaf_rn(b.y, vy.w, yx.w));
            yy.x = __fmaf_rn(b.y, vx.x, __fmaf_rn(b.z, vy.x, yy.x));
            yy.y = __fmaf_rn(b.y, vx.y, __fmaf_rn(b.z, vy.y, yy.y));
            yy.z = __fmaf_rn(b.y, vx.z, __fmaf_rn(b.z, vy.z, yy.z));
            yy.w = __fmaf_rn(b.y, vx.w, __fmaf_rn(b.z, vy.w, yy.w));
        }
        Y4[c] = yx;
        Y4[c + q4] = yy;
    }
}

// ---------------------------------------------------------------------------
// PCG
// ---------------------------------------------------------------------------
struct PcgCtl {
    int done;        // all columns converged: later kernels return at once
    int iters;       // iterations whose update ran
    int cnt_check;   // last-block counter of the convergence check (reset by the last block)
    int pad_;
};

__device__ __forceinline__ int ld_flag(const int *p) { return *(volatile const int *)p; }

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
        double srz = 0.0, sbb = 0.0;
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
            srz += b0 * z0 + b1 * z1;
            sbb += b0 * b0 + b1 * b1;
        }
        part_rz[(size_t)blockIdx.x * K + k] = srz;
        part_bb[(size_t)blockIdx.x * K + k] = sbb;
    }
}

// AP = H P (masked to active dofs) and the block partials of pap[k] = P.AP: block = 8 nodes x
// 32 columns (one per lane) or, with VEC (K a multiple of 4), 128 columns (four per lane)
template <bool VEC>
__global__ void __launch_bounds__(256) pcg_apply(const int *__restrict__ idx, const float4 *__restrict__ blk,
                                                 int n_nodes, int K, const float *__restrict__ Pf,
                                                 const double *__restrict__ P, const unsigned char *__restrict__ act,
                                                 float *__restrict__ AP, double *__restrict__ part,
                                                 const PcgCtl *ctl) {
    if (ld_flag(&ctl->done)) return;
    constexpr int CW = VEC ? 4 : 1;                 // columns per lane
    __shared__ HopTile T;
    __shared__ double s_p[8][32 * CW];
    hop_stage(idx, blk, n_nodes, T);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = blockIdx.x * 8 + w, k0 = blockIdx.y * 32 * CW + CW * lane;
    double pp[CW];
#pragma unroll
    for (int c = 0; c < CW; ++c) pp[c] = 0.0;
    if (n < n_nodes && k0 < K) {
        float y0[CW], y1[CW];
        if (VEC) {
            float4 yx, yy;
            hop_row4(T, w, K, k0, Pf, yx, yy);
            *reinterpret_cast<float4 *>(AP + ((size_t)n * 2) * K + k0) = yx;
            *reinterpret_cast<float4 *>(AP + ((size_t)n * 2 + 1) * K + k0) = yy;
            const float a0[4] = {yx.x, yx.y, yx.z, yx.w}, a1[4] = {yy.x, yy.y, yy.z, yy.w};
#pragma unroll
            for (int c = 0; c < CW; ++c) {
                y0[c] = a0[c];
                y1[c] = a1[c];
            }
        } else {
            float yx = 0.f, yy = 0.f;
            for (int q = 0; q < T.cnt[w]; ++q) {
                const int j = T.idx[w][q];
                const float4 b = T.blk[w][q];
                const float vx = __ldg(Pf + ((size_t)j * 2) * K + k0), vy = __ldg(Pf + ((size_t)j * 2 + 1) * K + k0);
                yx = __fmaf_rn(b.x, vx, __fmaf_rn(b.y, vy, yx));
                yy = __fmaf_rn(b.y, vx, __fmaf_rn(b.z, vy, yy));
            }
            AP[((size_t)n * 2) * K + k0] = yx;
            AP[((size_t)n * 2 + 1) * K + k0] = yy;
            y0[0] = yx;
            y1[0] = yy;
        }
        if (act[n]) {
#pragma unroll
            for (int c = 0; c < CW; ++c) {
                const size_t i0 = ((size_t)n * 2) * K + k0 + c;
                pp[c] = P[i0] * (double)y0[c] + P[i0 + K] * (double)y1[c];
            }
        }
    }
#pragma unroll
    for (int c = 0; c < CW; ++c) s_p[w][CW * lane + c] = pp[c];
    __syncthreads();
    for (int t = threadIdx.x; t < 32 * CW; t += blockDim.x) {
        const int k = blockIdx.y * 32 * CW + t;
        if (k >= K) continue;
        double sum = 0.0;
#pragma unroll
        for (int i = 0; i < 8; ++i) sum += s_p[i][t];
        part[(size_t)blockIdx.x * K + k] = sum;
    }
}

__global__ void __launch_bounds__(PT) pcg_step(int n_nodes, int K, const double *__restrict__ rz,
                                               const double *__restrict__ pap, const unsigned char *__restrict__ act,
                                               const double *__restrict__ Minv, double *__restrict__ X,
                                               double *__restrict__ R, double *__restrict__ Z,
                                               const double *__restrict__ P, const float *__restrict__ AP,
                                               double *__restrict__ part_rr, double *__restrict__ part_rz,
                                               const PcgCtl *ctl) {
    if (ld_flag(&ctl->done)) return;
    int n0, n1;
    node_range(n_nodes, n0, n1);
    for (int k = threadIdx.x; k < K; k += PT) {
        const double a = pap[k] > 0.0 ? rz[k] / pap[k] : 0.0;
        double srr = 0.0, srz = 0.0;
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
            srr += r0 * r0 + r1 * r1;
            srz += r0 * z0 + r1 * z1;
        }
        part_rr[(size_t)blockIdx.x * K + k] = srr;
        part_rz[(size_t)blockIdx.x * K + k] = srz;
    }
}

// out_a[k] (and out_b[k]) = sum over blocks b of part_a[b][k] (part_b): one warp per column, lane l
// sums blocks l, l + 32, ... in order, then a fixed shuffle tree (deterministic).  With `check`,
// the last block to finish decides convergence (every column: sqrt(out_a) <= rtol sqrt(bb)) and
// counts the iteration.
__global__ void pcg_colsum(int nb, int K, const double *__restrict__ part_a, const double *__restrict__ part_b,
                           double *__restrict__ out_a, double *__restrict__ out_b, const double *__restrict__ bb,
                           double rtol, int check, PcgCtl *ctl) {
    if (ld_flag(&ctl->done)) return;
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k < K) {
        double sa = 0.0, sb = 0.0;
        for (int b = lane; b < nb; b += 32) {
            sa += part_a[(size_t)b * K + k];
            if (part_b) sb += part_b[(size_t)b * K + k];
        }
        sa = warp_sum_d(sa);
        sb = warp_sum_d(sb);
        if (lane == 0) {
            out_a[k] = sa;
            if (out_b) out_b[k] = sb;
        }
    }
    if (!check) return;
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        s_last = atomicAdd(&ctl->cnt_check, 1) == (int)gridDim.x - 1;
        if (s_last) ctl->cnt_check = 0;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    int ok = 1;
    for (int c = threadIdx.x; c < K; c += blockDim.x) {
        const double bn = fmax(sqrt(__ldcg(bb + c)), 1e-300);
        ok &= sqrt(__ldcg(out_a + c)) <= rtol * bn;
    }
    ok = __syncthreads_and(ok);
    if (threadIdx.x == 0) {
        ctl->iters += 1;
        if (ok) ctl->done = 1;
    }
}

__global__ void __launch_bounds__(PT) pcg_dir(int n_nodes, int K, const double *__restrict__ rz_old,
                                              const double *__restrict__ rz_new, const double *__restrict__ Z,
                                              double *__restrict__ P, float *__restrict__ Pf, const PcgCtl *ctl) {
    if (ld_flag(&ctl->done)) return;
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

struct PcgWork {
    double *R, *Z, *P, *part_a, *part_b, *rz, *rz2, *pap, *rr, *bb;
    float *Pf, *AP;
    PcgCtl *ctl;
    char *op;
};

static int pcg_blocks(int n_nodes) {
    int nb = (n_nodes + 15) / 16;                 // >= 16 nodes per block
    return nb < 1 ? 1 : (nb > 1024 ? 1024 : nb);
}

static size_t carve(int n_nodes, int K, int node_chunk_k, char *base, PcgWork *w) {
    const size_t v = (size_t)n_nodes * 2 * K;
    const int nb = pcg_blocks(n_nodes), na = (n_nodes + 7) / 8;
    const int nparts = nb > na ? nb : na;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += al256(bytes);
        return p;
    };
    w->R = (double *)take(sizeof(double) * v);
    w->Z = (double *)take(sizeof(double) * v);
    w->P = (double *)take(sizeof(double) * v);
    w->Pf = (float *)take(sizeof(float) * v);
    w->AP = (float *)take(sizeof(float) * v);
    w->part_a = (double *)take(sizeof(double) * (size_t)nparts * K);
    w->part_b = (double *)take(sizeof(double) * (size_t)nparts * K);
    w->rz = (double *)take(sizeof(double) * K);
    w->rz2 = (double *)take(sizeof(double) * K);
    w->pap = (double *)take(sizeof(double) * K);
    w->rr = (double *)take(sizeof(double) * K);
    w->bb = (double *)take(sizeof(double) * K);
    w->ctl = (PcgCtl *)take(sizeof(PcgCtl));
    HopView hv;
    w->op = take(hop_layout(n_nodes, node_chunk_k, nullptr, &hv));
    return off;
}

static int assemble(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                    const float *chunk_hess, float inv_np, float alpha_reg, char *op, cudaStream_t s, HopView *hv) {
    hop_layout(n_nodes, node_chunk_k, op, hv);
    cudaError_t e = cudaMemsetAsync(hv->sids, 0xff, sizeof(int) * (size_t)node_chunk_k * n_nodes * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(hv->err, 0, sizeof(int), s);
    if (e != cudaSuccess) return cuda_status(e, "hessian assembly scratch");
    if (n_chunks > 0) {
        hop_scatter<<<(unsigned)((4 * (size_t)n_chunks + 255) / 256), 256, 0, s>>>(frame_dev, chunk_hess, hv->sids,
                                                                                 hv->sblk);
        D2IC_CHECK_LAUNCH("hop_scatter");
    }
    hop_merge<<<(unsigned)((32 * (size_t)n_nodes + 255) / 256), 256, 0, s>>>(frame_dev, hv->sids, hv->sblk, inv_np,
                                                                           alpha_reg, hv->idx, hv->blk, hv->err);
    D2IC_CHECK_LAUNCH("hop_merge");
    return D2IC_OK;
}

static int check_overflow(const HopView &hv, cudaStream_t s) {
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, hv.err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "hessian assembly");
    D2IC_REQUIRE(err == 0, "hessian assembly: a node couples to more than %d nodes", HOP);
    return D2IC_OK;
}

}  // namespace d2ic

using namespace d2ic;

extern "C" size_t d2ic_hessian_op_bytes(int n_nodes, int node_chunk_k) {
    HopView hv;
    if (n_nodes < 1) n_nodes = 1;
    if (node_chunk_k < 1) node_chunk_k = 1;
    return hop_layout(n_nodes, node_chunk_k, nullptr, &hv);
}

extern "C" int d2ic_hessian_assemble(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                                     const float *chunk_hess, float inv_np, float alpha_reg, void *op, size_t op_bytes,
                                     void *stream) {
    D2IC_REQUIRE(frame_dev && op && (chunk_hess || n_chunks == 0) && n_nodes >= 1 && node_chunk_k >= 1 && n_chunks >= 0,
                 "d2ic_hessian_assemble: bad arguments");
    D2IC_REQUIRE(((uintptr_t)op & 255) == 0, "d2ic_hessian_assemble: op must be 256-byte aligned");
    D2IC_REQUIRE(op_bytes >= d2ic_hessian_op_bytes(n_nodes, node_chunk_k), "d2ic_hessian_assemble: op buffer too small");
    cudaStream_t s = (cudaStream_t)stream;
    HopView hv;
    int st = assemble(frame_dev, n_chunks, n_nodes, node_chunk_k, chunk_hess, inv_np, alpha_reg, (char *)op, s, &hv);
    if (st) return st;
    return check_overflow(hv, s);
}

extern "C" int d2ic_hessian_apply(const void *op, int n_nodes, int node_chunk_k, const float *V, int K, float *Y,
                                  void *stream) {
    D2IC_REQUIRE(op && V && Y && n_nodes >= 1 && K >= 1 && node_chunk_k >= 1, "d2ic_hessian_apply: bad arguments");
    HopView hv;
    hop_layout(n_nodes, node_chunk_k, (char *)op, &hv);
    if (K % 4 == 0 && ((uintptr_t)V & 15) == 0 && ((uintptr_t)Y & 15) == 0 &&
        (long long)n_nodes * 2 * K < (1ll << 31)) {
        hop_apply4<<<(unsigned)((n_nodes + 7) / 8), 256, 0, (cudaStream_t)stream>>>(hv.idx, hv.blk, n_nodes, V, K,
                                                                                      Y);
        D2IC_CHECK_LAUNCH("hop_apply4");
    } else {
        hop_apply<<<dim3((unsigned)((n_nodes + 7) / 8), (unsigned)((K + 31) / 32)), 256, 0, (cudaStream_t)stream>>>(
            hv.idx, hv.blk, n_nodes, V, K, Y);
        D2IC_CHECK_LAUNCH("hop_apply");
    }
    return D2IC_OK;
}

extern "C" size_t d2ic_pcg_work_bytes(int n_nodes, int K, int node_chunk_k) {
    PcgWork w;
    if (n_nodes < 1) n_nodes = 1;
    if (K < 1) K = 1;
    if (node_chunk_k < 1) node_chunk_k = 1;
    return carve(n_nodes, K, node_chunk_k, nullptr, &w);
}

extern "C" int d2ic_pcg_solve(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                              const float *chunk_hess, float inv_np, float alpha_reg, const double *Minv,
                              const unsigned char *active, const double *B, double *X, int K, double rtol,
                              int max_iter, void *work, size_t work_bytes, int *iters_out, void *stream) {
    D2IC_REQUIRE(frame_dev && chunk_hess && Minv && active && B && X && work && K >= 1 && n_nodes >= 1 &&
                     node_chunk_k >= 1 && max_iter >= 0,
                 "d2ic_pcg_solve: bad arguments");
    D2IC_REQUIRE(((uintptr_t)work & 255) == 0, "d2ic_pcg_solve: work must be 256-byte aligned");
    PcgWork w;
    const size_t need = carve(n_nodes, K, node_chunk_k, (char *)work, &w);
    D2IC_REQUIRE(work_bytes >= need, "d2ic_pcg_solve: work %zu bytes < %zu needed", work_bytes, need);
    cudaStream_t s = (cudaStream_t)stream;
    HopView hv;
    int st = assemble(frame_dev, n_chunks, n_nodes, node_chunk_k, chunk_hess, inv_np, alpha_reg, w.op, s, &hv);
    if (st) return st;
    cudaError_t e = cudaMemsetAsync(w.ctl, 0, sizeof(PcgCtl), s);
    if (e != cudaSuccess) return cuda_status(e, "pcg control");
    const int nb = pcg_blocks(n_nodes);
    const int rb = (K + 7) / 8;                      // column sums: 8 warps (columns) per block
    pcg_init<<<nb, PT, 0, s>>>(n_nodes, K, B, active, Minv, X, w.R, w.Z, w.P, w.Pf, w.part_a, w.part_b);
    pcg_colsum<<<rb, 256, 0, s>>>(nb, K, w.part_a, w.part_b, w.rz, w.bb, nullptr, 0.0, 0, w.ctl);
    D2IC_CHECK_LAUNCH("pcg init");
    st = check_overflow(hv, s);                      // also waits for the assembly
    if (st) return st;
    const bool vec = K % 4 == 0;                     // Pf and AP are 256-byte aligned
    const int na = (n_nodes + 7) / 8;
    const dim3 ag((unsigned)na, (unsigned)(vec ? (K + 127) / 128 : (K + 31) / 32));
    constexpr int BATCH = 8;                         // iterations launched per host check of the flag
    int it = 0;
    PcgCtl host_ctl = {};
    double *rz = w.rz, *rz_new = w.rz2;
    while (it < max_iter) {
        const int nb_it = max_iter - it < BATCH ? max_iter - it : BATCH;
        for (int i = 0; i < nb_it; ++i) {
            if (vec)
                pcg_apply<true><<<ag, 256, 0, s>>>(hv.idx, hv.blk, n_nodes, K, w.Pf, w.P, active, w.AP, w.part_a, w.ctl);
            else
                pcg_apply<false><<<ag, 256, 0, s>>>(hv.idx, hv.blk, n_nodes, K, w.Pf, w.P, active, w.AP, w.part_a,
                                                    w.ctl);
            pcg_colsum<<<rb, 256, 0, s>>>(na, K, w.part_a, nullptr, w.pap, nullptr, nullptr, 0.0, 0, w.ctl);
            pcg_step<<<nb, PT, 0, s>>>(n_nodes, K, rz, w.pap, active, Minv, X, w.R, w.Z, w.P, w.AP, w.part_a,
                                       w.part_b, w.ctl);
            pcg_colsum<<<rb, 256, 0, s>>>(nb, K, w.part_a, w.part_b, w.rr, rz_new, w.bb, rtol, 1, w.ctl);
            pcg_dir<<<nb, PT, 0, s>>>(n_nodes, K, rz, rz_new, w.Z, w.P, w.Pf, w.ctl);
            double *t = rz;
            rz = rz_new;
            rz_new = t;
        }
        it += nb_it;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&host_ctl, w.ctl, sizeof(PcgCtl), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_status(e, "pcg iteration");
        if (host_ctl.done) break;
    }
    if (iters_out) *iters_out = host_ctl.iters;
    return D2IC_OK;
}
