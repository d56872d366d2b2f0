// Persistent cooperative nonlinear-CG engine for the global FE-DIC objective.
//
// One launch solves a batch of independent frames (the plain GlobalCGSolver
// drop-in is a batch of one).  All frames advance in lock-step "rounds"; one
// round evaluates, for every active frame, the objective and its gradient at
// the frame's current candidate point:
//
//   P phase  (pixels)  each warp takes chunks (<= 256 pixels of one element)
//                      and computes, for the candidate u_c = u + alpha * dir,
//                        r = I2(x + sum_a N_a u_c[a]) - I1,
//                      the chunk's sum r^2 (FP64) and its 8 nodal gradient
//                      partials sum r * dI2/dx * N_a (FP32).  No atomics on data.
//   barrier
//   N phase  (nodes)   per node: gather its chunk partials (node->chunk CSR),
//                      add the spring gradient over the neighbour table,
//                      write the trial gradient, trial point and trial
//                      direction; per group of 512 nodes reduce (FP64, fixed
//                      order) sum r^2, spring energy, g.g, g.(g - g_cur),
//                      g_cur.dir.
//   barrier + R        the last block to arrive reduces the group partials of
//                      each frame (fixed order) and runs the CG control of
//                      d2ic/solver_global_cg.py:362-461 (stop test, PR+ beta,
//                      restart on g.d >= 0, Armijo with 10 halvings and the
//                      forced 2^-10 step), then rebuilds the active list.
//
// Because every partial is written to its own slot and reduced in an order
// fixed by the frame's own data layout, a frame's result does not depend on
// which warps processed it or on which other frames shared the launch.
//
// The gradient at an accepted line-search point is produced by the same pass
// that evaluated it, so an iteration costs one pixel pass per line-search
// trial (the reference's separate value_and_grad pass is not repeated).
//
// Grid barriers are the engine's own (atomic counter + generation word) with a
// globaltimer-bounded wait: a block that waits longer than D2IC_WAIT_NS sets
// an abort flag and every block leaves the kernel at its next barrier.
#include "common.cuh"

namespace d2ic {

constexpr int NG = D2IC_NODE_GROUP;            // threads per block == nodes per group
constexpr int NWARP = NG / 32;
#ifndef D2IC_ENGINE_MINB
#define D2IC_ENGINE_MINB 1   // resident blocks per SM the register budget is sized for
#endif
// Staging each chunk's coefficient tile in shared memory measured slower than
// reading the taps through L1 (each coefficient is reused by ~16 pixels of the
// chunk, which L1 captures; the tile fill adds a dependent round trip per
// chunk), so it is compiled out by default.
#ifndef D2IC_ENGINE_TILE
#define D2IC_ENGINE_TILE 0
#endif
#ifndef D2IC_ENGINE_RPL
#define D2IC_ENGINE_RPL 8    // pixel records per lane prefetched at chunk start (<= 256 / 32)
#endif
constexpr unsigned long long WAIT_NS = 5ull * 1000ull * 1000ull * 1000ull;

enum { ST_EVAL = 0, ST_TRIAL = 1, ST_FORCED = 2, ST_DONE = 3 };
enum { P_JSUM = 0, P_EREG = 1, P_GG = 2, P_GDIFF = 3, P_GD = 4 };

struct FrameState {
    double J_cur, gg_cur, gg_prev, gdiff_cur, gd, J_last, gnorm;
    float alpha, beta;
    int state, k, t, restart, gd_known, nan_seen;
    int iu, igp, igc, igt, idp;
    int n_evals;
    int reported;   // outputs of a finished frame were written by an earlier launch
    int pad2_;
};

// per-frame commands written by the host between launches (control block, after the header)
enum { CMD_INIT = 0, CMD_RUN = 1, CMD_IDLE = 2 };

struct CtlHeader {
    unsigned bar_count;
    unsigned bar_gen;
    int abort;
    int err;
    int n_active;
    int total_chunks;
    int total_groups;
    int rounds;
    unsigned work;
    int max_rounds;
    int pad_[6];
};

struct Ctl {
    CtlHeader *h;
    int *cmd;      // n_frames: CMD_INIT / CMD_RUN / CMD_IDLE
    int *active;   // n_frames
    int *cpre;     // n_frames + 1
    int *gpre;     // n_frames + 1
    FrameState *fs;
};

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// control block: header | cmd | active | cpre | gpre | frame states
__host__ __device__ inline size_t ctl_layout(int n, size_t *o_active, size_t *o_cpre, size_t *o_gpre, size_t *o_fs) {
    size_t off = align256(sizeof(CtlHeader));
    off = align256(off + sizeof(int) * (size_t)n);          // cmd
    *o_active = off;
    off = align256(off + sizeof(int) * (size_t)n);
    *o_cpre = off;
    off = align256(off + sizeof(int) * (size_t)(n + 1));
    *o_gpre = off;
    off = align256(off + sizeof(int) * (size_t)(n + 1));
    *o_fs = off;
    off = align256(off + sizeof(FrameState) * (size_t)n);
    return off;
}

__device__ inline Ctl make_ctl(char *base, int n) {
    size_t oa, oc, og, of;
    ctl_layout(n, &oa, &oc, &og, &of);
    Ctl c;
    c.h = (CtlHeader *)base;
    c.cmd = (int *)(base + align256(sizeof(CtlHeader)));
    c.active = (int *)(base + oa);
    c.cpre = (int *)(base + oc);
    c.gpre = (int *)(base + og);
    c.fs = (FrameState *)(base + of);
    return c;
}

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_vol(const int *p) { return *(volatile const int *)p; }

// Control data is rewritten by other blocks during the launch: read it through
// L2 (never a possibly stale L1 line).
__device__ __forceinline__ FrameState load_fs(const FrameState *p) {
    static_assert(sizeof(FrameState) % 8 == 0, "FrameState size");
    FrameState s;
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(p);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(&s);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(FrameState) / 8); ++i) dst[i] = __ldcg(src + i);
    return s;
}

// node buffers of a frame: 0,1 = u ; 2,3,4 = g ; 5,6 = d
__device__ __forceinline__ float2 *nbuf(const d2ic_frame_t &F, int j) {
    return reinterpret_cast<float2 *>(F.node_ws) + (size_t)j * F.n_nodes;
}

// Candidate point of the current round: u (EVAL) or u + alpha * dir with
// dir = -g (restart / first iteration) or -g + beta * d_prev.  Explicit
// round-to-nearest operations so that the P and N phases produce identical bits.
struct Cand {
    const float2 *u, *g, *d;
    float alpha, beta;
    int mode;   // 0: u, 1: conjugate direction, 2: steepest descent
    __device__ __forceinline__ float2 at(int n, float2 &dir) const {
        const float2 un = __ldcg(u + n);
        if (mode == 0) {
            dir = make_float2(0.f, 0.f);
            return un;
        }
        const float2 gn = __ldcg(g + n);
        float dx = -gn.x, dy = -gn.y;
        if (mode == 1) {
            const float2 dn = __ldcg(d + n);
            dx = __fadd_rn(dx, __fmul_rn(beta, dn.x));
            dy = __fadd_rn(dy, __fmul_rn(beta, dn.y));
        }
        dir = make_float2(dx, dy);
        return make_float2(__fadd_rn(un.x, __fmul_rn(alpha, dx)), __fadd_rn(un.y, __fmul_rn(alpha, dy)));
    }
};

__device__ __forceinline__ Cand make_cand(const d2ic_frame_t &F, const FrameState *S) {
    Cand c;
    // L2 loads (not volatile) so that the eight reads are in flight together
    const int iu = __ldcg(&S->iu), igc = __ldcg(&S->igc), idp = __ldcg(&S->idp);
    const int st = __ldcg(&S->state);
    c.u = nbuf(F, iu);
    c.g = nbuf(F, 2 + igc);
    c.d = nbuf(F, 5 + idp);
    c.alpha = __ldcg(&S->alpha);
    c.beta = __ldcg(&S->beta);
    const int k = __ldcg(&S->k), rs = __ldcg(&S->restart);
    c.mode = (st == ST_EVAL) ? 0 : ((rs || k == 0) ? 2 : 1);
    return c;
}

// ---------------------------------------------------------------------------
// grid barrier (cooperative launch guarantees co-residency)
// ---------------------------------------------------------------------------
template <class F>
__device__ bool grid_barrier(CtlHeader *H, F &&on_last) {
    __shared__ int s_last;
    __shared__ unsigned s_gen;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire_u32(&H->bar_gen);
        __threadfence();
        const unsigned t = atomicAdd(&H->bar_count, 1u);
        s_last = (t == gridDim.x - 1);
        s_gen = gen;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        on_last();
        __syncthreads();
        if (threadIdx.x == 0) {
            H->bar_count = 0;
            __threadfence();
            atomicExch(&H->bar_gen, s_gen + 1);
        }
    } else if (threadIdx.x == 0) {
        const unsigned long long t0 = gtimer();
        while (ld_acquire_u32(&H->bar_gen) == s_gen) {
            if (ld_vol(&H->abort)) break;
            if (gtimer() - t0 > WAIT_NS) {
                H->err = D2IC_WAIT_TIMEOUT;
                atomicExch(&H->abort, 1);
                break;
            }
            __nanosleep(100);
        }
        __threadfence();
    }
    __syncthreads();
    return ld_vol(&H->abort) == 0;
}

// largest s in [0, n) with pre[s] <= x (pre ascending, pre[0] == 0)
__device__ __forceinline__ int find_slot(const int *pre, int n, int x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldcg(pre + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// P phase: one chunk per warp
// ---------------------------------------------------------------------------
constexpr int RPL = D2IC_ENGINE_RPL;          // pixel records per lane, prefetched together
constexpr int TILE_CAP = 1024;                // floats of the per-warp coefficient tile

// Since the Q4 weights of a pixel inside its element are a convex combination,
// every displaced pixel of a chunk lies in the chunk's pixel box shifted by
// [min_a u_a, max_a u_a]; that box plus the cubic stencil and one pixel of
// margin is staged in shared memory once per chunk.  A chunk whose tile would
// not fit, or a pixel that lands outside it, reads global memory instead; both
// paths feed the same tap arithmetic.
template <int KIND>
__device__ __forceinline__ void pixel_chunk(const d2ic_frame_t &F, const Cand &cd, int c, int lane, float *tile) {
    const int pb = __ldg(F.chunk_begin + c), pe = __ldg(F.chunk_begin + c + 1);
    const int2 box = __ldg(reinterpret_cast<const int2 *>(F.chunk_box) + c);
    const uint4 *pix = reinterpret_cast<const uint4 *>(F.pix);
    uint4 rec[RPL > 0 ? RPL : 1];
#pragma unroll
    for (int i = 0; i < RPL; ++i) {
        const int p = pb + lane + 32 * i;
        rec[i] = (p < pe) ? __ldg(pix + p) : make_uint4(0u, 0u, 0u, 0u);
    }
    float2 uc = make_float2(0.f, 0.f);
    int nd = 0, slot = 0;
    if (lane < 4) {
        nd = __ldg(F.chunk_nodes + 4 * c + lane);
        slot = (int)(((unsigned)__ldg(F.chunk_slot + c) >> (8 * lane)) & 0xffu);
        float2 dir;
        uc = cd.at(nd, dir);
    }
    float ux[4], uy[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        ux[a] = __shfl_sync(0xffffffffu, uc.x, a);
        uy[a] = __shfl_sync(0xffffffffu, uc.y, a);
    }
    const Img im{F.coeff, F.W, F.H, F.cpitch, F.pad};
    int tx0 = 0, ty0 = 0, tw = 0, th = 0;
    bool use_tile = false;
    if (KIND == D2IC_INTERP_CUBIC) {
        const float mnx = fminf(fminf(ux[0], ux[1]), fminf(ux[2], ux[3]));
        const float mxx = fmaxf(fmaxf(ux[0], ux[1]), fmaxf(ux[2], ux[3]));
        const float mny = fminf(fminf(uy[0], uy[1]), fminf(uy[2], uy[3]));
        const float mxy = fmaxf(fmaxf(uy[0], uy[1]), fmaxf(uy[2], uy[3]));
        const int bx0 = box.x & 0xffff, by0 = (int)((unsigned)box.x >> 16);
        const int bx1 = box.y & 0xffff, by1 = (int)((unsigned)box.y >> 16);
        tx0 = bx0 + (int)safe_floor(mnx) - 2;
        ty0 = by0 + (int)safe_floor(mny) - 2;
        tw = bx1 + (int)safe_floor(mxx) + 3 - tx0 + 1;
        th = by1 + (int)safe_floor(mxy) + 3 - ty0 + 1;
        use_tile = D2IC_ENGINE_TILE && tw >= 4 && th >= 4 && tw <= 64 && tw * th <= TILE_CAP;
        if (use_tile) {
            // one tile row per warp instruction: lane -> column (two columns per lane when tw > 32)
            const int c0 = clampi(tx0 + lane, -im.pad, im.W - 1 + im.pad) + im.pad;
            const int c1 = clampi(tx0 + lane + 32, -im.pad, im.W - 1 + im.pad) + im.pad;
            for (int ly = 0; ly < th; ++ly) {
                const float *row = im.c + (size_t)(clampi(ty0 + ly, -im.pad, im.H - 1 + im.pad) + im.pad) * im.cp;
                if (lane < tw) tile[ly * tw + lane] = __ldg(row + c0);
                if (lane + 32 < tw) tile[ly * tw + lane + 32] = __ldg(row + c1);
            }
            __syncwarp();
        }
    }
    float jr = 0.f;
    float gxa[4] = {0.f, 0.f, 0.f, 0.f}, gya[4] = {0.f, 0.f, 0.f, 0.f};
    auto one = [&](const uint4 r4) {
        const int x = (int)(r4.x & 0xffffu), y = (int)(r4.x >> 16);
        const float I1 = __uint_as_float(r4.y), xi = __uint_as_float(r4.z), eta = __uint_as_float(r4.w);
        const float a0 = 0.5f * (1.f - xi), a1 = 0.5f * (1.f + xi);
        const float b0 = 0.5f * (1.f - eta), b1 = 0.5f * (1.f + eta);
        const float N[4] = {a0 * b0, a1 * b0, a1 * b1, a0 * b1};
        const float dx = N[0] * ux[0] + N[1] * ux[1] + N[2] * ux[2] + N[3] * ux[3];
        const float dy = N[0] * uy[0] + N[1] * uy[1] + N[2] * uy[2] + N[3] * uy[3];
        int ix, iy;
        float tx, ty;
        split_coord(x, dx, ix, tx);
        split_coord(y, dy, iy, ty);
        float gx, gy, v;
        const int lx = ix - 1 - tx0, ly = iy - 1 - ty0;
        if (use_tile && lx >= 0 && ly >= 0 && lx <= tw - 4 && ly <= th - 4)
            v = sample_cubic_tile(tile, tw, lx, ly, tx, ty, gx, gy);
        else
            v = sample<KIND>(im, ix, iy, tx, ty, gx, gy);
        const float r = v - I1;
        jr += r * r;
        const float rgx = r * gx, rgy = r * gy;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            gxa[a] += rgx * N[a];
            gya[a] += rgy * N[a];
        }
    };
#pragma unroll
    for (int i = 0; i < RPL; ++i)
        if (pb + lane + 32 * i < pe) one(rec[i]);
    for (int p = pb + lane + 32 * RPL; p < pe; p += 32) one(__ldg(pix + p));   // chunks longer than the prefetch
    const DF js = df_warp_sum(DF{jr, 0.f});
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        gxa[a] = warp_sum_f(gxa[a]);
        gya[a] = warp_sum_f(gya[a]);
    }
    if (lane == 0) reinterpret_cast<float2 *>(F.chunk_J)[c] = make_float2(js.hi, js.lo);   // double-float
    if (lane < 4) {                                 // lane a stores node a's partial in the chunk's slot
        const float gx = lane == 0 ? gxa[0] : lane == 1 ? gxa[1] : lane == 2 ? gxa[2] : gxa[3];
        const float gy = lane == 0 ? gya[0] : lane == 1 ? gya[1] : lane == 2 ? gya[2] : gya[3];
        reinterpret_cast<float2 *>(F.node_grad)[(size_t)slot * F.n_nodes + nd] = make_float2(gx, gy);
    }
    __syncwarp();                                   // the tile is reused by the warp's next chunk
}

// ---------------------------------------------------------------------------
// N phase: one group of NG nodes per block
// ---------------------------------------------------------------------------
__device__ __forceinline__ void node_group(const d2ic_frame_t &F, const FrameState *S, int g, DF (*red)[NWARP]) {
    const Cand cd = make_cand(F, S);
    const int n = g * NG + threadIdx.x;
    const int igt = __ldcg(&S->igt), igc = __ldcg(&S->igc), iu = __ldcg(&S->iu), idp = __ldcg(&S->idp);
    DF q[5] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (n < F.n_nodes) {
        // All loads of a batch are issued before any is consumed: the node pass
        // is a short chain of L2 round trips instead of one per table entry.
        // Sums still run in table order.
        constexpr int NB = 4;
        const float2 gc = __ldcg(nbuf(F, 2 + igc) + n);  // issued with the candidate's own loads
        float2 dir;
        const float2 ui = cd.at(n, dir);
        // chunk partials from the node's K slots (unused slots hold 0), in slot order
        float sx = 0.f, sy = 0.f;
        const int K = F.node_chunk_k, Nn = F.n_nodes;
        const float2 *ng = reinterpret_cast<const float2 *>(F.node_grad) + n;
        for (int kb = 0; kb < K; kb += NB) {
            float2 v[NB];
#pragma unroll
            for (int q = 0; q < NB; ++q) v[q] = (kb + q < K) ? __ldcg(ng + (size_t)(kb + q) * Nn) : make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < NB; ++q)
                if (kb + q < K) {
                    sx += v[q].x;
                    sy += v[q].y;
                }
        }
        float rx = 0.f, ry = 0.f, en = 0.f;
        const int md = F.max_deg;
        const int *nbi = F.nbr_index + n;             // column-major: entry k at k * n_nodes
        const float *nbw = F.nbr_weight + n;
        bool alive = true;                               // entries after the first -1 are padding
        constexpr int NBN = 8;
        for (int kb = 0; kb < md && alive; kb += NBN) {
            int jj[NBN];
            float ww[NBN];
#pragma unroll
            for (int q = 0; q < NBN; ++q) {
                jj[q] = (kb + q < md) ? __ldg(nbi + (size_t)(kb + q) * Nn) : -1;
                ww[q] = (kb + q < md) ? __ldg(nbw + (size_t)(kb + q) * Nn) : 0.f;
            }
            float2 uj[NBN];
#pragma unroll
            for (int q = 0; q < NBN; ++q) {
                float2 dj;
                uj[q] = (jj[q] >= 0) ? cd.at(jj[q], dj) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int q = 0; q < NBN; ++q) {
                alive = alive && jj[q] >= 0;
                if (alive) {
                    const float ddx = ui.x - uj[q].x, ddy = ui.y - uj[q].y;
                    rx += ww[q] * ddx;
                    ry += ww[q] * ddy;
                    en += ww[q] * (ddx * ddx + ddy * ddy);
                }
            }
        }
        const float inv_np = 1.0f / (float)max(F.n_pix, 1);
        const float gx = sx * inv_np + F.alpha_reg * rx;
        const float gy = sy * inv_np + F.alpha_reg * ry;
        nbuf(F, 2 + igt)[n] = make_float2(gx, gy);
        nbuf(F, 1 - iu)[n] = ui;
        nbuf(F, 5 + (1 - idp))[n] = dir;
        // per-node terms of the inner products, exact in double-float (g - g_cur rounded
        // in FP32 as the reference's elementwise difference)
        q[P_EREG] = DF{0.25f * en, 0.f};
        q[P_GG] = df_add(df_prod(gx, gx), df_prod(gy, gy));
        q[P_GDIFF] = df_add(df_prod(gx, gx - gc.x), df_prod(gy, gy - gc.y));
        q[P_GD] = df_add(df_prod(gc.x, dir.x), df_prod(gc.y, dir.y));
    }
    // this group's share of the chunk sums of r^2
    {
        const int c0 = g * F.chunks_per_group;
        const int c1 = min(c0 + F.chunks_per_group, F.n_chunks);
        const float2 *cj = reinterpret_cast<const float2 *>(F.chunk_J);
        for (int c = c0 + (int)threadIdx.x; c < c1; c += NG) {
            const float2 v = __ldcg(cj + c);
            q[P_JSUM] = df_add(q[P_JSUM], DF{v.x, v.y});
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const DF v = df_warp_sum(q[i]);
        if (lane == 0) red[i][wid] = v;
    }
    __syncthreads();
    if (wid == 0) {                                // warp 0: one warp-sum per quantity, fixed order
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const DF v = df_warp_sum(lane < NWARP ? red[i][lane] : DF{0.f, 0.f});
            if (lane == 0) F.group_part[(size_t)g * D2IC_NPART + i] = df_to_double(v);
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// R step (last block at the end-of-round barrier)
// ---------------------------------------------------------------------------
__device__ void hist_row(const d2ic_frame_t &F, int k, double a, double b, double c) {
    if (F.hist && k < F.max_iter) {
        F.hist[3 * k + 0] = (float)a;
        F.hist[3 * k + 1] = (float)b;
        F.hist[3 * k + 2] = (float)c;
    }
}

__device__ void accept_point(FrameState &S, double J, double gg, double gdiff) {
    S.J_cur = J;
    S.gg_prev = S.gg_cur;
    S.gg_cur = gg;
    S.gdiff_cur = gdiff;
    const int gp = S.igp;
    S.igp = S.igc;
    S.igc = S.igt;
    S.igt = gp;
    S.iu = 1 - S.iu;
    S.idp = 1 - S.idp;
}

__device__ void start_iter(FrameState &S, const d2ic_frame_t &F) {
    S.gnorm = sqrt(S.gg_cur);
    if (S.gnorm < F.tol) {                       // stop branch: k unchanged
        hist_row(F, S.k, S.J_cur, S.gnorm, 0.0);
        S.state = ST_DONE;
        return;
    }
    double beta = 0.0;
    if (S.k > 0) {
        const double x = S.gdiff_cur / (S.gg_prev + 1e-16);
        beta = (x != x) ? x : fmax(x, 0.0);      // jnp.maximum keeps NaN
    }
    S.beta = (float)beta;
    S.alpha = 1.0f;
    S.t = 0;
    S.restart = 0;
    S.gd_known = 0;
    S.state = ST_TRIAL;
}

__device__ void frame_decide(FrameState &S, const d2ic_frame_t &F, const double *q, int eval_only) {
    const double J = 0.5 * q[P_JSUM] / (double)max(F.n_pix, 1) + (double)F.alpha_reg * q[P_EREG];
    if (J != J || q[P_GG] != q[P_GG]) S.nan_seen = 1;
    S.n_evals += 1;
    // control-flow guard: an iteration takes at most 11 evaluations plus one restart
    if (S.n_evals > 12 * max(F.max_iter, 0) + 4) {
        S.state = ST_DONE;
        return;
    }
    switch (S.state) {
        case ST_EVAL:
            accept_point(S, J, q[P_GG], q[P_GDIFF]);
            if (eval_only || F.max_iter <= 0) {
                S.state = ST_DONE;
                return;
            }
            start_iter(S, F);
            return;
        case ST_TRIAL: {
            if (!S.gd_known) {
                S.gd_known = 1;
                S.gd = q[P_GD];
                if (S.gd >= 0.0) {                 // not a descent direction: restart with -g
                    S.restart = 1;
                    S.gd = -S.gg_cur;
                    S.alpha = 1.0f;
                    return;                        // re-evaluate trial 0 along -g
                }
            }
            if (J <= S.J_cur + 1e-4 * (double)S.alpha * S.gd) {
                hist_row(F, S.k, J, S.gnorm, (double)S.alpha);
                S.k += 1;
                accept_point(S, J, q[P_GG], q[P_GDIFF]);
                if (S.k >= F.max_iter) S.state = ST_DONE;
                else start_iter(S, F);
            } else {
                S.J_last = J;
                S.t += 1;
                S.alpha *= 0.5f;
                if (S.t >= 10) S.state = ST_FORCED;   // alpha == 2^-10 is applied anyway
            }
            return;
        }
        case ST_FORCED:
            hist_row(F, S.k, S.J_last, S.gnorm, (double)S.alpha);
            S.k += 1;
            accept_point(S, J, q[P_GG], q[P_GDIFF]);
            if (S.k >= F.max_iter) S.state = ST_DONE;
            else start_iter(S, F);
            return;
        default:
            return;
    }
}

// exclusive block-wide scan of three counters (warp shuffles + one shared pass)
__device__ __forceinline__ void block_scan3(int &a, int &b, int &c, int &ta, int &tb, int &tc) {
    __shared__ int s_w[NWARP][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int ia = a, ib = b, ic = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o),
                  xc = __shfl_up_sync(0xffffffffu, ic, o);
        if (lane >= o) { ia += xa; ib += xb; ic += xc; }
    }
    if (lane == 31) { s_w[wid][0] = ia; s_w[wid][1] = ib; s_w[wid][2] = ic; }
    __syncthreads();
    int oa = 0, ob = 0, oc = 0;
    ta = tb = tc = 0;
    for (int w = 0; w < NWARP; ++w) {
        if (w == wid) { oa = ta; ob = tb; oc = tc; }
        ta += s_w[w][0]; tb += s_w[w][1]; tc += s_w[w][2];
    }
    a = oa + ia - a;
    b = ob + ib - b;
    c = oc + ic - c;
    __syncthreads();
}

// rebuild the active list and prefix sums (whole block)
__device__ void rebuild_active(const d2ic_frame_t *frames, int n_frames, Ctl &C) {
    const int per = (n_frames + NG - 1) / NG;
    const int f0 = threadIdx.x * per, f1 = min(f0 + per, n_frames);
    int cnt = 0, ch = 0, gr = 0;
    for (int f = f0; f < f1; ++f)
        if (ld_vol(&C.fs[f].state) != ST_DONE) {
            ++cnt;
            ch += frames[f].n_chunks;
            gr += frames[f].n_groups;
        }
    int ta, tb, tc;
    block_scan3(cnt, ch, gr, ta, tb, tc);
    if (threadIdx.x == 0) {
        C.h->n_active = ta;
        C.h->total_chunks = tb;
        C.h->total_groups = tc;
        C.cpre[ta] = tb;
        C.gpre[ta] = tc;
    }
    int slot = cnt, cp = ch, gp = gr;
    for (int f = f0; f < f1; ++f)
        if (ld_vol(&C.fs[f].state) != ST_DONE) {
            C.active[slot] = f;
            C.cpre[slot] = cp;
            C.gpre[slot] = gp;
            ++slot;
            cp += frames[f].n_chunks;
            gp += frames[f].n_groups;
        }
    __syncthreads();
}

// Start of a launch: new frames (CMD_INIT) get a fresh CG state, idle slots are
// parked as finished-and-reported, running frames keep their state; frames
// that finished in an earlier launch are marked reported (their outputs were
// written at the end of that launch).
__device__ void r_init(const d2ic_frame_t *frames, int n_frames, Ctl &C) {
    for (int f = threadIdx.x; f < n_frames; f += NG) {
        const int cmd = ld_vol(C.cmd + f);
        if (cmd == CMD_INIT) {
            FrameState S;
            S.J_cur = S.gg_cur = S.gg_prev = S.gdiff_cur = S.gd = S.J_last = S.gnorm = 0.0;
            S.alpha = 0.f;
            S.beta = 0.f;
            S.k = S.t = S.restart = S.gd_known = S.nan_seen = S.n_evals = 0;
            S.iu = 0; S.igp = 0; S.igc = 1; S.igt = 2; S.idp = 0;
            S.state = ST_EVAL;
            S.reported = 0;
            S.pad2_ = 0;
            C.fs[f] = S;
            C.cmd[f] = CMD_RUN;
        } else if (cmd == CMD_IDLE) {
            C.fs[f].state = ST_DONE;
            C.fs[f].reported = 1;
        } else if (ld_vol(&C.fs[f].state) == ST_DONE) {
            C.fs[f].reported = 1;
        }
    }
    __syncthreads();
    rebuild_active(frames, n_frames, C);
}

__device__ void r_step(const d2ic_frame_t *frames, int n_frames, Ctl &C, int eval_only) {
    __shared__ int s_finished;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_finished = 0;
    __syncthreads();
    const int na = ld_vol(&C.h->n_active);
    for (int s = wid; s < na; s += NWARP) {
        const int f = ld_vol(C.active + s);
        const d2ic_frame_t &F = frames[f];
        FrameState S;
        if (lane == 0) S = load_fs(C.fs + f);          // issued together with the partial loads below
        double q[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int g = lane; g < F.n_groups; g += 32) {
#pragma unroll
            for (int i = 0; i < 5; ++i) q[i] += __ldcg(F.group_part + (size_t)g * D2IC_NPART + i);
        }
#pragma unroll
        for (int i = 0; i < 5; ++i) q[i] = warp_sum_d(q[i]);
        if (lane == 0) {
            frame_decide(S, F, q, eval_only);
            C.fs[f] = S;
            if (S.state == ST_DONE) s_finished = 1;
        }
    }
    __syncthreads();
    if (s_finished) rebuild_active(frames, n_frames, C);   // else the active lists stay as they are
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------
template <int KIND>
__global__ void __launch_bounds__(NG, D2IC_ENGINE_MINB) cg_engine(const d2ic_frame_t *__restrict__ frames, int n_frames,
                                                   char *ctl_base, int eval_only, const float *u_eval,
                                                   double *J_out, float *grad_out, unsigned long long *trace,
                                                   int trace_rounds, int max_rounds) {
    __shared__ DF red[5][NWARP];
    extern __shared__ float s_tile[];              // NWARP * TILE_CAP floats
    Ctl C = make_ctl(ctl_base, n_frames);
    const int lane = threadIdx.x & 31;
    // optional phase trace: block 0 stamps [round start, after P barrier, end of its N, -, -, after R
    // barrier, end of its own P work]; the last block stamps the start and end of its R step into
    // slots 3 and 4
    const bool tr = trace != nullptr && blockIdx.x == 0 && threadIdx.x == 0;
    int round = 0;

    // ---- init of newly admitted frames: u <- u0, zero g/d buffers and gradient slots, NaN history ----
    for (int f = 0; f < n_frames; ++f) {
        if (ld_vol(C.cmd + f) != CMD_INIT) continue;
        const d2ic_frame_t &F = frames[f];
        const int nn = F.n_nodes;
        const float2 *u0 = reinterpret_cast<const float2 *>((eval_only && u_eval && f == 0) ? u_eval : F.u0);
        for (int i = blockIdx.x * NG + threadIdx.x; i < nn; i += gridDim.x * NG) {
            nbuf(F, 0)[i] = u0 ? u0[i] : make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 1; j < 7; ++j) nbuf(F, j)[i] = make_float2(0.f, 0.f);
        }
        // gradient slots that no chunk owns must read as 0
        float2 *ng = reinterpret_cast<float2 *>(F.node_grad);
        for (size_t i = blockIdx.x * NG + threadIdx.x; i < (size_t)F.node_chunk_k * nn; i += (size_t)gridDim.x * NG)
            ng[i] = make_float2(0.f, 0.f);
        if (F.hist)
            for (int i = blockIdx.x * NG + threadIdx.x; i < 3 * F.max_iter; i += gridDim.x * NG)
                F.hist[i] = __int_as_float(0x7fc00000);
    }
    if (!grid_barrier(C.h, [&] { r_init(frames, n_frames, C); })) goto finish;

    while (round < max_rounds) {                    // a slice: at most max_rounds rounds, state kept in HBM
        const int na = ld_vol(&C.h->n_active);
        if (na == 0) break;
        const bool trr = tr && round < trace_rounds;
        if (trr) trace[7 * round + 0] = gtimer();
        // ---- P phase: chunk c of the active list goes to global warp c mod (warps in grid) ----
        {
            const int total = ld_vol(&C.h->total_chunks);
            const int gw = (int)((blockIdx.x * NG + threadIdx.x) >> 5);
            const int nw = (int)((gridDim.x * NG) >> 5);
            int cbase = 0, cend = 0;
            const d2ic_frame_t *Fp = frames;
            Cand cd;
            for (int c = gw; c < total; c += nw) {
                if (c >= cend) {                      // chunks ascend per warp: frames change forward only
                    const int s = find_slot(C.cpre, na, c);
                    const int f = __ldcg(C.active + s);
                    cbase = __ldcg(C.cpre + s);
                    cend = __ldcg(C.cpre + s + 1);
                    Fp = frames + f;
                    cd = make_cand(*Fp, C.fs + f);
                }
                pixel_chunk<KIND>(*Fp, cd, c - cbase, lane, s_tile + (threadIdx.x >> 5) * TILE_CAP);
            }
        }
        if (trace != nullptr && blockIdx.x == 0 && round < trace_rounds) {
            __syncthreads();
            if (threadIdx.x == 0) trace[7 * round + 6] = gtimer();
        }
        if (!grid_barrier(C.h, [] {})) break;
        if (trr) trace[7 * round + 1] = gtimer();
        // ---- N phase ----
        {
            const int tg = ld_vol(&C.h->total_groups);
            for (int gi = blockIdx.x; gi < tg; gi += gridDim.x) {
                const int s = find_slot(C.gpre, na, gi);
                const int f = __ldcg(C.active + s);
                node_group(frames[f], C.fs + f, gi - __ldcg(C.gpre + s), red);
            }
        }
        if (trr) trace[7 * round + 2] = gtimer();
        if (!grid_barrier(C.h, [&] {
                const bool rt = trace != nullptr && threadIdx.x == 0 && round < trace_rounds;
                if (rt) trace[7 * round + 3] = gtimer();
                r_step(frames, n_frames, C, eval_only);
                if (rt) trace[7 * round + 4] = gtimer();
            }))
            break;
        if (trr) trace[7 * round + 5] = gtimer();
        ++round;
    }

finish:
    // ---- outputs of frames that finished in this launch; running frames report D2IC_RUNNING ----
    const bool aborted = ld_vol(&C.h->abort) != 0;
    for (int f = 0; f < n_frames; ++f) {
        const d2ic_frame_t &F = frames[f];
        const FrameState *S = C.fs + f;
        const bool done = ld_vol(&S->state) == ST_DONE;
        if (!(aborted || eval_only || (done && !ld_vol(&S->reported)))) {
            if (!done && blockIdx.x == 0 && threadIdx.x == 0 && F.status) *F.status = D2IC_RUNNING;
            continue;
        }
        const int iu = ld_vol(&S->iu), igc = ld_vol(&S->igc);
        const int nn = F.n_nodes;
        float2 *uo = reinterpret_cast<float2 *>(F.u_out);
        for (int i = blockIdx.x * NG + threadIdx.x; i < nn; i += gridDim.x * NG) {
            if (uo) uo[i] = __ldcg(nbuf(F, iu) + i);
            if (eval_only && grad_out && f == 0) reinterpret_cast<float2 *>(grad_out)[i] = __ldcg(nbuf(F, 2 + igc) + i);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (F.n_iters) *F.n_iters = ld_vol(&S->k);
            if (F.n_evals) *F.n_evals = ld_vol(&S->n_evals);
            int st = D2IC_OK;
            if (aborted) st = ld_vol(&C.h->err);
            else if (ld_vol(&S->nan_seen)) st = D2IC_NAN_DETECTED;
            else if (ld_vol(&S->k) >= F.max_iter && F.max_iter > 0) st = D2IC_MAX_ITERS;
            if (F.status) *F.status = st;
            if (eval_only && J_out && f == 0) *J_out = *(volatile const double *)&S->J_cur;
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
constexpr size_t ENGINE_SMEM = sizeof(float) * NWARP * TILE_CAP;   // per-warp coefficient tiles

template <int KIND>
static cudaError_t occupancy(int *blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(cg_engine<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ENGINE_SMEM);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, cg_engine<KIND>, NG, ENGINE_SMEM);
}

struct DevInfo {
    int sms = 0, bps[2] = {0, 0};
};
static DevInfo g_dev[64];

static int dev_info(int dev, DevInfo **out) {
    if (dev < 0 || dev >= 64) {
        set_error("device index %d out of range", dev);
        return D2IC_BAD_ARG;
    }
    DevInfo &d = g_dev[dev];
    if (d.sms == 0) {
        cudaError_t e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return cuda_status(e, "cudaDeviceGetAttribute");
        e = occupancy<D2IC_INTERP_CUBIC>(&d.bps[0]);
        if (e != cudaSuccess) return cuda_status(e, "occupancy");
        e = occupancy<D2IC_INTERP_LINEAR>(&d.bps[1]);
        if (e != cudaSuccess) return cuda_status(e, "occupancy");
    }
    *out = &d;
    return D2IC_OK;
}

static int launch_engine(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes, int kind,
                         int grid_blocks, int eval_only, const float *u_eval, double *J_out, float *grad_out,
                         unsigned long long *trace, int trace_rounds, cudaStream_t s, int max_rounds = 0x7fffffff,
                         bool new_batch = true) {
    D2IC_REQUIRE(frames && control, "cg engine: null pointer");
    D2IC_REQUIRE(n_frames >= 1 && n_frames <= D2IC_MAX_FRAMES, "cg engine: n_frames %d out of [1, %d]", n_frames,
                 D2IC_MAX_FRAMES);
    D2IC_REQUIRE(kind == D2IC_INTERP_CUBIC || kind == D2IC_INTERP_LINEAR, "cg engine: unknown interpolation %d", kind);
    D2IC_REQUIRE(((uintptr_t)control & 255) == 0, "cg engine: control scratch must be 256-byte aligned");
    const size_t need = d2ic_cg_control_bytes(n_frames);
    D2IC_REQUIRE(control_bytes >= need, "cg engine: control scratch %zu bytes < %zu needed", control_bytes, need);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    DevInfo *di = nullptr;
    int st = dev_info(dev, &di);
    if (st) return st;
    const int maxb = di->sms * di->bps[kind == D2IC_INTERP_LINEAR];
    D2IC_REQUIRE(maxb > 0, "cg engine: kernel cannot be resident on this device");
    int blocks = grid_blocks > 0 ? (grid_blocks < maxb ? grid_blocks : maxb) : maxb;
    // header always; with new_batch also the command words (all frames CMD_INIT == 0)
    const size_t clear = new_batch ? align256(sizeof(CtlHeader)) + sizeof(int) * (size_t)n_frames : sizeof(CtlHeader);
    e = cudaMemsetAsync(control, 0, clear, s);
    if (e != cudaSuccess) return cuda_status(e, "control reset");
    char *cb = (char *)control;
    // cooperative launch through cudaLaunchKernelEx (co-residency checked by the driver; capturable)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(NG);
    cfg.dynamicSmemBytes = ENGINE_SMEM;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (kind == D2IC_INTERP_CUBIC)
        e = cudaLaunchKernelEx(&cfg, cg_engine<D2IC_INTERP_CUBIC>, frames, n_frames, cb, eval_only, u_eval, J_out,
                               grad_out, trace, trace_rounds, max_rounds);
    else
        e = cudaLaunchKernelEx(&cfg, cg_engine<D2IC_INTERP_LINEAR>, frames, n_frames, cb, eval_only, u_eval, J_out,
                               grad_out, trace, trace_rounds, max_rounds);
    if (e != cudaSuccess) return cuda_status(e, "cooperative launch of cg_engine");
    return D2IC_OK;
}

}  // namespace d2ic

using namespace d2ic;

extern "C" size_t d2ic_cg_control_bytes(int n_frames) {
    if (n_frames < 1) n_frames = 1;
    size_t a, b, c, d;
    return ctl_layout(n_frames, &a, &b, &c, &d);
}

extern "C" size_t d2ic_frame_workspace_bytes(int n_nodes, int n_chunks, int node_chunk_k) {
    const int ng = (n_nodes + NG - 1) / NG;
    if (node_chunk_k < 1) node_chunk_k = 1;
    size_t off = align256(sizeof(float) * 14 * (size_t)n_nodes);
    off += align256(sizeof(double) * (size_t)n_chunks);
    off += align256(sizeof(float) * 2 * (size_t)node_chunk_k * n_nodes);
    off += align256(sizeof(double) * D2IC_NPART * (size_t)(ng > 0 ? ng : 1));
    return off;
}

extern "C" int d2ic_frame_bind_workspace(d2ic_frame_t *f, void *ws) {
    D2IC_REQUIRE(f && ws, "d2ic_frame_bind_workspace: null pointer");
    D2IC_REQUIRE(((uintptr_t)ws & 255) == 0, "d2ic_frame_bind_workspace: workspace must be 256-byte aligned");
    D2IC_REQUIRE(f->n_nodes >= 1 && f->n_chunks >= 0 && f->node_chunk_k >= 1 && f->node_chunk_k <= 255,
                 "d2ic_frame_bind_workspace: bad sizes");
    char *p = (char *)ws;
    f->node_ws = (float *)p;
    p += align256(sizeof(float) * 14 * (size_t)f->n_nodes);
    f->chunk_J = (double *)p;
    p += align256(sizeof(double) * (size_t)f->n_chunks);
    f->node_grad = (float *)p;
    p += align256(sizeof(float) * 2 * (size_t)f->node_chunk_k * f->n_nodes);
    f->group_part = (double *)p;
    f->n_groups = (f->n_nodes + NG - 1) / NG;
    f->chunks_per_group = (f->n_chunks + f->n_groups - 1) / f->n_groups;
    return D2IC_OK;
}

extern "C" int d2ic_device_info(int device, int *num_sms, int *engine_blocks_per_sm) {
    DevInfo *di = nullptr;
    int st = dev_info(device, &di);
    if (st) return st;
    if (num_sms) *num_sms = di->sms;
    if (engine_blocks_per_sm) *engine_blocks_per_sm = di->bps[0];
    return D2IC_OK;
}

extern "C" int d2ic_cg_solve_batched(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes,
                                     int interp_kind, int grid_blocks, void *stream) {
    return launch_engine(frames, n_frames, control, control_bytes, interp_kind, grid_blocks, 0, nullptr, nullptr,
                         nullptr, nullptr, 0, (cudaStream_t)stream);
}

extern "C" size_t d2ic_cg_command_offset(void) { return align256(sizeof(CtlHeader)); }

extern "C" int d2ic_cg_slice(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes,
                             int interp_kind, int grid_blocks, int max_rounds, void *stream) {
    D2IC_REQUIRE(max_rounds >= 1, "d2ic_cg_slice: max_rounds must be >= 1 (got %d)", max_rounds);
    return launch_engine(frames, n_frames, control, control_bytes, interp_kind, grid_blocks, 0, nullptr, nullptr,
                         nullptr, nullptr, 0, (cudaStream_t)stream, max_rounds, false);
}

extern "C" int d2ic_cg_solve_traced(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes,
                                    int interp_kind, int grid_blocks, unsigned long long *trace, int trace_rounds,
                                    void *stream) {
    D2IC_REQUIRE(trace && trace_rounds > 0, "d2ic_cg_solve_traced: need a trace buffer");
    return launch_engine(frames, n_frames, control, control_bytes, interp_kind, grid_blocks, 0, nullptr, nullptr,
                         nullptr, trace, trace_rounds, (cudaStream_t)stream);
}

extern "C" int d2ic_eval_objective(const d2ic_frame_t *frame, const float *u, void *control, size_t control_bytes,
                                   int interp_kind, double *J_out, float *grad_out, void *stream) {
    D2IC_REQUIRE(u && J_out && grad_out, "d2ic_eval_objective: null pointer");
    return launch_engine(frame, 1, control, control_bytes, interp_kind, 0, 1, u, J_out, grad_out, nullptr, 0,
                         (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Solve without allocating: scratch in a fixed device array
// ---------------------------------------------------------------------------
// For callers that cannot call cudaMalloc (an allocator-less runtime, a
// plugin host that owns all device memory, code running where allocation is
// forbidden): the engine's scratch -- the frame descriptor copy, the control
// block and the per-frame workspace -- is carved from this file-scope device
// array instead of caller memory.  Every GPU that loads the library holds the
// array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[D2IC_NOALLOC_SCRATCH_BYTES];
static void *g_noalloc_addr[64];   // device address of the array, per device (host-side stand-in is not usable)

extern "C" int d2ic_cg_solve_noalloc(const d2ic_frame_t *frame, int interp_kind, void *stream) {
    D2IC_REQUIRE(frame, "d2ic_cg_solve_noalloc: null frame");
    D2IC_REQUIRE(frame->n_nodes >= 1 && frame->n_chunks >= 0, "d2ic_cg_solve_noalloc: bad sizes");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    D2IC_REQUIRE(dev >= 0 && dev < 64, "d2ic_cg_solve_noalloc: device index %d out of range", dev);
    const size_t desc_bytes = align256(sizeof(d2ic_frame_t));
    const size_t ctl_bytes = d2ic_cg_control_bytes(1);
    D2IC_REQUIRE(frame->node_chunk_k >= 1 && frame->node_chunk_k <= 255, "d2ic_cg_solve_noalloc: bad node_chunk_k");
    const size_t ws_bytes = d2ic_frame_workspace_bytes(frame->n_nodes, frame->n_chunks, frame->node_chunk_k);
    const size_t need = desc_bytes + ctl_bytes + ws_bytes;
    D2IC_REQUIRE(need <= (size_t)D2IC_NOALLOC_SCRATCH_BYTES,
                 "d2ic_cg_solve_noalloc: frame needs %zu bytes of scratch (%d nodes, %d chunks), more than the "
                 "fixed %zu-byte array; use d2ic_cg_solve_batched with caller-allocated scratch",
                 need, frame->n_nodes, frame->n_chunks, (size_t)D2IC_NOALLOC_SCRATCH_BYTES);
    if (g_noalloc_addr[dev] == nullptr) {      // set-up, once per device, with that device current
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(noalloc scratch)");
        g_noalloc_addr[dev] = p;
    }
    char *base = (char *)g_noalloc_addr[dev];
    d2ic_frame_t f = *frame;                   // caller's inputs/outputs, workspace from the array
    int st = d2ic_frame_bind_workspace(&f, base + desc_bytes + ctl_bytes);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // pageable-source copy: returns once `f` has been staged, so the stack copy may go out of scope
    e = cudaMemcpyAsync(base, &f, sizeof(f), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_status(e, "noalloc descriptor copy");
    // the launch clears the control header on `s`; the kernel initialises every workspace word it reads
    return launch_engine((const d2ic_frame_t *)base, 1, base + desc_bytes, ctl_bytes, interp_kind, 0, 0, nullptr,
                         nullptr, nullptr, nullptr, 0, s);
}
