// Persistent cooperative nonlinear-CG engine for the global FE-DIC objective.
//
// One launch solves a batch of independent frames (the plain GlobalCGSolver
// drop-in is a batch of one, run by a one-frame instance of the kernel).  All
// frames advance in lock-step "rounds"; one round evaluates, for every active
// frame, the objective and its gradient at the frame's current candidate point:
//
//   pixel pass   each warp takes chunks (<= 256 pixels of one element) and
//                computes, for the candidate u_c = u + alpha * dir,
//                  r = I2(x + sum_a N_a u_c[a]) - I1,
//                the chunk's sum r^2 (double-float) and its 8 nodal gradient
//                partials sum r * dI2/dx * N_a (FP32), written to the chunk's
//                own node slots; then it counts its chunks into the node
//                groups (32 nodes) they touch.  No atomics on data.
//   node work    the warp that owns a group waits (bounded) until every chunk
//                of the group has counted, gathers each node's slots, adds the
//                spring gradient over the neighbour table, writes the trial
//                gradient, point and direction, and reduces (fixed order) sum
//                r^2, spring energy, g.g, g.(g - g_cur), g_cur.dir; the warp
//                that completes a supergroup of 16 groups reduces it, and the
//                warp that completes a frame's last supergroup runs the CG
//                control of d2ic/solver_global_cg.py:362-461 (stop test, PR+
//                beta, restart on g.d >= 0, Armijo with 10 halvings and the
//                forced 2^-10 step); the frame's round counter releases the
//                next round.
//
// Because every partial is written to its own slot and reduced in an order
// fixed by the frame's own data layout, a frame's result does not depend on
// which warps processed it or on which other frames shared the launch.
//
// The gradient at an accepted line-search point is produced by the same pass
// that evaluated it, so an iteration costs one pixel pass per line-search
// trial (the reference's separate value_and_grad pass is not repeated).
//
// Every wait is bounded by the globaltimer (the launch's grid barrier, the group
// and round waits: WAIT_NS; the TMA/cp.async completions: TMA_WAIT_NS): a warp
// that waits longer sets D2IC_WAIT_TIMEOUT and an abort flag, drains its own
// copies and every block leaves the kernel.
#include <cuda.h>   // CUtensorMap and its enums (the encoder is fetched from the driver at run time)
#include <stddef.h>
#include <string.h>

#include <atomic>

#include "common.cuh"

namespace d2ic {

constexpr int NT = 512;                        // threads per block
constexpr int NWARP = NT / 32;
static_assert(NWARP == 16, "a supergroup is the warps of one block");
constexpr int GN = D2IC_NODE_GROUP;            // nodes per group: one per lane of the warp that reduces it
static_assert(GN == 32, "a node group is one warp");
// Groups per supergroup.  A frame's group range in the active list is padded to a multiple of
// SG, so when every warp owns at most one group, supergroup sg of a frame is owned by warps
// 0 .. SG-1 of one block and is reduced through that block's shared memory.
constexpr int SG = 16;
__host__ __device__ constexpr int pad_groups(int n) { return (n + SG - 1) / SG * SG; }
#ifndef D2IC_ENGINE_MINB
#define D2IC_ENGINE_MINB 1   // resident blocks per SM the register budget is sized for
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
enum { CMD_INIT = 0, CMD_RUN = 1, CMD_IDLE = 2, CMD_HOLD = 3 };

struct CtlHeader {
    unsigned bar_count;
    unsigned bar_gen;
    int abort;
    int err;
    int n_active;
    int total_chunks;
    int total_groups;
    unsigned rounds_done;   // rounds completed in this launch (released by the round's last frame step)
    int finished;           // a frame finished in this round: the active list is rebuilt before release
    int max_rounds;
    int frames_done;        // frames whose control step ran in the current round
    int slice_stop;         // the slice ends after the released round (set before the release)
    int irq;                // written by the host while a slice runs: end the slice at the next round end
    int list_buf;           // which of the two copies of the active list the current round reads
    unsigned blocks_past;   // block arrivals at round ends: every block has finished a round's list reads
    int pad_;
};
static_assert(sizeof(CtlHeader) == 64, "control header layout");

// stop_flags of a slice: end it early
enum { STOP_ON_FINISH = D2IC_STOP_ON_FINISH,   // after a round in which a frame finished
       STOP_ON_IRQ = D2IC_STOP_ON_IRQ };         // after a round that ends with the header's irq word set

// The active list is double-buffered: a round reads copy h->list_buf while the warp that ends
// the round may rebuild the list into the other copy (a frame finished) and flips list_buf before
// the release.  Warps still walking the round's list -- lookups of padding groups, or the
// rebuilding warp itself after the release -- therefore never see a half-written list.  Before it
// writes, the rebuilding warp of round r waits until every block has passed the end of round r-1
// (blocks_past), so no block still reads an older round's copy either.
struct Ctl {
    CtlHeader *h;
    int *cmd;      // n_frames: CMD_INIT / CMD_RUN / CMD_IDLE / CMD_HOLD
    int *active;   // two copies of n_frames
    int *cpre;     // two copies of n_frames + 1
    int *gpre;     // two copies of n_frames + 1
    FrameState *fs;
    int n;         // n_frames
    __device__ __forceinline__ int *act(int b) const { return active + b * n; }
    __device__ __forceinline__ int *cp(int b) const { return cpre + b * (n + 1); }
    __device__ __forceinline__ int *gp(int b) const { return gpre + b * (n + 1); }
};

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// control block: header | cmd | active | cpre | gpre | frame states
__host__ __device__ inline size_t ctl_layout(int n, size_t *o_active, size_t *o_cpre, size_t *o_gpre, size_t *o_fs) {
    size_t off = align256(sizeof(CtlHeader));
    off = align256(off + sizeof(int) * (size_t)n);          // cmd
    *o_active = off;                                        // two copies of each list array
    off = align256(off + 2 * sizeof(int) * (size_t)n);
    *o_cpre = off;
    off = align256(off + 2 * sizeof(int) * (size_t)(n + 1));
    *o_gpre = off;
    off = align256(off + 2 * sizeof(int) * (size_t)(n + 1));
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
    c.n = n;
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
// mode 0: u, 1: conjugate direction, 2: steepest descent.
__device__ __forceinline__ float2 cand_value(float2 un, float2 gn, float2 dn, float alpha, float beta, int mode,
                                             float2 &dir) {
    if (mode == 0) {
        dir = make_float2(0.f, 0.f);
        return un;
    }
    float dx = -gn.x, dy = -gn.y;
    if (mode == 1) {
        dx = __fadd_rn(dx, __fmul_rn(beta, dn.x));
        dy = __fadd_rn(dy, __fmul_rn(beta, dn.y));
    }
    dir = make_float2(dx, dy);
    return make_float2(__fadd_rn(un.x, __fmul_rn(alpha, dx)), __fadd_rn(un.y, __fmul_rn(alpha, dy)));
}

// The candidate rule of a frame for the current round, read from its state
// with L2 loads (not volatile) so that the reads are in flight together.
struct FInfo {
    float alpha, beta;
    int mode, iu, igc, idp, igt;
};
__device__ __forceinline__ FInfo frame_info(const FrameState *S) {
    FInfo fi;
    fi.iu = __ldcg(&S->iu);
    fi.igc = __ldcg(&S->igc);
    fi.idp = __ldcg(&S->idp);
    fi.igt = __ldcg(&S->igt);
    const int st = __ldcg(&S->state), k = __ldcg(&S->k), rs = __ldcg(&S->restart);
    fi.alpha = __ldcg(&S->alpha);
    fi.beta = __ldcg(&S->beta);
    fi.mode = (st == ST_EVAL) ? 0 : ((rs || k == 0) ? 2 : 1);
    return fi;
}

struct Cand {
    const float2 *u, *g, *d;
    float alpha, beta;
    int mode;
    __device__ __forceinline__ float2 at(int n, float2 &dir) const {
        const float2 un = __ldcg(u + n);
        const float2 gn = mode != 0 ? __ldcg(g + n) : make_float2(0.f, 0.f);
        const float2 dn = mode == 1 ? __ldcg(d + n) : make_float2(0.f, 0.f);
        return cand_value(un, gn, dn, alpha, beta, mode, dir);
    }
};

__device__ __forceinline__ Cand make_cand(const d2ic_frame_t &F, const FInfo &fi) {
    Cand c;
    c.u = nbuf(F, fi.iu);
    c.g = nbuf(F, 2 + fi.igc);
    c.d = nbuf(F, 5 + fi.idp);
    c.alpha = fi.alpha;
    c.beta = fi.beta;
    c.mode = fi.mode;
    return c;
}

__device__ __forceinline__ Cand make_cand(const d2ic_frame_t &F, const FrameState *S) {
    return make_cand(F, frame_info(S));
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

// the same search over a copy of the prefix sums in shared memory
__device__ __forceinline__ int find_slot_smem(const int *pre, int n, int x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Self-check of an index taken from the active list or its prefix sums: in [0, n) it is returned;
// otherwise the launch aborts with D2IC_INTERNAL and 0 is returned, so that the access it guards
// stays inside its table.
__device__ __forceinline__ int checked_index(int v, int n, CtlHeader *H) {
    if ((unsigned)v < (unsigned)n) return v;
    H->err = D2IC_INTERNAL;
    atomicExch(&H->abort, 1);
    return 0;
}

// ---------------------------------------------------------------------------
// P phase: one chunk per warp, software-pipelined
// ---------------------------------------------------------------------------
// Each warp walks its chunks (a contiguous range for one frame, c, c + W,
// c + 2W, ... for W warps in the grid with several) with three stages in flight:
//   chunk i + 2: metadata (pixel range, nodes, slots) loaded into registers;
//   chunk i + 1: pixel records copied into the warp's shared-memory buffer by
//                one TMA bulk copy (cp.async.bulk, completion on an mbarrier),
//                nodal candidate inputs (u, g, d) copied by cp.async onto the
//                same mbarrier;
//   chunk i:     sampled and reduced.
// A warp therefore never waits on a metadata -> records / candidates round
// trip.
// Each chunk also stages its window of the deformed image's coefficients
// (tile_w x tile_h floats) with a 2-D TMA copy on the same mbarrier.  The
// window is placed from the chunk's candidate of the previous pass, with a
// margin of TILE_MARGIN pixels on every side (stored per chunk in
// chunk_tile); a pixel whose 4x4 stencil is not inside it (a larger move, the
// first pass) reads global memory with the same arithmetic.
constexpr int CHUNK_BYTES = D2IC_CHUNK_MAX * 16;            // one staged record buffer
constexpr int TILE_BYTES = D2IC_TILE_MAX_FLOATS * 4;        // one staged coefficient tile
static_assert(TILE_BYTES % 128 == 0, "tile buffers keep 128-byte alignment");
constexpr int WARP_SMEM = 2 * CHUNK_BYTES + 2 * TILE_BYTES;
constexpr int TILE_MARGIN = 2;
constexpr int TILE_NONE = (int)0x80008000u;                 // no valid origin (col = row = -32768)
constexpr unsigned long long TMA_WAIT_NS = 200ull * 1000ull * 1000ull;
constexpr int FCACHE = 64;
constexpr int CAND_N = 12;    // candidate copies per staged chunk (lanes 0..11)    // active frames whose per-round lookup data is kept in shared memory

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long *b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
// 1-D TMA: global -> this CTA's shared memory, completion counted on mbarrier b
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(b))
                 : "memory");
}
// 2-D TMA: the tensor map's box at tensor coordinates (x, y) -> shared memory
__device__ __forceinline__ void tensor_load_2d(void *dst, const void *map, int x, int y, unsigned long long *b) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_addr(b))
        : "memory");
}
// 8-byte asynchronous copy global -> shared (no register holds the value); the mbarrier's
// pending count is decremented when this thread's earlier cp.async copies have completed
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_arrive(unsigned long long *b) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// false if the phase did not complete within TMA_WAIT_NS
__device__ __forceinline__ bool mbar_wait(unsigned long long *b, unsigned parity) {
    if (mbar_test(b, parity)) return true;
    const unsigned long long t0 = gtimer();
    while (!mbar_test(b, parity))
        if (gtimer() - t0 > TMA_WAIT_NS) return false;
    return true;
}

// One chunk's metadata as the pipeline carries it.  nd / slot hold local node
// (lane) a's index and slot rank in lanes 0..3.
struct ChunkMeta {
    int s, f, c, pb, pe, nd, slot;   // active slot, frame, chunk within the frame, ...
    int box0, box1, tile;            // packed pixel-box corners and tile origin (col | row << 16)
};

__device__ __forceinline__ ChunkMeta load_meta(const d2ic_frame_t *frames, int f, int c, int lane) {
    const d2ic_frame_t &F = frames[f];
    ChunkMeta m;
    m.s = 0;
    m.f = f;
    m.c = c;
    m.pb = __ldg(F.chunk_begin + c);
    m.pe = __ldg(F.chunk_begin + c + 1);
    m.box0 = __ldg(F.chunk_box + 2 * c);
    m.box1 = __ldg(F.chunk_box + 2 * c + 1);
    m.tile = F.tile_w > 0 ? __ldcg(F.chunk_tile + c) : TILE_NONE;   // rewritten every pass: L2
    m.nd = 0;
    m.slot = 0;
    if (lane < 4) {
        m.nd = __ldg(F.chunk_nodes + 4 * c + lane);
        m.slot = (int)(((unsigned)__ldg(F.chunk_slot + c) >> (8 * lane)) & 0xffu);
    }
    return m;
}

// Where a chunk's records and coefficient tile come from in this pass.
struct Stage {
    bool staged, tiled;   // records in shared memory; coefficient tile in shared memory
    int tx0, ty0;         // tile origin (pixel column / row of tile element (0, 0))
};

// Tile origin for the next pass from this pass's nodal candidates: the
// smallest tap column / row any pixel of the chunk can reach, less the margin.
__device__ __forceinline__ int tile_origin(int box0, const float ux[4], const float uy[4]) {
    const float mnx = fminf(fminf(ux[0], ux[1]), fminf(ux[2], ux[3]));
    const float mny = fminf(fminf(uy[0], uy[1]), fminf(uy[2], uy[3]));
    const int ox = (box0 & 0xffff) + (int)safe_floor(mnx) - 1 - TILE_MARGIN;
    const int oy = (int)((unsigned)box0 >> 16) + (int)safe_floor(mny) - 1 - TILE_MARGIN;
    if (ox <= -32768 || ox >= 32768 || oy <= -32768 || oy >= 32768) return TILE_NONE;   // also NaN candidates
    return (ox & 0xffff) | (int)((unsigned)oy << 16);
}

__device__ __forceinline__ int atom_acq_rel_add(int *p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

template <int KIND>
__device__ __forceinline__ void chunk_compute(const d2ic_frame_t &F, const ChunkMeta &m, float2 uc, const Stage &st,
                                              const uint4 *srec, const float *tile, int lane) {
    const bool staged = st.staged;
    const bool tiled = KIND == D2IC_INTERP_CUBIC && st.tiled;
    const int tw = F.tile_w, th = F.tile_h, tx0 = st.tx0, ty0 = st.ty0;
    const int n = max(m.pe - m.pb, 0);
    const uint4 *gpix = reinterpret_cast<const uint4 *>(F.pix) + m.pb;
    float ux[4], uy[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        ux[a] = __shfl_sync(0xffffffffu, uc.x, a);
        uy[a] = __shfl_sync(0xffffffffu, uc.y, a);
    }
    const Img im{F.coeff, F.W, F.H, F.cpitch, F.pad};
    // Whole chunk inside the tile: a pixel's displacement is a convex combination of its
    // element's nodal candidates, so its stencil corner lies in the chunk's pixel box shifted by
    // [floor(min u), floor(max u)] (taken with 0.5 px of slack).  Then no pixel needs the
    // per-pixel test or the global-memory path.
    bool fast = false;
    if (tiled && staged && n <= D2IC_CHUNK_MAX) {
        bool fin = true;
#pragma unroll
        for (int a = 0; a < 4; ++a) fin = fin && isfinite(ux[a]) && isfinite(uy[a]);
        if (fin) {
            const float mnx = fminf(fminf(ux[0], ux[1]), fminf(ux[2], ux[3]));
            const float mxx = fmaxf(fmaxf(ux[0], ux[1]), fmaxf(ux[2], ux[3]));
            const float mny = fminf(fminf(uy[0], uy[1]), fminf(uy[2], uy[3]));
            const float mxy = fmaxf(fmaxf(uy[0], uy[1]), fmaxf(uy[2], uy[3]));
            const int lx0 = (m.box0 & 0xffff) + (int)safe_floor(mnx - 0.5f) - 1 - tx0;
            const int lx1 = (m.box1 & 0xffff) + (int)safe_floor(mxx + 0.5f) - 1 - tx0;
            const int ly0 = (int)((unsigned)m.box0 >> 16) + (int)safe_floor(mny - 0.5f) - 1 - ty0;
            const int ly1 = (int)((unsigned)m.box1 >> 16) + (int)safe_floor(mxy + 0.5f) - 1 - ty0;
            fast = lx0 >= 0 && lx1 <= tw - 4 && ly0 >= 0 && ly1 <= th - 4;
        }
    }
    float jr = 0.f;
    float gxa[4] = {0.f, 0.f, 0.f, 0.f}, gya[4] = {0.f, 0.f, 0.f, 0.f};
    // fast path: the stencil corner is clamped into the tile only as a guard of the shared-memory
    // bounds (it is already inside)
    auto one_fast = [&](const uint4 r4) {
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
        float gx, gy;
        const int lx = min(max(ix - 1 - tx0, 0), tw - 4), ly = min(max(iy - 1 - ty0, 0), th - 4);
        const float v = sample_cubic_tile(tile, tw, lx, ly, tx, ty, gx, gy);
        const float r = v - I1;
        jr += r * r;
        const float rgx = r * gx, rgy = r * gy;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            gxa[a] += rgx * N[a];
            gya[a] += rgy * N[a];
        }
    };
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
        const int lx = ix - 1 - tx0, ly = iy - 1 - ty0;   // stencil corner inside the tile
        if (tiled && (unsigned)lx <= (unsigned)(tw - 4) && (unsigned)ly <= (unsigned)(th - 4))
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
    if (fast) {
#pragma unroll 4
        for (int i = 0; i < D2IC_CHUNK_MAX / 32; ++i) {
            const int p = lane + 32 * i;
            if (p < n) one_fast(srec[p]);
        }
    } else if (staged) {
#pragma unroll 4
        for (int i = 0; i < D2IC_CHUNK_MAX / 32; ++i) {
            const int p = lane + 32 * i;
            if (p < n) one(srec[p]);
        }
        for (int p = lane + D2IC_CHUNK_MAX; p < n; p += 32) one(__ldg(gpix + p));   // beyond the staged buffer
    } else {
        for (int p = lane; p < n; p += 32) one(__ldg(gpix + p));
    }
    const DF js = df_warp_sum(DF{jr, 0.f});
    // The 8 nodal partials summed over the warp by a reduce-scatter butterfly: at each of the
    // steps over lane bits 4, 3, 2 a lane keeps half of its values and adds its partner's copy of
    // that half (7 shuffles instead of 40); bits 1, 0 finish the sums.  Value k = (gx_0..3,
    // gy_0..3)[k] ends in lane 16 (k >> 2) + 8 ((k >> 1) & 1) + 4 (k & 1).
    float v4[4];
    {
        const bool b = (lane >> 4) & 1;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float give = b ? gxa[q] : gya[q];
            const float keep = b ? gya[q] : gxa[q];
            v4[q] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
        }
    }
    float v2[2];
    {
        const bool b = (lane >> 3) & 1;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const float give = b ? v4[q] : v4[q + 2];
            const float keep = b ? v4[q + 2] : v4[q];
            v2[q] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
        }
    }
    float v1;
    {
        const bool b = (lane >> 2) & 1;
        const float give = b ? v2[0] : v2[1];
        const float keep = b ? v2[1] : v2[0];
        v1 = keep + __shfl_xor_sync(0xffffffffu, give, 4);
    }
    v1 += __shfl_xor_sync(0xffffffffu, v1, 2);
    v1 += __shfl_xor_sync(0xffffffffu, v1, 1);
    // lane a < 4 takes gx_a (k = a) and gy_a (k = 4 + a)
    const int la = lane & 3;
    const float gxs = __shfl_sync(0xffffffffu, v1, 8 * ((la >> 1) & 1) + 4 * (la & 1));
    const float gys = __shfl_sync(0xffffffffu, v1, 16 + 8 * ((la >> 1) & 1) + 4 * (la & 1));
    if (lane == 0 && tw > 0) F.chunk_tile[m.c] = tile_origin(m.box0, ux, uy);
    // lane a stores node a's partial in the chunk's slot of that node; node 0's slot also
    // carries the chunk's sum of r^2 (double-float), so every chunk is counted exactly once
    if (lane < 4)
        reinterpret_cast<float4 *>(F.node_grad)[(size_t)m.slot * F.n_nodes + m.nd] =
            make_float4(gxs, gys, lane == 0 ? js.hi : 0.f, lane == 0 ? js.lo : 0.f);
    __syncwarp();                                   // every lane is done with the staged buffers
}

// One count per distinct node group among a chunk's four nodes; the group's reducer waits
// until it has as many counts as chunks touch the group.  Each quad of lanes (4 j .. 4 j + 3)
// holds the node groups of one chunk (grp < 0: no chunk).
__device__ __forceinline__ void count_chunk_groups_quad(int *group_cnt, int grp, int lane) {
    const int q0 = lane & ~3, a = lane & 3;
    const int g0 = __shfl_sync(0xffffffffu, grp, q0), g1 = __shfl_sync(0xffffffffu, grp, q0 + 1),
              g2 = __shfl_sync(0xffffffffu, grp, q0 + 2);
    const bool first = a == 0 || (a == 1 && grp != g0) || (a == 2 && grp != g0 && grp != g1) ||
                       (a == 3 && grp != g0 && grp != g1 && grp != g2);
    if (grp >= 0 && first) atomicAdd(group_cnt + grp, 1);
}

// ---------------------------------------------------------------------------
// N work: one group of GN = 32 nodes per warp (lane = node)
// ---------------------------------------------------------------------------
// Per node, in two parts.  node_pre needs nothing from this round's pixel pass (the
// candidate point, the trial direction, the current gradient and the spring terms), so a
// warp runs it before it waits for its group's chunks; node_post gathers the chunk
// partials from the node's K slots (slot order), writes the trial gradient, point and
// direction, and returns the node's terms of sum r^2, spring energy, g.g, g.(g - g_cur)
// and g_cur.dir in double-float.
struct NodePre {
    float2 ui, dir, gc;
    float rx, ry, en;
};

__device__ __forceinline__ NodePre node_pre(const d2ic_frame_t &F, const FInfo &fi, int n) {
    NodePre p;
    p.rx = p.ry = p.en = 0.f;
    p.ui = p.dir = p.gc = make_float2(0.f, 0.f);
    if (n >= F.n_nodes) return p;
    const Cand cd = make_cand(F, fi);
    // All loads of a batch are issued before any is consumed: a short chain of L2 round
    // trips instead of one per table entry.  Sums still run in table order.
    p.gc = __ldcg(nbuf(F, 2 + fi.igc) + n);
    p.ui = cd.at(n, p.dir);
    const int md = F.max_deg, Nn = F.n_nodes;
    const int *nbi = F.nbr_index + n;             // column-major: entry k at k * n_nodes
    const float *nbw = F.nbr_weight + n;
    bool alive = true;                               // entries after the first -1 are padding
    constexpr int NBN = 8;
    for (int kb = 0; kb < md && alive; kb += NBN) {
        int jj[NBN];
        float ww[NBN];
#pragma unroll
        for (int t = 0; t < NBN; ++t) {
            jj[t] = (kb + t < md) ? __ldg(nbi + (size_t)(kb + t) * Nn) : -1;
            ww[t] = (kb + t < md) ? __ldg(nbw + (size_t)(kb + t) * Nn) : 0.f;
        }
        float2 uj[NBN];
#pragma unroll
        for (int t = 0; t < NBN; ++t) {
            float2 dj;
            uj[t] = (jj[t] >= 0) ? cd.at(jj[t], dj) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int t = 0; t < NBN; ++t) {
            alive = alive && jj[t] >= 0;
            if (alive) {
                const float ddx = p.ui.x - uj[t].x, ddy = p.ui.y - uj[t].y;
                p.rx += ww[t] * ddx;
                p.ry += ww[t] * ddy;
                p.en += ww[t] * (ddx * ddx + ddy * ddy);
            }
        }
    }
    return p;
}

__device__ __forceinline__ void node_post(const d2ic_frame_t &F, const FInfo &fi, int n, const NodePre &p, DF q[5]) {
#pragma unroll
    for (int i = 0; i < 5; ++i) q[i] = DF{0.f, 0.f};
    if (n >= F.n_nodes) return;
    float sx = 0.f, sy = 0.f;
    DF sj = {0.f, 0.f};
    const int K = F.node_chunk_k, Nn = F.n_nodes;
    const float4 *ng = reinterpret_cast<const float4 *>(F.node_grad) + n;
    constexpr int NB = 8;
    for (int kb = 0; kb < K; kb += NB) {
        float4 v[NB];
#pragma unroll
        for (int t = 0; t < NB; ++t) v[t] = (kb + t < K) ? __ldcg(ng + (size_t)(kb + t) * Nn) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int t = 0; t < NB; ++t)
            if (kb + t < K) {
                sx += v[t].x;
                sy += v[t].y;
                sj = df_add(sj, DF{v[t].z, v[t].w});
            }
    }
    const float inv_np = 1.0f / (float)max(F.n_pix, 1);
    const float gx = sx * inv_np + F.alpha_reg * p.rx;
    const float gy = sy * inv_np + F.alpha_reg * p.ry;
    nbuf(F, 2 + fi.igt)[n] = make_float2(gx, gy);
    nbuf(F, 1 - fi.iu)[n] = p.ui;
    nbuf(F, 5 + (1 - fi.idp))[n] = p.dir;
    // per-node terms of the inner products, exact in double-float (g - g_cur rounded
    // in FP32 as the reference's elementwise difference)
    q[P_JSUM] = sj;
    q[P_EREG] = DF{0.25f * p.en, 0.f};
    q[P_GG] = df_add(df_prod(gx, gx), df_prod(gy, gy));
    q[P_GDIFF] = df_add(df_prod(gx, gx - p.gc.x), df_prod(gy, gy - p.gc.y));
    q[P_GD] = df_add(df_prod(p.gc.x, p.dir.x), df_prod(p.gc.y, p.dir.y));
}

// ---------------------------------------------------------------------------
// R step (last block at the end-of-round barrier)
// ---------------------------------------------------------------------------
// The descriptor scalars the control step reads, loaded once at its start.
struct FConst {
    float *hist;
    double tol;
    float alpha_reg;
    int max_iter, n_pix;
};

// Values of a control step that need FP64 division or square root, computed for the whole
// warp at once (GB300's FP64 pipe is narrow, so each FP64 instruction is costly): the
// objective J of this round's point, and, for the state after accepting this point, sqrt(g.g)
// and the PR+ ratio g.(g - g_prev) / (g_prev.g_prev + 1e-16).
struct StepVals {
    double J, gnorm, ratio;
};

__device__ void hist_row(const FConst &F, int k, double a, double b, double c) {
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

// Called right after accept_point of this round's point, so v.gnorm = sqrt(S.gg_cur) and
// v.ratio = S.gdiff_cur / (S.gg_prev + 1e-16).
__device__ void start_iter(FrameState &S, const FConst &F, const StepVals &v) {
    S.gnorm = v.gnorm;
    if (S.gnorm < F.tol) {                       // stop branch: k unchanged
        hist_row(F, S.k, S.J_cur, S.gnorm, 0.0);
        S.state = ST_DONE;
        return;
    }
    double beta = 0.0;
    if (S.k > 0) {
        const double x = v.ratio;
        beta = (x != x) ? x : fmax(x, 0.0);      // jnp.maximum keeps NaN
    }
    S.beta = (float)beta;
    S.alpha = 1.0f;
    S.t = 0;
    S.restart = 0;
    S.gd_known = 0;
    S.state = ST_TRIAL;
}

__device__ void frame_decide(FrameState &S, const FConst &F, const double *q, const StepVals &v, int eval_only) {
    const double J = v.J;
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
            start_iter(S, F, v);
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
                else start_iter(S, F, v);
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
            else start_iter(S, F, v);
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

// A frame takes part in this launch's rounds: not finished and not held (CMD_HOLD keeps an admitted
// frame's state but leaves it out of the launch).  The command words are constant once r_init ran.
__device__ __forceinline__ bool in_launch(Ctl &C, int f) {
    return ld_vol(&C.fs[f].state) != ST_DONE && ld_vol(C.cmd + f) != CMD_HOLD;
}

// rebuild the active list and prefix sums (whole block)
__device__ void rebuild_active(const d2ic_frame_t *frames, int n_frames, Ctl &C) {
    const int per = (n_frames + NT - 1) / NT;
    const int f0 = threadIdx.x * per, f1 = min(f0 + per, n_frames);
    int cnt = 0, ch = 0, gr = 0;
    for (int f = f0; f < f1; ++f)
        if (in_launch(C, f)) {
            ++cnt;
            ch += frames[f].n_chunks;
            gr += pad_groups(frames[f].n_groups);
        }
    int ta, tb, tc;
    block_scan3(cnt, ch, gr, ta, tb, tc);
    const int lb = ld_vol(&C.h->list_buf);         // start of a launch: nothing reads the list yet
    if (threadIdx.x == 0) {
        C.h->n_active = ta;
        C.h->total_chunks = tb;
        C.h->total_groups = tc;
        C.cp(lb)[ta] = tb;
        C.gp(lb)[ta] = tc;
    }
    int slot = cnt, cp = ch, gp = gr;
    for (int f = f0; f < f1; ++f)
        if (in_launch(C, f)) {
            C.act(lb)[slot] = f;
            C.cp(lb)[slot] = cp;
            C.gp(lb)[slot] = gp;
            ++slot;
            cp += frames[f].n_chunks;
            gp += pad_groups(frames[f].n_groups);
        }
    __syncthreads();
}

// Start of a launch: new frames (CMD_INIT) get a fresh CG state, idle slots are
// parked as finished-and-reported, running and held frames keep their state (held
// ones stay out of the active list); frames that finished in an earlier launch are
// marked reported (their outputs were written at the end of that launch).
__device__ void r_init(const d2ic_frame_t *frames, int n_frames, Ctl &C) {
    for (int f = threadIdx.x; f < n_frames; f += NT) {
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

// Wait (bounded) until blocks_past reaches target; on a timeout the launch aborts and the list
// is left as it is.
__device__ __forceinline__ int wait_blocks_past(CtlHeader *H, unsigned target) {
    if (ld_acquire_u32(&H->blocks_past) >= target) return 1;
    const unsigned long long t0 = gtimer();
    while (ld_acquire_u32(&H->blocks_past) < target) {
        if (ld_vol(&H->abort)) return 0;
        if (gtimer() - t0 > WAIT_NS) {
            H->err = D2IC_WAIT_TIMEOUT;
            atomicExch(&H->abort, 1);
            return 0;
        }
        __nanosleep(32);
    }
    return 1;
}

// The CG control of one frame, run by the warp that reduced the frame's last
// node group: the group partials are summed in group order (double-float,
// then FP64) and the frame state advanced.  Nothing else reads the frame's
// state in this round once all its groups are reduced.
// Active list rebuilt by one warp (the warp that ends a round): lane l scans a contiguous
// block of frames, a warp scan gives each block its slot and prefix offsets.
__device__ void rebuild_active_warp(const d2ic_frame_t *frames, int n_frames, Ctl &C, int lane) {
    const int per = (n_frames + 31) / 32;
    const int f0 = min(lane * per, n_frames), f1 = min(f0 + per, n_frames);
    int cnt = 0, ch = 0, gr = 0;
    for (int f = f0; f < f1; ++f)
        if (in_launch(C, f)) {
            ++cnt;
            ch += frames[f].n_chunks;
            gr += pad_groups(frames[f].n_groups);
        }
    int ic = cnt, ih = ch, ig = gr;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(0xffffffffu, ic, o), b = __shfl_up_sync(0xffffffffu, ih, o),
                  c = __shfl_up_sync(0xffffffffu, ig, o);
        if (lane >= o) {
            ic += a;
            ih += b;
            ig += c;
        }
    }
    const int ta = __shfl_sync(0xffffffffu, ic, 31), tb = __shfl_sync(0xffffffffu, ih, 31),
              tc = __shfl_sync(0xffffffffu, ig, 31);
    // the copy no block reads (see Ctl); read once, before lane 0 flips it below
    const int nb = 1 - __shfl_sync(0xffffffffu, lane == 0 ? ld_vol(&C.h->list_buf) : 0, 0);
    int slot = ic - cnt, cp = ih - ch, gp = ig - gr;
    for (int f = f0; f < f1; ++f)
        if (in_launch(C, f)) {
            C.act(nb)[slot] = f;
            C.cp(nb)[slot] = cp;
            C.gp(nb)[slot] = gp;
            ++slot;
            cp += frames[f].n_chunks;
            gp += pad_groups(frames[f].n_groups);
        }
    if (lane == 0) {
        C.h->n_active = ta;
        C.h->total_chunks = tb;
        C.h->total_groups = tc;
        C.cp(nb)[ta] = tb;
        C.gp(nb)[ta] = tc;
        C.h->list_buf = nb;                          // published by the round's release
    }
    __syncwarp();
}

__device__ void frame_r(const d2ic_frame_t &F, int f, Ctl &C, int eval_only, int lane) {
    DF q[5] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    FrameState S;
    if (lane == 0) S = load_fs(C.fs + f);              // in flight with the partials below
    FConst fc;
    fc.hist = F.hist;
    fc.tol = F.tol;
    fc.alpha_reg = F.alpha_reg;
    fc.max_iter = F.max_iter;
    fc.n_pix = F.n_pix;
    const int nsg = (F.n_groups + SG - 1) / SG;
    const float2 *sp = reinterpret_cast<const float2 *>(F.group_part) + (size_t)F.n_groups * D2IC_NPART;
    for (int g = lane; g < nsg; g += 32) {
        float2 v[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) v[i] = __ldcg(sp + (size_t)g * D2IC_NPART + i);
#pragma unroll
        for (int i = 0; i < 5; ++i) q[i] = df_add(q[i], DF{v[i].x, v[i].y});
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) q[i] = df_warp_sum(q[i]);
    // lane i < 5 converts sum i to FP64: one conversion for all five
    DF sel = q[0];
#pragma unroll
    for (int i = 1; i < 5; ++i)
        if (lane == i) sel = q[i];
    const double mine = df_to_double(sel);
    double qd[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) qd[i] = __shfl_sync(0xffffffffu, mine, i);
    // one division for two quotients: lane 0 the image term of J, lane 1 the PR+ ratio
    const double gg_old = __shfl_sync(0xffffffffu, lane == 0 ? S.gg_cur : 0.0, 0);
    const double num = lane == 0 ? 0.5 * qd[P_JSUM] : qd[P_GDIFF];
    const double den = lane == 0 ? (double)max(fc.n_pix, 1) : gg_old + 1e-16;
    const double quo = num / den;
    StepVals v;
    v.ratio = __shfl_sync(0xffffffffu, quo, 1);
    v.gnorm = sqrt(qd[P_GG]);
    if (lane == 0) {
        v.J = quo + (double)fc.alpha_reg * qd[P_EREG];
        frame_decide(S, fc, qd, v, eval_only);
        C.fs[f] = S;
        if (S.state == ST_DONE) atomicExch(&C.h->finished, 1);
    }
}

// The active list (n_active = na <= FCACHE) with its prefix sums and each frame's candidate
// rule, copied into the block's shared memory (whole block).
__device__ void load_list(Ctl &C, int lb, int na, int *s_cpre, int *s_gpre, int *s_act, FInfo *s_fi) {
    if (na > FCACHE) return;
    for (int s = threadIdx.x; s <= na; s += NT) {
        s_cpre[s] = __ldcg(C.cp(lb) + s);
        s_gpre[s] = __ldcg(C.gp(lb) + s);
    }
    for (int s = threadIdx.x; s < na; s += NT) {
        const int f = checked_index(__ldcg(C.act(lb) + s), C.n, C.h);
        s_act[s] = f;
        s_fi[s] = frame_info(C.fs + f);
    }
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------
// ONE: a launch of exactly one frame; the pixel pass then reads that frame's descriptor at a
// fixed address, so its fields are loop invariants (loaded once, not per chunk; measured 2-5%
// faster per round).
template <int KIND, bool ONE = false>
__global__ void __launch_bounds__(NT, D2IC_ENGINE_MINB) cg_engine(const d2ic_frame_t *__restrict__ frames, int n_frames,
                                                   char *ctl_base, int eval_only, const float *u_eval,
                                                   double *J_out, float *grad_out, unsigned long long *trace,
                                                   int trace_rounds, int max_rounds, int stop_flags) {
    __shared__ unsigned long long s_bar[NWARP][2];   // per-warp mbarriers of the two record buffers
    // per warp and buffer: the nodal candidate inputs of the staged chunk, u of node a at [a], g at
    // [4 + a], the previous direction at [8 + a] (cp.async, completing on the buffer's mbarrier)
    __shared__ __align__(16) float2 s_cand[NWARP][2][CAND_N];
    __shared__ int s_cpre[FCACHE + 1];               // per-round copies of the active list (na <= FCACHE)
    __shared__ int s_gpre[FCACHE + 1];
    __shared__ int s_act[FCACHE];
    __shared__ FInfo s_fi[FCACHE];
    __shared__ int s_hdr[6];                         // n_active, total_chunks, total_groups, abort, slice_stop,
                                                     // list_buf
    __shared__ DF s_gq[NWARP][D2IC_NPART];           // group partials of this block's supergroup
    __shared__ int s_sgcnt;                          // groups of this block's supergroup reduced this round
    // per warp: two record buffers, then two coefficient-tile buffers (all 128-byte aligned)
    extern __shared__ __align__(128) unsigned char s_dyn[];
    Ctl C = make_ctl(ctl_base, n_frames);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char *wbuf = s_dyn + (size_t)wid * WARP_SMEM;
    unsigned pipe_i = 0;   // chunks this warp has staged: buffer i & 1, completion parity (i >> 1) & 1
    if (lane == 0) {
        mbar_init(&s_bar[wid][0], 1 + CAND_N);   // lane 0's expect_tx + one per candidate copy
        mbar_init(&s_bar[wid][1], 1 + CAND_N);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // descriptors (and their tensor maps) may have been rewritten since the previous launch
    for (int f = threadIdx.x; f < n_frames; f += NT)
        if (frames[f].tile_w > 0)
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(frames[f].coeff_map) : "memory");
    const bool tiles_ok = (smem_addr(s_dyn) & 127) == 0;   // tile buffers need 128-byte alignment
    __syncthreads();
    // optional phase trace per round: warp 0 of block 0 stamps [0] round start, [1] end of its pixel
    // work, [2] end of its group work, [5] after the barrier; the warp that runs a frame's control
    // stamps [3] and [4] around it
    const bool tr = trace != nullptr && blockIdx.x == 0 && threadIdx.x == 0;
    int round = 0;
    if (threadIdx.x == 0) s_sgcnt = 0;
    // A warp's first chunk of the next round, staged before the round's release (its records,
    // coefficient tile and the metadata of the chunk after it do not depend on the control step);
    // used if the active list is unchanged, else drained.
    bool pf = false;
    int pf_na = 0, pf_total = 0;
    ChunkMeta pf_m0{}, pf_m1{};
    Stage pf_st0{};

    // ---- init of newly admitted frames: u <- u0, zero g/d buffers and gradient slots, NaN history ----
    for (int f = 0; f < n_frames; ++f) {
        if (ld_vol(C.cmd + f) != CMD_INIT) continue;
        const d2ic_frame_t &F = frames[f];
        const int nn = F.n_nodes;
        const float2 *u0 = reinterpret_cast<const float2 *>((eval_only && u_eval && f == 0) ? u_eval : F.u0);
        for (int i = blockIdx.x * NT + threadIdx.x; i < nn; i += gridDim.x * NT) {
            nbuf(F, 0)[i] = u0 ? u0[i] : make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 1; j < 7; ++j) nbuf(F, j)[i] = make_float2(0.f, 0.f);
        }
        // gradient slots that no chunk owns must read as 0; group counters start at 0
        float4 *ng = reinterpret_cast<float4 *>(F.node_grad);
        for (size_t i = blockIdx.x * NT + threadIdx.x; i < (size_t)F.node_chunk_k * nn; i += (size_t)gridDim.x * NT)
            ng[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        const int n_cnt = F.n_groups + (F.n_groups + SG - 1) / SG + 1;
        for (int i = blockIdx.x * NT + threadIdx.x; i < n_cnt; i += gridDim.x * NT) F.group_cnt[i] = 0;
        if (F.hist)
            for (int i = blockIdx.x * NT + threadIdx.x; i < 3 * F.max_iter; i += gridDim.x * NT)
                F.hist[i] = __int_as_float(0x7fc00000);
        // first-pass tile origins from u0 (the first pass evaluates u0 itself)
        if (F.tile_w > 0)
            for (int c = blockIdx.x * NT + threadIdx.x; c < F.n_chunks; c += gridDim.x * NT) {
                float ux[4], uy[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const int nd = __ldg(F.chunk_nodes + 4 * c + a);
                    const float2 v = u0 ? u0[nd] : make_float2(0.f, 0.f);
                    ux[a] = v.x;
                    uy[a] = v.y;
                }
                F.chunk_tile[c] = tile_origin(__ldg(F.chunk_box + 2 * c), ux, uy);
            }
    }
    if (!grid_barrier(C.h, [&] { r_init(frames, n_frames, C); })) goto finish;
    // The block's copy of the round state: the header, and for up to FCACHE active frames the
    // active list with its prefix sums and each frame's candidate rule.
    if (threadIdx.x == 0) {
        s_hdr[0] = ld_vol(&C.h->n_active);
        s_hdr[1] = ld_vol(&C.h->total_chunks);
        s_hdr[2] = ld_vol(&C.h->total_groups);
        s_hdr[3] = ld_vol(&C.h->abort);
        s_hdr[4] = 0;
        s_hdr[5] = ld_vol(&C.h->list_buf);
    }
    __syncthreads();
    load_list(C, s_hdr[5], s_hdr[0], s_cpre, s_gpre, s_act, s_fi);
    __syncthreads();

    while (round < max_rounds) {                    // a slice: at most max_rounds rounds, state kept in HBM
        const int na = s_hdr[0];
        const int total = s_hdr[1];
        const int tg = s_hdr[2];
        const int lb = s_hdr[5];
        if (na == 0 || s_hdr[3] || s_hdr[4]) break;
        const bool trr = tr && round < trace_rounds;
        if (trr) trace[7 * round + 0] = gtimer();
        // the active list only shrinks within a launch: the same count means the same list
        const bool pf_use = pf && na == pf_na && total == pf_total;
        if (pf && !pf_use) {
            if (lane < CAND_N) mbar_arrive(&s_bar[wid][pipe_i & 1]);   // no candidates for the dropped chunk
            if (!mbar_wait(&s_bar[wid][pipe_i & 1], (pipe_i >> 1) & 1u) && lane == 0) {   // bounded
                C.h->err = D2IC_WAIT_TIMEOUT;
                atomicExch(&C.h->abort, 1);
            }
            ++pipe_i;
        }
        pf = false;
        const ChunkMeta pm0 = pf_m0, pm1 = pf_m1;
        const Stage pst0 = pf_st0;
        pf_m0 = ChunkMeta{};   // constants while the round runs (nothing to keep in registers)
        pf_m1 = ChunkMeta{};
        pf_st0 = Stage{};
        // ---- P phase: chunks of the active list spread over the warps (see below) ----
        {
            const bool cached = na <= FCACHE;
            const int gw = (int)((blockIdx.x * NT + threadIdx.x) >> 5);
            const int nw = (int)((gridDim.x * NT) >> 5);
            int cur = 0;   // active slot of the last located chunk (chunks ascend per warp)
            auto fetch_meta = [&](int g) {
                int s, f, base;
                if (cached) {
                    while (cur + 1 < na && s_cpre[cur + 1] <= g) ++cur;
                    s = cur;
                    f = s_act[s];
                    base = s_cpre[s];
                } else {
                    s = find_slot(C.cp(lb), na, g);
                    f = checked_index(__ldcg(C.act(lb) + s), n_frames, C.h);
                    base = __ldcg(C.cp(lb) + s);
                }
                ChunkMeta m = load_meta(frames, f, checked_index(g - base, frames[f].n_chunks, C.h), lane);
                m.s = s;
                return m;
            };
            // stage a chunk: TMA bulk copy of its records, 2-D TMA copy of its coefficient tile
            auto issue_tma = [&](const ChunkMeta &m, unsigned i) {
                const d2ic_frame_t &F = frames[ONE ? 0 : m.f];
                const int n = max(m.pe - m.pb, 0);
                const unsigned bytes = (unsigned)min(n, D2IC_CHUNK_MAX) * 16u;
                const uint4 *src = reinterpret_cast<const uint4 *>(F.pix) + m.pb;
                Stage st;
                st.staged = bytes > 0 && ((reinterpret_cast<uintptr_t>(src) & 15) == 0);
                st.tiled = false;
                st.tx0 = 0;
                st.ty0 = 0;
                if (KIND == D2IC_INTERP_CUBIC && tiles_ok && F.tile_w > 0 && m.tile != TILE_NONE) {
                    st.tx0 = (int)(short)(m.tile & 0xffff) & ~3;   // TMA x: a multiple of 4 floats
                    st.ty0 = (int)(short)((unsigned)m.tile >> 16);
                    st.tiled = st.tx0 >= -F.pad && st.ty0 >= -F.pad && st.tx0 + F.tile_w <= F.W + F.pad &&
                               st.ty0 + F.tile_h <= F.H + F.pad;   // inside the halo'd array: no fill
                }
                unsigned long long *bar = &s_bar[wid][i & 1];
                if (lane == 0) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // after the buffers' generic reads
                    const unsigned tbytes = st.tiled ? (unsigned)(F.tile_w * F.tile_h) * 4u : 0u;
                    mbar_arrive_tx(bar, (st.staged ? bytes : 0u) + tbytes);
                    if (st.staged) bulk_load(wbuf + (i & 1) * CHUNK_BYTES, src, bytes, bar);
                    if (st.tiled)
                        tensor_load_2d(wbuf + 2 * CHUNK_BYTES + (i & 1) * TILE_BYTES, F.coeff_map, st.tx0 + F.pad,
                                       st.ty0 + F.pad, bar);
                }
                return st;
            };
            // the chunk's nodal candidate inputs into s_cand (lane 4 k + a copies array k of node a),
            // counted on the chunk's mbarrier
            auto load_cand = [&](const ChunkMeta &m, unsigned i) {
                const int a = lane & 3, k = lane >> 2;
                const int nd = __shfl_sync(0xffffffffu, m.nd, a);
                if (lane < CAND_N) {
                    const d2ic_frame_t &F = frames[ONE ? 0 : m.f];
                    const FInfo fi = cached ? s_fi[m.s] : frame_info(C.fs + m.f);
                    const int j = k == 0 ? fi.iu : (k == 1 ? 2 + fi.igc : 5 + fi.idp);
                    cp_async8(&s_cand[wid][i & 1][lane], nbuf(F, j) + nd);
                    cp_async_arrive(&s_bar[wid][i & 1]);
                }
            };
            ChunkMeta m0{}, m1{}, m2{};
            Stage st0{}, st1{};
            bool p_ok = true;
            // One frame: warp gw takes the contiguous chunk range [cb, ce) (neighbouring elements
            // share coefficient rows in cache; measured faster).  Several frames: chunk g goes to
            // warp g mod (warps), so that every step of the pass spans few frames (measured faster
            // for batches of small frames).
            // With fewer node groups than warps, group gi is reduced by warp gi (below); when the
            // spare chunks fit on the other warps, those warps take them, so that the group
            // reducers finish their own pixel work first and wait for none of it.
            const bool contiguous = na == 1;
            int cb = gw, ce = total;
            if (contiguous) {
                const int base = total / nw, extra = total - base * nw;
                if (tg < nw && extra <= nw - tg) {
                    const int k = max(gw - tg, 0);
                    cb = gw * base + min(k, extra);
                    ce = cb + base + (gw >= tg && k < extra ? 1 : 0);
                } else {
                    cb = (int)(((long long)gw * total) / nw);
                    ce = (int)(((long long)(gw + 1) * total) / nw);
                }
            }
            const int cs = contiguous ? 1 : nw;
            if (cb < ce) {
                if (pf_use) {
                    m0 = pm0;
                    st0 = pst0;
                    m1 = pm1;
                } else {
                    m0 = fetch_meta(cb);
                    st0 = issue_tma(m0, pipe_i);
                    if (cb + cs < ce) m1 = fetch_meta(cb + cs);
                }
                load_cand(m0, pipe_i);
            }
            for (int g = cb; g < ce; g += cs) {
                const bool has1 = g + cs < ce;
                if (g + 2 * cs < ce) m2 = fetch_meta(g + 2 * cs);
                if (has1) {
                    st1 = issue_tma(m1, pipe_i + 1);
                    load_cand(m1, pipe_i + 1);
                }
                const bool got = mbar_wait(&s_bar[wid][pipe_i & 1], (pipe_i >> 1) & 1u);
                if (!__all_sync(0xffffffffu, got)) {
                    if (lane == 0) {
                        C.h->err = D2IC_WAIT_TIMEOUT;
                        atomicExch(&C.h->abort, 1);
                    }
                    if (has1) mbar_wait(&s_bar[wid][(pipe_i + 1) & 1], ((pipe_i + 1) >> 1) & 1u);   // bounded
                    p_ok = false;
                    break;
                }
                float2 uc = make_float2(0.f, 0.f);
                if (lane < 4) {
                    const FInfo fi = cached ? s_fi[m0.s] : frame_info(C.fs + m0.f);
                    const float2 *sc = s_cand[wid][pipe_i & 1];
                    float2 dir;
                    uc = cand_value(sc[lane], sc[4 + lane], sc[8 + lane], fi.alpha, fi.beta, fi.mode, dir);
                }
                chunk_compute<KIND>(frames[ONE ? 0 : m0.f], m0, uc, st0,
                                    reinterpret_cast<const uint4 *>(wbuf + (pipe_i & 1) * CHUNK_BYTES),
                                    reinterpret_cast<const float *>(wbuf + 2 * CHUNK_BYTES + (pipe_i & 1) * TILE_BYTES),
                                    lane);
                ++pipe_i;
                m0 = m1;
                st0 = st1;
                m1 = m2;
            }
            // ---- count this warp's chunks into their node groups: one fence for the whole pass
            // (a fence per chunk would also wait for the pipeline's prefetch loads in flight) ----
            // Eight chunks per step: lane 4 j + a reads node a of chunk j, so the node loads of
            // the eight are in flight together.
            __threadfence();
            __syncwarp();
            if (p_ok) {
                for (int g0 = cb; g0 < ce; g0 += 8 * cs) {
                    const int g = g0 + (lane >> 2) * cs;
                    int grp = -1;
                    int *cnt = nullptr;
                    if (g < ce) {
                        int f, base;
                        if (cached) {
                            const int sl = na == 1 ? 0 : find_slot_smem(s_cpre, na, g);
                            f = s_act[sl];
                            base = s_cpre[sl];
                        } else {
                            const int sl = find_slot(C.cp(lb), na, g);
                            f = checked_index(__ldcg(C.act(lb) + sl), n_frames, C.h);
                            base = __ldcg(C.cp(lb) + sl);
                        }
                        const d2ic_frame_t &F = frames[f];
                        const int c = checked_index(g - base, F.n_chunks, C.h);
                        grp = __ldg(F.chunk_nodes + 4 * c + (lane & 3)) / GN;
                        cnt = F.group_cnt;
                    }
                    count_chunk_groups_quad(cnt, grp, lane);
                }
            }
            if (trr) trace[7 * round + 1] = gtimer();
            // ---- N work: group gi of the active list goes to global warp gi mod (warps in grid); the
            // warp waits until every chunk with a node in the group has written its slots.  With
            // at most one group per warp, a supergroup is the warps of one block and is reduced
            // in shared memory; otherwise through the frame's global partials. ----
            const bool blockred = tg <= nw;
            int gcur = 0;
            for (int gi = gw; gi < tg; gi += nw) {
                int s, f, base;
                if (cached) {
                    while (gcur + 1 < na && s_gpre[gcur + 1] <= gi) ++gcur;
                    s = gcur;
                    f = s_act[s];
                    base = s_gpre[s];
                } else {
                    s = find_slot(C.gp(lb), na, gi);
                    f = checked_index(__ldcg(C.act(lb) + s), n_frames, C.h);
                    base = __ldcg(C.gp(lb) + s);
                }
                const d2ic_frame_t &F = frames[f];
                const int g = gi - base;
                if (g >= F.n_groups) continue;         // padding of the frame's group range
                if (g < 0) {                           // self-check: the prefix sums are ascending
                    checked_index(g, 0, C.h);
                    continue;
                }
                const FInfo fi = cached ? s_fi[s] : frame_info(C.fs + f);
                const NodePre pre = node_pre(F, fi, g * GN + lane);   // independent of the pixel pass
                int ok = 1;
                if (lane == 0) {
                    const int need = __ldg(F.group_need + g);
                    const unsigned *cnt = reinterpret_cast<const unsigned *>(F.group_cnt + g);
                    if ((int)ld_acquire_u32(cnt) < need) {
                        const unsigned long long t0 = gtimer();
                        while ((int)ld_acquire_u32(cnt) < need) {
                            if (ld_vol(&C.h->abort)) {
                                ok = 0;
                                break;
                            }
                            if (gtimer() - t0 > WAIT_NS) {
                                C.h->err = D2IC_WAIT_TIMEOUT;
                                atomicExch(&C.h->abort, 1);
                                ok = 0;
                                break;
                            }
                            __nanosleep(32);
                        }
                    }
                }
                __syncwarp();                          // the slots seen by lane 0 are seen by the warp
                if (!__shfl_sync(0xffffffffu, ok, 0)) break;
                DF q[5];
                node_post(F, fi, g * GN + lane, pre, q);
#pragma unroll
                for (int i = 0; i < 5; ++i) q[i] = df_warp_sum(q[i]);
                // group -> supergroup (SG groups) -> frame: the warp that completes a level reduces
                // it; a supergroup's sum is the same lane-ordered warp sum on both paths
                const int ngr = F.n_groups, nsg = (ngr + SG - 1) / SG, sg = g / SG;
                const int members = min(SG, ngr - sg * SG);
                float2 *gp = reinterpret_cast<float2 *>(F.group_part);
                int last = 0;
                if (blockred) {                        // members are warps 0 .. members-1 here
                    if (lane == 0) {
#pragma unroll
                        for (int i = 0; i < 5; ++i) s_gq[wid][i] = q[i];
                        F.group_cnt[g] = 0;            // every chunk of this round has counted
                        __threadfence_block();
                        last = atomicAdd(&s_sgcnt, 1) == members - 1;
                        if (last) {
                            s_sgcnt = 0;
                            __threadfence_block();
                        }
                    }
                } else if (lane == 0) {
#pragma unroll
                    for (int i = 0; i < 5; ++i) gp[(size_t)g * D2IC_NPART + i] = make_float2(q[i].hi, q[i].lo);
                    F.group_cnt[g] = 0;                // every chunk of this round has counted
                    last = atom_acq_rel_add(F.group_cnt + ngr + sg, 1) == members - 1;
                    if (last) F.group_cnt[ngr + sg] = 0;
                }
                __syncwarp();
                if (__shfl_sync(0xffffffffu, last, 0)) {
                    DF v[5];
                    const int gg = sg * SG + lane;
#pragma unroll
                    for (int i = 0; i < 5; ++i) {
                        DF t = DF{0.f, 0.f};
                        if (lane < members) {
                            if (blockred) {
                                t = s_gq[lane][i];
                            } else {
                                const float2 t2 = __ldcg(gp + (size_t)gg * D2IC_NPART + i);
                                t = DF{t2.x, t2.y};
                            }
                        }
                        v[i] = df_warp_sum(t);
                    }
                    int lastf = 0;
                    if (lane == 0) {
                        float2 *sp = gp + (size_t)(ngr + sg) * D2IC_NPART;
#pragma unroll
                        for (int i = 0; i < 5; ++i) sp[i] = make_float2(v[i].hi, v[i].lo);
                        lastf = atom_acq_rel_add(F.group_cnt + ngr + nsg, 1) == nsg - 1;
                        if (lastf) F.group_cnt[ngr + nsg] = 0;
                    }
                    __syncwarp();
                    if (__shfl_sync(0xffffffffu, lastf, 0)) {   // the frame's last supergroup
                        const bool rt = trace != nullptr && lane == 0 && round < trace_rounds;
                        if (rt) trace[7 * round + 3] = gtimer();
                        frame_r(F, f, C, eval_only, lane);
                        int last_frame = 0;
                        if (lane == 0) last_frame = na == 1 || atom_acq_rel_add(&C.h->frames_done, 1) == na - 1;
                        __syncwarp();
                        if (__shfl_sync(0xffffffffu, last_frame, 0)) {
                            // every frame of the round has run its control step, so every block's
                            // work of the round is done: rebuild the active list and release the round
                            if (lane == 0) C.h->frames_done = 0;
                            int stop = 0;
                            if (ld_vol(&C.h->finished)) {
                                // no block still reads the list copy of an earlier round (bounded)
                                int past = 1;
                                if (lane == 0) past = wait_blocks_past(C.h, gridDim.x * (unsigned)round);
                                if (__shfl_sync(0xffffffffu, past, 0))
                                    rebuild_active_warp(frames, n_frames, C, lane);
                                if (lane == 0) C.h->finished = 0;
                                stop = stop_flags & STOP_ON_FINISH;
                            }
                            if (lane == 0 && (stop || ((stop_flags & STOP_ON_IRQ) && ld_vol(&C.h->irq))))
                                C.h->slice_stop = 1;   // published by the release below
                            __syncwarp();
                            if (lane == 0) {
                                __threadfence();
                                atomicExch(&C.h->rounds_done, (unsigned)(round + 1));
                            }
                        }
                        if (rt) trace[7 * round + 4] = gtimer();
                    }
                }
            }
            if (trr) trace[7 * round + 2] = gtimer();
            // stage the next round's first chunk (same ranges if the active list is unchanged).  Only
            // from the shared-memory copy of the list: the global one may be rebuilt meanwhile.
            if (cached && p_ok && cb < ce && round + 1 < max_rounds && !ld_vol(&C.h->abort)) {
                cur = 0;
                pf_m0 = fetch_meta(cb);
                pf_st0 = issue_tma(pf_m0, pipe_i);
                if (cb + cs < ce) pf_m1 = fetch_meta(cb + cs);
                pf = true;
                pf_na = na;
                pf_total = total;
            }
        }
        // ---- end of round: wait until the warp that ran the round's last frame step releases it
        // (rounds_done is monotonic, so a block that arrives after the release passes at once) ----
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(&C.h->blocks_past, 1u);           // this block's list reads of the round are done
            const unsigned target = (unsigned)(round + 1);
            if (ld_acquire_u32(&C.h->rounds_done) < target) {
                const unsigned long long t0 = gtimer();
                while (ld_acquire_u32(&C.h->rounds_done) < target) {
                    if (ld_vol(&C.h->abort)) break;
                    if (gtimer() - t0 > WAIT_NS) {
                        C.h->err = D2IC_WAIT_TIMEOUT;
                        atomicExch(&C.h->abort, 1);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            __threadfence();
        }
        __syncthreads();
        // one round trip for the next round's state: the header (thread 0) and, for the list as it
        // was, each frame's candidate rule; a changed list (a frame finished) is reloaded
        if (threadIdx.x == 0) {
            s_hdr[0] = ld_vol(&C.h->n_active);
            s_hdr[1] = ld_vol(&C.h->total_chunks);
            s_hdr[2] = ld_vol(&C.h->total_groups);
            s_hdr[3] = ld_vol(&C.h->abort);
            s_hdr[4] = ld_vol(&C.h->slice_stop);
            s_hdr[5] = ld_vol(&C.h->list_buf);
        }
        if (na <= FCACHE)
            for (int s = threadIdx.x; s < na; s += NT) s_fi[s] = frame_info(C.fs + s_act[s]);
        __syncthreads();
        if (s_hdr[0] != na && s_hdr[0] > 0 && !s_hdr[3]) {
            load_list(C, s_hdr[5], s_hdr[0], s_cpre, s_gpre, s_act, s_fi);
            __syncthreads();
        }
        if (trr) trace[7 * round + 5] = gtimer();
        ++round;
    }

    if (pf) {                                       // no copy in flight at exit (bounded wait)
        if (lane < CAND_N) mbar_arrive(&s_bar[wid][pipe_i & 1]);
        mbar_wait(&s_bar[wid][pipe_i & 1], (pipe_i >> 1) & 1u);
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
        for (int i = blockIdx.x * NT + threadIdx.x; i < nn; i += gridDim.x * NT) {
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
constexpr size_t ENGINE_SMEM = (size_t)NWARP * WARP_SMEM;   // per warp: 2 record + 2 tile buffers

template <int KIND>
static cudaError_t occupancy(int *blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(cg_engine<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ENGINE_SMEM);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(cg_engine<KIND, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ENGINE_SMEM);
    if (e != cudaSuccess) return e;
    int one = 0;   // the one-frame instance must fit as many blocks as the general one
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&one, cg_engine<KIND, true>, NT, ENGINE_SMEM);
    if (e != cudaSuccess) return e;
    int many = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&many, cg_engine<KIND>, NT, ENGINE_SMEM);
    *blocks_per_sm = one < many ? one : many;
    return e;
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
                         bool new_batch = true, int stop_flags = 0) {
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
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = ENGINE_SMEM;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const bool one = n_frames == 1;
    if (kind == D2IC_INTERP_CUBIC)
        e = one ? cudaLaunchKernelEx(&cfg, cg_engine<D2IC_INTERP_CUBIC, true>, frames, n_frames, cb, eval_only, u_eval,
                                     J_out, grad_out, trace, trace_rounds, max_rounds, stop_flags)
                : cudaLaunchKernelEx(&cfg, cg_engine<D2IC_INTERP_CUBIC>, frames, n_frames, cb, eval_only, u_eval, J_out,
                                     grad_out, trace, trace_rounds, max_rounds, stop_flags);
    else
        e = one ? cudaLaunchKernelEx(&cfg, cg_engine<D2IC_INTERP_LINEAR, true>, frames, n_frames, cb, eval_only,
                                     u_eval, J_out, grad_out, trace, trace_rounds, max_rounds, stop_flags)
                : cudaLaunchKernelEx(&cfg, cg_engine<D2IC_INTERP_LINEAR>, frames, n_frames, cb, eval_only, u_eval,
                                     J_out, grad_out, trace, trace_rounds, max_rounds, stop_flags);
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

// Workspace of one frame: 7 node buffers (u x2, g x3, dir x2), the K gradient
// slots per node (16 bytes: gx, gy and the chunk's r^2 sum as a double-float),
// the partials (D2IC_NPART double-float pairs) of every group and then of every
// supergroup of SG groups, the completion counters (groups, supergroups, the
// frame's count of supergroups), and the tile origins (4 bytes per chunk).
static size_t ws_layout(int n_nodes, int n_chunks, int node_chunk_k, size_t off[5]) {
    const size_t ng = (size_t)(n_nodes + GN - 1) / GN;
    size_t o = 0;
    off[0] = o;                                               // node_ws
    o += align256(sizeof(float) * 14 * (size_t)n_nodes);
    off[1] = o;                                               // node_grad
    o += align256(sizeof(float) * 4 * (size_t)node_chunk_k * n_nodes);
    off[2] = o;                                               // group_part
    const size_t ns = (ng + SG - 1) / SG;                     // supergroups of SG groups
    o += align256(sizeof(float) * 2 * D2IC_NPART * (ng + ns));
    off[3] = o;                                               // group_cnt
    o += align256(sizeof(int) * (ng + ns + 1));
    off[4] = o;                                               // chunk_tile
    o += align256(sizeof(int) * (size_t)(n_chunks > 0 ? n_chunks : 1));
    return o;
}

extern "C" size_t d2ic_frame_workspace_bytes(int n_nodes, int n_chunks, int node_chunk_k) {
    size_t off[5];
    if (node_chunk_k < 1) node_chunk_k = 1;
    if (n_nodes < 1) n_nodes = 1;
    return ws_layout(n_nodes, n_chunks, node_chunk_k, off);
}

extern "C" int d2ic_frame_bind_workspace(d2ic_frame_t *f, void *ws) {
    D2IC_REQUIRE(f && ws, "d2ic_frame_bind_workspace: null pointer");
    D2IC_REQUIRE(((uintptr_t)ws & 255) == 0, "d2ic_frame_bind_workspace: workspace must be 256-byte aligned");
    D2IC_REQUIRE(f->n_nodes >= 1 && f->n_chunks >= 0 && f->node_chunk_k >= 1 && f->node_chunk_k <= 255,
                 "d2ic_frame_bind_workspace: bad sizes");
    size_t off[5];
    ws_layout(f->n_nodes, f->n_chunks, f->node_chunk_k, off);
    char *p = (char *)ws;
    f->node_ws = (float *)(p + off[0]);
    f->node_grad = (float *)(p + off[1]);
    f->group_part = (float *)(p + off[2]);
    f->group_cnt = (int *)(p + off[3]);
    f->chunk_tile = (int *)(p + off[4]);
    f->n_groups = (f->n_nodes + GN - 1) / GN;
    return D2IC_OK;
}

// Tensor-map encoding comes from the driver through the runtime's entry-point
// query, so the library does not link libcuda directly.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

extern "C" int d2ic_frame_encode_tiles(d2ic_frame_t *f, int tile_w, int tile_h) {
    static_assert(sizeof(d2ic_frame_t) % 64 == 0, "descriptor arrays keep every tensor map 64-byte aligned");
    static_assert(offsetof(d2ic_frame_t, coeff_map) == 0 && sizeof(f->coeff_map) == sizeof(CUtensorMap),
                  "tensor map first in the descriptor");
    D2IC_REQUIRE(f, "d2ic_frame_encode_tiles: null frame");
    memset(f->coeff_map, 0, sizeof(f->coeff_map));
    f->tile_w = 0;
    f->tile_h = 0;
    if (tile_w == 0) return D2IC_OK;
    D2IC_REQUIRE(tile_w >= 4 && tile_w % 4 == 0 && tile_h >= 4 && tile_w <= 256 && tile_h <= 256 &&
                     tile_w * tile_h <= D2IC_TILE_MAX_FLOATS,
                 "d2ic_frame_encode_tiles: tile %d x %d (width a multiple of 4, at most %d floats)", tile_w, tile_h,
                 D2IC_TILE_MAX_FLOATS);
    D2IC_REQUIRE(f->coeff && ((uintptr_t)f->coeff & 15) == 0, "d2ic_frame_encode_tiles: coeff must be 16-byte aligned");
    D2IC_REQUIRE(f->pad % 4 == 0 && f->cpitch % 4 == 0 && f->W >= 1 && f->H >= 1 && f->cpitch >= f->W + 2 * f->pad,
                 "d2ic_frame_encode_tiles: pad and cpitch must be multiples of 4 (pad %d, cpitch %d)", f->pad,
                 f->cpitch);
    D2IC_REQUIRE(f->W + 2 * f->pad < 32768 && f->H + 2 * f->pad < 32768,
                 "d2ic_frame_encode_tiles: image %d x %d too large for tile origins", f->W, f->H);
    EncodeTiledFn fn = encode_tiled_fn();
    if (!fn) {
        set_error("d2ic_frame_encode_tiles: the driver provides no cuTensorMapEncodeTiled");
        return D2IC_UNSUPPORTED;
    }
    alignas(64) CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)(f->W + 2 * f->pad), (cuuint64_t)(f->H + 2 * f->pad)};
    const cuuint64_t strides[1] = {(cuuint64_t)f->cpitch * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)tile_w, (cuuint32_t)tile_h};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)f->coeff, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("d2ic_frame_encode_tiles: cuTensorMapEncodeTiled failed (%d)", (int)r);
        return D2IC_CUDA_ERROR;
    }
    memcpy(f->coeff_map, &map, sizeof(map));
    f->tile_w = tile_w;
    f->tile_h = tile_h;
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

extern "C" int d2ic_cg_slice_ex(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes,
                                int interp_kind, int grid_blocks, int max_rounds, int stop_flags, void *stream) {
    D2IC_REQUIRE(max_rounds >= 1, "d2ic_cg_slice_ex: max_rounds must be >= 1 (got %d)", max_rounds);
    D2IC_REQUIRE((stop_flags & ~(D2IC_STOP_ON_FINISH | D2IC_STOP_ON_IRQ)) == 0, "d2ic_cg_slice_ex: unknown stop flags %d",
                 stop_flags);
    return launch_engine(frames, n_frames, control, control_bytes, interp_kind, grid_blocks, 0, nullptr, nullptr,
                         nullptr, nullptr, 0, (cudaStream_t)stream, max_rounds, false, stop_flags);
}

extern "C" size_t d2ic_cg_irq_offset(void) { return offsetof(CtlHeader, irq); }

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
// device address of the array, per device (the host-side name is a stand-in, not a device address);
// atomic so that threads making their first call on a device at the same time do not race
static std::atomic<void *> g_noalloc_addr[64];

// Writes a frame descriptor into the scratch array.  The descriptor travels as a kernel argument,
// copied at launch, so no host buffer has to outlive the call and the host does not wait.
__global__ void noalloc_put_descriptor(const d2ic_frame_t f, d2ic_frame_t *dst) {
    static_assert(sizeof(d2ic_frame_t) % 8 == 0, "descriptor copied in 8-byte words");
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(&f);
    unsigned long long *d = reinterpret_cast<unsigned long long *>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(d2ic_frame_t) / 8); i += blockDim.x) d[i] = src[i];
}

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
    void *addr = g_noalloc_addr[dev].load(std::memory_order_relaxed);
    if (addr == nullptr) {                     // set-up, once per device, with that device current
        e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(noalloc scratch)");
        g_noalloc_addr[dev].store(addr, std::memory_order_relaxed);
    }
    char *base = (char *)addr;
    d2ic_frame_t f = *frame;                   // caller's inputs/outputs, workspace from the array
    int st = d2ic_frame_bind_workspace(&f, base + desc_bytes + ctl_bytes);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    noalloc_put_descriptor<<<1, 64, 0, s>>>(f, (d2ic_frame_t *)base);
    D2IC_CHECK_LAUNCH("noalloc descriptor write");
    // the launch clears the control header on `s`; the kernel initialises every workspace word it reads
    return launch_engine((const d2ic_frame_t *)base, 1, base + desc_bytes, ctl_bytes, interp_kind, 0, 0, nullptr,
                         nullptr, nullptr, nullptr, 0, s);
}
