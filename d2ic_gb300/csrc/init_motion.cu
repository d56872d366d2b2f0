// Initial motion: integer-translation ZNCC search at element centres and
// inverse-distance projection of the centre displacements onto the nodes.
//
// ZNCC (d2ic/solver_translation_zncc.py:89-168): one block per centre; the
// template (win x win) and the search patch ((win + 2 s)^2) are staged in
// shared memory; each thread scores one (up to 1024 offsets) or several of the (2 s + 1)^2 offsets with a
// two-pass (mean, then centred sums) window normalisation; the block keeps the
// first maximum in row-major (ky, kx) order.  FP32 arithmetic on the CUDA
// cores: nothing here is a dense contraction.
#include "common.cuh"

namespace d2ic {

__global__ void __launch_bounds__(1024) zncc_kernel(const float *__restrict__ ref, int Hr, int Wr, const float *__restrict__ def, int Hd,
                            int Wd, const float2 *__restrict__ centers, int win, int search, float2 *__restrict__ u_out,
                            float *__restrict__ score_out) {
    extern __shared__ float sm[];
    const int ps = win + 2 * search;
    float *tpl = sm;                 // win * win, normalised template
    float *pat = sm + win * win;     // ps * ps
    __shared__ float s_red[32];
    __shared__ int s_idx[32];
    __shared__ float s_mean, s_inv;
    const int c = blockIdx.x;
    const float2 ctr = centers[c];
    // half to even, as jnp.rint; non-finite or far-away centres fail the bounds test below
    const bool finite = fabsf(ctr.x) < 1e7f && fabsf(ctr.y) < 1e7f;
    const int x = finite ? (int)rintf(ctr.x) : -(1 << 28), y = finite ? (int)rintf(ctr.y) : -(1 << 28);
    const int r = win / 2;
    const bool tpl_ok = (y - r >= 0) && (y + r < Hr) && (x - r >= 0) && (x + r < Wr);
    const int xs = x - search, ys = y - search, xe = x + search, ye = y + search;
    const bool patch_ok = (ys - r >= 0) && (ye + r < Hd) && (xs - r >= 0) && (xe + r < Wd);
    if (!(tpl_ok && patch_ok)) {
        if (threadIdx.x == 0) {
            u_out[c] = make_float2(0.f, 0.f);
            score_out[c] = __int_as_float(0x7fc00000);
        }
        return;
    }
    const int n = win * win;
    for (int i = threadIdx.x; i < n; i += blockDim.x) tpl[i] = __ldg(ref + (size_t)(y - r + i / win) * Wr + (x - r + i % win));
    for (int i = threadIdx.x; i < ps * ps; i += blockDim.x)
        pat[i] = __ldg(def + (size_t)(ys - r + i / ps) * Wd + (xs - r + i % ps));
    __syncthreads();
    // template mean and population std (two passes)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float a = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a += tpl[i];
    a = warp_sum_f(a);
    if (lane == 0) s_red[wid] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < nw; ++w) t += s_red[w];
        s_mean = t / (float)n;
    }
    __syncthreads();
    const float mu = s_mean;
    a = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float d = tpl[i] - mu;
        a += d * d;
    }
    a = warp_sum_f(a);
    __syncthreads();
    if (lane == 0) s_red[wid] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < nw; ++w) t += s_red[w];
        s_inv = 1.0f / (sqrtf(t / (float)n) + 1e-12f);
    }
    __syncthreads();
    const float inv = s_inv;
    for (int i = threadIdx.x; i < n; i += blockDim.x) tpl[i] = (tpl[i] - mu) * inv;
    __syncthreads();
    // score every offset
    const int npa = 2 * search + 1;
    float best = -INFINITY;
    int bidx = 0x7fffffff;
    for (int o = threadIdx.x; o < npa * npa; o += blockDim.x) {
        const int ky = o / npa, kx = o % npa;
        const float *w0 = pat + ky * ps + kx;
        float s = 0.f;
        for (int i = 0; i < win; ++i)
            for (int j = 0; j < win; ++j) s += w0[i * ps + j];
        const float mw = s / (float)n;
        float v = 0.f, cr = 0.f;
        for (int i = 0; i < win; ++i)
            for (int j = 0; j < win; ++j) {
                const float d = w0[i * ps + j] - mw;
                v += d * d;
                cr += d * tpl[i * win + j];
            }
        const float sc = cr / (sqrtf(v / (float)n) + 1e-12f) / (float)n;
        if (sc > best || (sc != sc && best == best)) {   // NaN wins, as argmax
            best = sc;
            bidx = o;
        }
    }
    // block argmax: larger score, then smaller index
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, off);
        if (ob > best || (ob == best && oi < bidx)) {
            best = ob;
            bidx = oi;
        }
    }
    __syncthreads();
    if (lane == 0) {
        s_red[wid] = best;
        s_idx[wid] = bidx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = s_red[0];
        int bi = s_idx[0];
        for (int w = 1; w < nw; ++w)
            if (s_red[w] > b || (s_red[w] == b && s_idx[w] < bi)) {
                b = s_red[w];
                bi = s_idx[w];
            }
        const int ky = bi / npa, kx = bi % npa;
        u_out[c] = make_float2((float)(xs + kx - x), (float)(ys + ky - y));
        score_out[c] = b;
    }
}

// IDW (power p) of centre displacements onto nodes: one warp per NPW nodes (8 warps per block; 4
// nodes on large meshes, 1 where 4 would leave SMs idle), the centres staged in shared-memory tiles
// of 256 that the block's warps share; lane l takes centres l, l + 32, ... of each tile against all
// of the warp's nodes, so one centre read serves NPW pairs.  FP64 sqrt/divide are slow on GB300, so per-pair math is FP32 (squared
// distances of pixel-grid coordinates are exact in FP32 up to 2^24) with the reciprocal correctly
// rounded; each lane sums a tile (8 centres) in FP32 and adds that into FP64 accumulators, and the
// lanes' FP64 sums are reduced over the warp at the end.  A centre closer than 1e-6 gives the node
// its displacement: the smallest such centre index, tracked without a branch (its infinite weight
// is discarded).  Centres with a NaN displacement are dropped.
constexpr int IDW_TILE = 256;
template <int IDW_NODES>
__global__ void __launch_bounds__(256) idw_kernel(const float2 *__restrict__ nodes, int n_nodes,
                                                  const float2 *__restrict__ centers, const float2 *__restrict__ disp,
                                                  int nc, float power, float2 *__restrict__ out) {
    __shared__ float2 sc[IDW_TILE], sd[IDW_TILE];
    const int lane = threadIdx.x & 31;
    const int i0 = (blockIdx.x * 8 + (threadIdx.x >> 5)) * IDW_NODES;
    float2 p[IDW_NODES];
    double sw[IDW_NODES], sx[IDW_NODES], sy[IDW_NODES];
    int ex[IDW_NODES];
#pragma unroll
    for (int j = 0; j < IDW_NODES; ++j) {
        p[j] = (i0 + j < n_nodes) ? nodes[i0 + j] : make_float2(0.f, 0.f);
        sw[j] = sx[j] = sy[j] = 0.0;
        ex[j] = 0x7fffffff;
    }
    const bool p2 = (power == 2.0f);
    for (int base = 0; base < nc; base += IDW_TILE) {
        const int m = min(IDW_TILE, nc - base);
        __syncthreads();
        if ((int)threadIdx.x < m) {
            sc[threadIdx.x] = centers[base + threadIdx.x];
            sd[threadIdx.x] = disp[base + threadIdx.x];
        }
        __syncthreads();
        if (i0 >= n_nodes) continue;
        float tw[IDW_NODES], tx[IDW_NODES], ty[IDW_NODES];
#pragma unroll
        for (int j = 0; j < IDW_NODES; ++j) tw[j] = tx[j] = ty[j] = 0.f;
        for (int k = lane; k < m; k += 32) {
            const float2 d = sd[k];
            if (d.x != d.x || d.y != d.y) continue;      // centres with NaN displacement are dropped
            const float2 c = sc[k];
#pragma unroll
            for (int j = 0; j < IDW_NODES; ++j) {
                const float dx = c.x - p[j].x, dy = c.y - p[j].y;
                const float d2 = dx * dx + dy * dy;
                ex[j] = d2 < 1e-12f ? min(ex[j], base + k) : ex[j];   // dist < 1e-6
                const float w = p2 ? __frcp_rn(d2) : powf(sqrtf(d2), -power);
                tw[j] += w;
                tx[j] += w * d.x;
                ty[j] += w * d.y;
            }
        }
#pragma unroll
        for (int j = 0; j < IDW_NODES; ++j) {
            sw[j] += (double)tw[j];
            sx[j] += (double)tx[j];
            sy[j] += (double)ty[j];
        }
    }
    if (i0 >= n_nodes) return;
#pragma unroll
    for (int j = 0; j < IDW_NODES; ++j) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sw[j] += __shfl_xor_sync(0xffffffffu, sw[j], o);
            sx[j] += __shfl_xor_sync(0xffffffffu, sx[j], o);
            sy[j] += __shfl_xor_sync(0xffffffffu, sy[j], o);
            ex[j] = min(ex[j], __shfl_xor_sync(0xffffffffu, ex[j], o));
        }
        if (lane == j && i0 + j < n_nodes) {
            if (ex[j] != 0x7fffffff) out[i0 + j] = disp[ex[j]];
            else if (sw[j] > 0.0) out[i0 + j] = make_float2((float)(sx[j] / sw[j]), (float)(sy[j] / sw[j]));
            else out[i0 + j] = make_float2(0.f, 0.f);
        }
    }
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_zncc_match(const float *ref, int Hr, int Wr, const float *def, int Hd, int Wd,
                               const float *centers, int n_centers, int win, int search, float *u_out,
                               float *score_out, void *stream) {
    D2IC_REQUIRE(ref && def && u_out && score_out && (centers || n_centers == 0), "d2ic_zncc_match: null pointer");
    D2IC_REQUIRE(win > 0 && (win % 2) == 1, "d2ic_zncc_match: win must be odd and positive (got %d)", win);
    D2IC_REQUIRE(search >= 0 && n_centers >= 0 && Hr > 0 && Wr > 0 && Hd > 0 && Wd > 0, "d2ic_zncc_match: bad sizes");
    const size_t smem = sizeof(float) * ((size_t)win * win + (size_t)(win + 2 * search) * (win + 2 * search));
    D2IC_REQUIRE(smem <= 200 * 1024, "d2ic_zncc_match: win/search too large for shared memory (%zu bytes)", smem);
    if (n_centers == 0) return D2IC_OK;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(zncc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_status(e, "zncc smem attribute");
    }
    // one thread per offset where they fit in a block (289 offsets at search 8: 320 threads), so that
    // no thread scores a second offset while the others wait
    const int npa = 2 * search + 1;
    const int threads = npa * npa >= 1024 ? 1024 : ((npa * npa + 31) / 32) * 32;
    zncc_kernel<<<n_centers, threads < 64 ? 64 : threads, smem, (cudaStream_t)stream>>>(
        ref, Hr, Wr, def, Hd, Wd, (const float2 *)centers, win, search, (float2 *)u_out, score_out);
    D2IC_CHECK_LAUNCH("zncc_kernel");
    return D2IC_OK;
}

extern "C" int d2ic_idw_project(const float *nodes, int n_nodes, const float *centers, const float *disp,
                                int n_centers, float power, float *u_out, void *stream) {
    D2IC_REQUIRE(nodes && u_out && (n_centers == 0 || (centers && disp)), "d2ic_idw_project: null pointer");
    D2IC_REQUIRE(n_nodes >= 0 && n_centers >= 0, "d2ic_idw_project: bad sizes");
    if (n_nodes == 0) return D2IC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (n_nodes >= 4 * 8 * 912)   // at least ~2 waves of 4-node warps (3 blocks per SM on 152 SMs)
        idw_kernel<4><<<(n_nodes + 31) / 32, 256, 0, s>>>((const float2 *)nodes, n_nodes, (const float2 *)centers,
                                                          (const float2 *)disp, n_centers, power, (float2 *)u_out);
    else
        idw_kernel<1><<<(n_nodes + 7) / 8, 256, 0, s>>>((const float2 *)nodes, n_nodes, (const float2 *)centers,
                                                        (const float2 *)disp, n_centers, power, (float2 *)u_out);
    D2IC_CHECK_LAUNCH("idw_kernel");
    return D2IC_OK;
}
