// Initial motion: integer-translation ZNCC search at element centres and
// inverse-distance projection of the centre displacements onto the nodes.
//
// ZNCC (d2ic/solver_translation_zncc.py:89-168): one block per centre; the
// template (win x win) and the search patch ((win + 2 s)^2) are staged in
// shared memory; each thread scores a subset of the (2 s + 1)^2 offsets with a
// two-pass (mean, then centred sums) window normalisation; the block keeps the
// first maximum in row-major (ky, kx) order.  FP32 arithmetic on the CUDA
// cores: nothing here is a dense contraction.
#include "common.cuh"

namespace d2ic {

__global__ void zncc_kernel(const float *__restrict__ ref, int Hr, int Wr, const float *__restrict__ def, int Hd,
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

// IDW (power p) of centre displacements onto nodes.  FP64 sqrt/divide are
// slow on GB300, so per-pair math is FP32 (squared distances of pixel-grid
// coordinates are exact in FP32 up to 2^24) with Kahan-compensated FP32 sums
// inside each 256-centre tile and FP64 accumulation across tiles.
__global__ void idw_kernel(const float2 *__restrict__ nodes, int n_nodes, const float2 *__restrict__ centers,
                           const float2 *__restrict__ disp, int nc, float power, float2 *__restrict__ out) {
    __shared__ float2 sc[256], sd[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float2 p = (i < n_nodes) ? nodes[i] : make_float2(0.f, 0.f);
    double sw = 0.0, sx = 0.0, sy = 0.0;
    int exact = -1;
    float2 ev = make_float2(0.f, 0.f);
    const bool p2 = (power == 2.0f);
    for (int base = 0; base < nc; base += 256) {
        const int m = min(256, nc - base);
        __syncthreads();
        if (threadIdx.x < m) {
            sc[threadIdx.x] = centers[base + threadIdx.x];
            sd[threadIdx.x] = disp[base + threadIdx.x];
        }
        __syncthreads();
        if (i < n_nodes && exact < 0) {
            float tw = 0.f, tx = 0.f, ty = 0.f, cw = 0.f, cx = 0.f, cy = 0.f;   // tile sums + compensation
            for (int k = 0; k < m; ++k) {
                const float2 d = sd[k];
                if (d.x != d.x || d.y != d.y) continue;      // centres with NaN displacement are dropped
                const float dx = sc[k].x - p.x, dy = sc[k].y - p.y;
                const float d2 = dx * dx + dy * dy;
                if (d2 < 1e-12f) {                            // dist < 1e-6: take this centre's value
                    exact = base + k;
                    ev = d;
                    break;
                }
                const float w = p2 ? 1.0f / d2 : powf(sqrtf(d2), -power);
                float y = w - cw, t = tw + y;
                cw = (t - tw) - y;
                tw = t;
                y = w * d.x - cx; t = tx + y; cx = (t - tx) - y; tx = t;
                y = w * d.y - cy; t = ty + y; cy = (t - ty) - y; ty = t;
            }
            sw += (double)tw - (double)cw;
            sx += (double)tx - (double)cx;
            sy += (double)ty - (double)cy;
        }
    }
    if (i >= n_nodes) return;
    if (exact >= 0) out[i] = ev;
    else if (sw > 0.0) out[i] = make_float2((float)(sx / sw), (float)(sy / sw));
    else out[i] = make_float2(0.f, 0.f);
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
    zncc_kernel<<<n_centers, 256, smem, (cudaStream_t)stream>>>(ref, Hr, Wr, def, Hd, Wd, (const float2 *)centers, win,
                                                               search, (float2 *)u_out, score_out);
    D2IC_CHECK_LAUNCH("zncc_kernel");
    return D2IC_OK;
}

extern "C" int d2ic_idw_project(const float *nodes, int n_nodes, const float *centers, const float *disp,
                                int n_centers, float power, float *u_out, void *stream) {
    D2IC_REQUIRE(nodes && u_out && (n_centers == 0 || (centers && disp)), "d2ic_idw_project: null pointer");
    D2IC_REQUIRE(n_nodes >= 0 && n_centers >= 0, "d2ic_idw_project: bad sizes");
    if (n_nodes == 0) return D2IC_OK;
    idw_kernel<<<(n_nodes + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        (const float2 *)nodes, n_nodes, (const float2 *)centers, (const float2 *)disp, n_centers, power, (float2 *)u_out);
    D2IC_CHECK_LAUNCH("idw_kernel");
    return D2IC_OK;
}
