// Pixel-asset setup on the device: the element of every pixel on a tensor-grid
// mesh (d2ic/pixel_assets.py:135-237 for the grids mask_to_mesh builds), and the
// local (xi, eta) coordinates of every pixel in its Q4 element by Newton's method
// (d2ic/pixel_assets.py:277-294, the reference's _newton_quadrature), in FP64.
//
// Each step is the host restatement's operation sequence with correctly rounded
// FP64 intrinsics (no contraction into FMAs): shape functions and derivatives,
// residual and Jacobian as left-to-right sums of products, the 2x2 solve by LU
// with partial pivoting, and the update.  A pixel whose update is exactly zero
// keeps its coordinates for every later step, so it stops there.  The results
// are therefore bit-identical to the host restatement.
#include "common.cuh"

namespace d2ic {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// (xi, eta) of the point (px, py) in the Q4 element with node coordinates X, Y: at most `iters`
// Newton steps from (0, 0), stopping after the first exactly-zero update.
__device__ __forceinline__ void newton_local(const double X[4], const double Y[4], double px, double py, int iters,
                                             double &xi_out, double &eta_out) {
        double xi = 0.0, eta = 0.0;
        for (int it = 0; it < iters; ++it) {
            const double om_x = sub(1.0, xi), op_x = add(1.0, xi), om_e = sub(1.0, eta), op_e = add(1.0, eta);
            const double n0 = mul(mul(0.25, om_x), om_e), n1 = mul(mul(0.25, op_x), om_e);
            const double n2 = mul(mul(0.25, op_x), op_e), n3 = mul(mul(0.25, om_x), op_e);
            const double dx0 = mul(-0.25, om_e), dx1 = mul(0.25, om_e), dx2 = mul(0.25, op_e), dx3 = mul(-0.25, op_e);
            const double de0 = mul(-0.25, om_x), de1 = mul(-0.25, op_x), de2 = mul(0.25, op_x), de3 = mul(0.25, om_x);
            const double fx = sub(add(add(add(mul(n0, X[0]), mul(n1, X[1])), mul(n2, X[2])), mul(n3, X[3])), px);
            const double fy = sub(add(add(add(mul(n0, Y[0]), mul(n1, Y[1])), mul(n2, Y[2])), mul(n3, Y[3])), py);
            const double j11 = add(add(add(mul(dx0, X[0]), mul(dx1, X[1])), mul(dx2, X[2])), mul(dx3, X[3]));
            const double j21 = add(add(add(mul(dx0, Y[0]), mul(dx1, Y[1])), mul(dx2, Y[2])), mul(dx3, Y[3]));
            const double j12 = add(add(add(mul(de0, X[0]), mul(de1, X[1])), mul(de2, X[2])), mul(de3, X[3]));
            const double j22 = add(add(add(mul(de0, Y[0]), mul(de1, Y[1])), mul(de2, Y[2])), mul(de3, Y[3]));
            // LU with partial pivoting: rows swapped when |a21| > |a11|
            const bool swap = fabs(j21) > fabs(j11);
            const double p11 = swap ? j21 : j11, p12 = swap ? j22 : j12, p21 = swap ? j11 : j21, p22 = swap ? j12 : j22;
            const double q1 = swap ? fy : fx, q2 = swap ? fx : fy;
            const double l21 = dvd(p21, p11);
            const double d2 = dvd(sub(q2, mul(l21, q1)), sub(p22, mul(l21, p12)));
            const double d1 = dvd(sub(q1, mul(p12, d2)), p11);
            xi = sub(xi, d1);
            eta = sub(eta, d2);
            const bool moving = d1 != 0.0 || d2 != 0.0 || !isfinite(d1) || !isfinite(d2);
            if (!moving) break;
        }
        xi_out = xi;
        eta_out = eta;
}

__global__ void __launch_bounds__(256) local_coords_kernel(const double *__restrict__ pc, const int *__restrict__ pn,
                                                           const double *__restrict__ nodes, long long n, int iters,
                                                           double *__restrict__ xi_out, double *__restrict__ eta_out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        double X[4], Y[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int k = pn[4 * p + a];
            X[a] = nodes[2 * (long long)k];
            Y[a] = nodes[2 * (long long)k + 1];
        }
        newton_local(X, Y, pc[2 * p], pc[2 * p + 1], iters, xi_out[p], eta_out[p]);
    }
}

// number of entries of the ascending array g[0..n) that are <= x (searchsorted, side "right")
__device__ __forceinline__ int count_le(const double *g, int n, double x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (g[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// The four cells around the pixel whose closed rectangles can hold it (the last grid line <= x
// and the one before, likewise in y); the lowest element index among those that do.
__global__ void __launch_bounds__(256) structured_assign_kernel(const double *__restrict__ pc, long long n,
                                                                const double *__restrict__ gx, int nx,
                                                                const double *__restrict__ gy, int ny,
                                                                const long long *__restrict__ cell,
                                                                long long *__restrict__ elts) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const double x = pc[2 * p], y = pc[2 * p + 1];
        const int ixr = count_le(gx, nx, x) - 1, iyr = count_le(gy, ny, y) - 1;
        long long best = -1;
        for (int dx = 0; dx < 2; ++dx) {
            const int cx = ixr - dx;
            if (cx < 0 || cx > nx - 2 || !(gx[cx] <= x && x <= gx[cx + 1])) continue;
            for (int dy = 0; dy < 2; ++dy) {
                const int cy = iyr - dy;
                if (cy < 0 || cy > ny - 2 || !(gy[cy] <= y && y <= gy[cy + 1])) continue;
                const long long e = cell[(long long)cy * (nx - 1) + cx];
                if (e >= 0 && (best < 0 || e < best)) best = e;
            }
        }
        elts[p] = best;
    }
}

// ---------------------------------------------------------------------------
// Frame layout straight from the ROI mask on a tensor-grid mesh
// ---------------------------------------------------------------------------
// The host path samples every pixel of the padded node bbox, keeps the ROI pixels, assigns each
// to the lowest-index element whose closed cell contains its centre, sorts by element (stable)
// and cuts element runs into chunks.  On a tensor grid every element is one axis-aligned cell,
// so the same layout is built element by element: one warp per element walks its cell's pixels
// in row-major order (the order a stable sort by element keeps), counts and places the ROI
// pixels it owns, and the chunk tables follow from the per-element counts.  Every integer
// table and every FP64 quantity (Newton coordinates, spring weights) uses the host operations
// in the same order, so the layout is identical to the host-built one.
struct GridGeo {
    const double *gx, *gy;         // grid lines (ascending)
    int nx, ny;
    const int *cell;               // (ny - 1) x (nx - 1): element of the cell (lowest index), -1 for none
    const int *elem_cell;          // per element: ix | iy << 16 of its cell
    const unsigned char *roi;      // H x W ROI mask, or null (every pixel)
    int H, W, i0, i1, j0, j1;      // image size and the padded node bbox [i0, i1) x [j0, j1)
};

// inclusive pixel rows / columns whose centres lie in the element's closed cell, inside the bbox
__device__ __forceinline__ void elem_rect(const GridGeo &G, int e, int &ix, int &iy, int &ca, int &cb, int &ra,
                                          int &rb) {
    const int ec = __ldg(G.elem_cell + e);
    ix = ec & 0xffff;
    iy = (int)((unsigned)ec >> 16);
    ca = max((int)ceil(G.gx[ix] - 0.5), G.j0);
    cb = min((int)floor(G.gx[ix + 1] - 0.5), G.j1 - 1);
    ra = max((int)ceil(G.gy[iy] - 0.5), G.i0);
    rb = min((int)floor(G.gy[iy + 1] - 0.5), G.i1 - 1);
}

// ROI pixel (r, c) of element e's cell that e owns: no lower-index element's closed cell holds its
// centre (only possible on a shared grid line)
__device__ __forceinline__ bool pix_owned(const GridGeo &G, int e, int ix, int iy, int r, int c) {
    if (G.roi && !G.roi[(size_t)r * G.W + c]) return false;
    const double x = c + 0.5, y = r + 0.5;
    const bool l = ix > 0 && x == G.gx[ix], rt = ix + 3 <= G.nx && x == G.gx[ix + 1];
    const bool t = iy > 0 && y == G.gy[iy], b = iy + 3 <= G.ny && y == G.gy[iy + 1];
    if (!(l || rt || t || b)) return true;
    for (int dy = -1; dy <= 1; ++dy) {
        if ((dy < 0 && !t) || (dy > 0 && !b)) continue;
        for (int dx = -1; dx <= 1; ++dx) {
            if ((dx < 0 && !l) || (dx > 0 && !rt)) continue;
            const int o = __ldg(G.cell + (size_t)(iy + dy) * (G.nx - 1) + ix + dx);
            if (o >= 0 && o < e) return false;
        }
    }
    return true;
}

// pass 1: owned ROI pixels per element (one warp per element)
__global__ void __launch_bounds__(256) grid_count(GridGeo G, int n_elem, int *__restrict__ count) {
    const int lane = threadIdx.x & 31;
    const int e = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (e >= n_elem) return;
    int ix, iy, ca, cb, ra, rb;
    elem_rect(G, e, ix, iy, ca, cb, ra, rb);
    int cnt = 0;
    for (int r = ra; r <= rb; ++r)
        for (int c0 = ca; c0 <= cb; c0 += 32) {
            const int c = c0 + lane;
            cnt += __popc(__ballot_sync(0xffffffffu, c <= cb && pix_owned(G, e, ix, iy, r, c)));
        }
    if (lane == 0) count[e] = cnt;
}

// chunk k of element-local rank q (len pixels cut into nch runs at (len k) / nch)
__device__ __forceinline__ int chunk_of_rank(int q, int len, int nch) {
    auto start = [&](int k) { return (int)(((long long)len * k) / nch); };
    int k = (int)(((long long)q * nch) / len);
    while (k + 1 < nch && start(k + 1) <= q) ++k;
    while (k > 0 && start(k) > q) --k;
    return k;
}

constexpr int GRID_MAX_CHUNKS = 32;   // chunks per element handled by pass 2

// pass 2: element-major pixel positions, chunk begins, nodes, elements and pixel boxes
__global__ void __launch_bounds__(256) grid_place(GridGeo G, int n_elem, const int *__restrict__ elem_off,
                                                  const int *__restrict__ elem_choff, const int *__restrict__ elements,
                                                  unsigned *__restrict__ rc_out, int *__restrict__ chunk_of,
                                                  int *__restrict__ chunk_begin, int *__restrict__ chunk_nodes,
                                                  int *__restrict__ chunk_elem, int *__restrict__ chunk_box,
                                                  int *__restrict__ err) {
    __shared__ int s_box[8][GRID_MAX_CHUNKS][4];   // per warp: min col, min row, max col, max row
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int e = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (e >= n_elem) return;
    const int off = elem_off[e], len = elem_off[e + 1] - off;
    const int choff = elem_choff[e], nch = elem_choff[e + 1] - choff;
    if (len == 0) return;
    if (nch > GRID_MAX_CHUNKS) {
        if (lane == 0) atomicExch(err, 1);
        return;
    }
    for (int k = lane; k < nch; k += 32) {
        s_box[w][k][0] = 0x7fffffff;
        s_box[w][k][1] = 0x7fffffff;
        s_box[w][k][2] = -1;
        s_box[w][k][3] = -1;
    }
    __syncwarp();
    int ix, iy, ca, cb, ra, rb;
    elem_rect(G, e, ix, iy, ca, cb, ra, rb);
    int base = 0;
    for (int r = ra; r <= rb; ++r)
        for (int c0 = ca; c0 <= cb; c0 += 32) {
            const int c = c0 + lane;
            const bool keep = c <= cb && pix_owned(G, e, ix, iy, r, c);
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int q = base + __popc(bal & ((1u << lane) - 1u));
                if (q < len) {
                    const int k = chunk_of_rank(q, len, nch);
                    rc_out[off + q] = (unsigned)c | ((unsigned)r << 16);
                    chunk_of[off + q] = choff + k;
                    atomicMin(&s_box[w][k][0], c);
                    atomicMin(&s_box[w][k][1], r);
                    atomicMax(&s_box[w][k][2], c);
                    atomicMax(&s_box[w][k][3], r);
                } else {
                    atomicExch(err, 2);   // the count of pass 1 does not hold (cannot happen)
                }
            }
            base += __popc(bal);
        }
    __syncwarp();
    // the end of the element's last chunk: the next element's first begin (the same value) or, for
    // the last element with pixels, n_pix
    if (lane == 0) chunk_begin[choff + nch] = off + len;
    for (int k = lane; k < nch; k += 32) {
        const int ci = choff + k;
        chunk_begin[ci] = off + (int)(((long long)len * k) / nch);
        chunk_elem[ci] = e;
#pragma unroll
        for (int a = 0; a < 4; ++a) chunk_nodes[4 * ci + a] = __ldg(elements + 4 * e + a);
        chunk_box[2 * ci] = (int)((unsigned)s_box[w][k][0] | ((unsigned)s_box[w][k][1] << 16));
        chunk_box[2 * ci + 1] = (int)((unsigned)s_box[w][k][2] | ((unsigned)s_box[w][k][3] << 16));
    }
}

// pass 3: the 16-byte pixel records, with the row pairing inside full 16-column chunks (cubic)
template <int KIND>
__global__ void __launch_bounds__(256) grid_records(long long n_pix, const unsigned *__restrict__ rc,
                                                    const int *__restrict__ chunk_of,
                                                    const int *__restrict__ chunk_begin,
                                                    const int *__restrict__ chunk_box, const int *__restrict__ chunk_nodes,
                                                    const double *__restrict__ nodes, int iters, Img ref,
                                                    uint4 *__restrict__ pix) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n_pix) return;
    const unsigned v = rc[p];
    const int col = (int)(v & 0xffffu), row = (int)(v >> 16);
    const int c = chunk_of[p];
    long long dest = p;
    if (KIND == D2IC_INTERP_CUBIC) {
        const unsigned b0 = (unsigned)chunk_box[2 * c], b1 = (unsigned)chunk_box[2 * c + 1];
        const int bx0 = (int)(b0 & 0xffffu), by0 = (int)(b0 >> 16);
        const int w = (int)(b1 & 0xffffu) - bx0 + 1, h = (int)(b1 >> 16) - by0 + 1;
        const int cb = chunk_begin[c], len = chunk_begin[c + 1] - cb;
        if (w == 16 && h % 8 == 0 && len == 16 * h) {
            const int rr = row - by0, cc = col - bx0;
            dest = cb + 32 * ((rr & 3) + ((rr >> 3) << 2)) + 16 * ((rr >> 2) & 1) + cc;
        }
    }
    double X[4], Y[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int n = __ldg(chunk_nodes + 4 * c + a);
        X[a] = nodes[2 * (size_t)n];
        Y[a] = nodes[2 * (size_t)n + 1];
    }
    double xi, eta;
    newton_local(X, Y, col + 0.5, row + 0.5, iters, xi, eta);
    float a, b;
    const float I1 = sample<KIND>(ref, col, row, 0.f, 0.f, a, b);
    pix[dest] = make_uint4(v, __float_as_uint(I1), __float_as_uint((float)xi), __float_as_uint((float)eta));
}

// the elements (cells) around grid node n = iy nx + ix
__device__ __forceinline__ int node_cells(const GridGeo &G, int n, int cells[4]) {
    const int ix = n % G.nx, iy = n / G.nx;
    int m = 0;
    for (int dy = -1; dy <= 0; ++dy)
        for (int dx = -1; dx <= 0; ++dx) {
            const int cx = ix + dx, cy = iy + dy;
            if (cx < 0 || cy < 0 || cx > G.nx - 2 || cy > G.ny - 2) continue;
            const int e = __ldg(G.cell + (size_t)cy * (G.nx - 1) + cx);
            if (e >= 0) cells[m++] = e;
        }
    return m;
}

// pass 4: per chunk, its rank among the chunks of each of its nodes (ascending chunk order) and
// its count into the node groups it touches
__global__ void __launch_bounds__(256) grid_chunk_meta(GridGeo G, int n_chunks, const int *__restrict__ chunk_elem,
                                                       const int *__restrict__ chunk_nodes,
                                                       const int *__restrict__ elem_choff, int *__restrict__ chunk_slot,
                                                       int *__restrict__ group_need) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_chunks) return;
    const int e = chunk_elem[c];
    const int k = c - elem_choff[e];
    unsigned slot = 0;
    int g[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int n = chunk_nodes[4 * c + a];
        int cells[4];
        const int m = node_cells(G, n, cells);
        int rank = k;
        for (int i = 0; i < m; ++i)
            if (cells[i] < e) rank += elem_choff[cells[i] + 1] - elem_choff[cells[i]];
        slot |= (unsigned)(rank & 0xff) << (8 * a);
        g[a] = n / D2IC_NODE_GROUP;
    }
    chunk_slot[c] = (int)slot;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        bool first = true;
        for (int b = 0; b < a; ++b) first = first && g[b] != g[a];
        if (first) atomicAdd(group_need + g[a], 1);
    }
}

// the sorted distinct nodes sharing an element with node n (the host's lexsorted unique directed
// element edges); returns the count (at most 8 on a grid)
__device__ __forceinline__ int node_neighbours(const GridGeo &G, const int *elements, int n, int nb[8]) {
    int cells[4];
    const int m = node_cells(G, n, cells);
    int cnt = 0;
    for (int i = 0; i < m; ++i)
        for (int a = 0; a < 4; ++a) {
            const int j = __ldg(elements + 4 * cells[i] + a);
            if (j == n) continue;
            bool seen = false;
            for (int q = 0; q < cnt; ++q) seen = seen || nb[q] == j;
            if (!seen && cnt < 8) nb[cnt++] = j;
        }
    for (int i = 1; i < cnt; ++i) {                 // insertion sort, ascending
        const int v = nb[i];
        int q = i - 1;
        while (q >= 0 && nb[q] > v) {
            nb[q + 1] = nb[q];
            --q;
        }
        nb[q + 1] = v;
    }
    return cnt;
}

// pass 5: per node, chunks meeting at it (-> node_chunk_k) and spring degree (-> max_deg)
__global__ void __launch_bounds__(256) grid_node_stats(GridGeo G, int n_nodes, const int *__restrict__ elements,
                                                       const int *__restrict__ elem_choff, int *__restrict__ stats) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= n_nodes) return;
    int cells[4];
    const int m = node_cells(G, n, cells);
    int kc = 0;
    for (int i = 0; i < m; ++i) kc += elem_choff[cells[i] + 1] - elem_choff[cells[i]];
    int nb[8];
    const int deg = node_neighbours(G, elements, n, nb);
    atomicMax(stats + 0, kc);
    atomicMax(stats + 1, deg);
}

// pass 6: spring tables (max_deg x n_nodes, column-major): neighbour, and the weight
// float32(1 / (|x_j - x_i| + 1e-6)) * 0.5 * (rho_i + rho_j) in float32
__global__ void __launch_bounds__(256) grid_springs(GridGeo G, int n_nodes, const int *__restrict__ elements,
                                                    const double *__restrict__ nodes, const float *__restrict__ rho,
                                                    int max_deg, int *__restrict__ nbr_index,
                                                    float *__restrict__ nbr_weight) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= n_nodes) return;
    int nb[8];
    const int deg = node_neighbours(G, elements, n, nb);
    const double xi = nodes[2 * (size_t)n], yi = nodes[2 * (size_t)n + 1];
    for (int q = 0; q < max_deg; ++q) {
        int j = -1;
        float wc = 0.f;
        if (q < deg) {
            j = nb[q];
            const double dx = __dsub_rn(nodes[2 * (size_t)j], xi), dy = __dsub_rn(nodes[2 * (size_t)j + 1], yi);
            const double nrm = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
            const float w = (float)__ddiv_rn(1.0, __dadd_rn(nrm, 1e-6));
            wc = __fmul_rn(__fmul_rn(w, 0.5f), __fadd_rn(rho[n], rho[j]));
        }
        nbr_index[(size_t)q * n_nodes + n] = j;
        nbr_weight[(size_t)q * n_nodes + n] = wc;
    }
}

}  // namespace d2ic

using namespace d2ic;

extern "C" int d2ic_structured_assign(const double *pixel_coords, long long n_pix, const double *gx, int nx,
                                      const double *gy, int ny, const long long *cell, long long *elts,
                                      void *stream) {
    D2IC_REQUIRE(n_pix >= 0 && nx >= 2 && ny >= 2, "d2ic_structured_assign: bad sizes");
    if (n_pix == 0) return D2IC_OK;
    D2IC_REQUIRE(pixel_coords && gx && gy && cell && elts, "d2ic_structured_assign: null pointer");
    long long blocks = (n_pix + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    structured_assign_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(pixel_coords, n_pix, gx, nx, gy, ny, cell,
                                                                            elts);
    D2IC_CHECK_LAUNCH("structured_assign_kernel");
    return D2IC_OK;
}

extern "C" int d2ic_local_coordinates(const double *pixel_coords, const int *pixel_nodes, const double *nodes,
                                      long long n_pix, int iters, double *xi, double *eta, void *stream) {
    D2IC_REQUIRE(n_pix >= 0 && iters >= 0, "d2ic_local_coordinates: bad sizes");
    if (n_pix == 0) return D2IC_OK;
    D2IC_REQUIRE(pixel_coords && pixel_nodes && nodes && xi && eta, "d2ic_local_coordinates: null pointer");
    long long blocks = (n_pix + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    local_coords_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(pixel_coords, pixel_nodes, nodes, n_pix, iters,
                                                                       xi, eta);
    D2IC_CHECK_LAUNCH("local_coords_kernel");
    return D2IC_OK;
}

// ---- frame layout from the ROI mask on a tensor-grid mesh ----

static GridGeo grid_geo(const d2ic_grid_t *g) {
    GridGeo G;
    G.gx = g->gx;
    G.gy = g->gy;
    G.nx = g->nx;
    G.ny = g->ny;
    G.cell = g->cell;
    G.elem_cell = g->elem_cell;
    G.roi = g->roi;
    G.H = g->H;
    G.W = g->W;
    G.i0 = g->i0;
    G.i1 = g->i1;
    G.j0 = g->j0;
    G.j1 = g->j1;
    return G;
}

static int grid_check(const d2ic_grid_t *g, const char *name) {
    D2IC_REQUIRE(g && g->gx && g->gy && g->cell && g->elem_cell && g->elements && g->nodes, "%s: null pointer", name);
    D2IC_REQUIRE(g->nx >= 2 && g->ny >= 2 && g->nx < 65536 && g->ny < 65536 && g->n_elem >= 0 && g->H > 0 &&
                     g->W > 0 && g->H < 65536 && g->W < 65536 && g->n_nodes == g->nx * g->ny,
                 "%s: bad grid sizes", name);
    D2IC_REQUIRE(0 <= g->i0 && g->i0 <= g->i1 && g->i1 <= g->H && 0 <= g->j0 && g->j0 <= g->j1 && g->j1 <= g->W,
                 "%s: bad pixel box", name);
    return D2IC_OK;
}

extern "C" int d2ic_grid_count(const d2ic_grid_t *grid, int *elem_count, void *stream) {
    int st = grid_check(grid, "d2ic_grid_count");
    if (st) return st;
    D2IC_REQUIRE(elem_count, "d2ic_grid_count: null pointer");
    if (grid->n_elem == 0) return D2IC_OK;
    grid_count<<<(unsigned)((32 * (size_t)grid->n_elem + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        grid_geo(grid), grid->n_elem, elem_count);
    D2IC_CHECK_LAUNCH("grid_count");
    return D2IC_OK;
}

extern "C" size_t d2ic_grid_scratch_bytes(long long n_pix, int n_chunks) {
    const size_t np = (size_t)(n_pix > 0 ? n_pix : 1), nc = (size_t)(n_chunks > 0 ? n_chunks : 1);
    return ((4 * np + 255) & ~(size_t)255) * 2 + ((4 * nc + 255) & ~(size_t)255);
}

extern "C" int d2ic_grid_layout(const d2ic_grid_t *grid, const int *elem_off, const int *elem_choff, long long n_pix,
                                int n_chunks, int kind, const float *ref_coeff, int cpitch, int pad, void *scratch,
                                size_t scratch_bytes, d2ic_pixrec_t *pix, int *chunk_begin, int *chunk_nodes,
                                int *chunk_box, int *chunk_slot, int *group_need, int *stats, void *stream) {
    int st = grid_check(grid, "d2ic_grid_layout");
    if (st) return st;
    D2IC_REQUIRE(elem_off && elem_choff && ref_coeff && scratch && chunk_begin && chunk_nodes && chunk_box &&
                     chunk_slot && group_need && stats && (pix || n_pix == 0) && n_pix >= 0 && n_chunks >= 0,
                 "d2ic_grid_layout: bad arguments");
    D2IC_REQUIRE(kind == D2IC_INTERP_CUBIC || kind == D2IC_INTERP_LINEAR, "d2ic_grid_layout: unknown kind %d", kind);
    D2IC_REQUIRE(scratch_bytes >= d2ic_grid_scratch_bytes(n_pix, n_chunks), "d2ic_grid_layout: scratch too small");
    D2IC_REQUIRE(((uintptr_t)scratch & 255) == 0, "d2ic_grid_layout: scratch must be 256-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    const GridGeo G = grid_geo(grid);
    char *sp = (char *)scratch;
    auto take = [&](size_t bytes) {
        char *p = sp;
        sp += (bytes + 255) & ~(size_t)255;
        return p;
    };
    unsigned *rc = (unsigned *)take(sizeof(unsigned) * (size_t)(n_pix > 0 ? n_pix : 1));
    int *chunk_of = (int *)take(sizeof(int) * (size_t)(n_pix > 0 ? n_pix : 1));
    int *chunk_elem = (int *)take(sizeof(int) * (size_t)(n_chunks > 0 ? n_chunks : 1));
    const int ng = (grid->n_nodes + D2IC_NODE_GROUP - 1) / D2IC_NODE_GROUP;
    cudaError_t e = cudaMemsetAsync(group_need, 0, sizeof(int) * (size_t)ng, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(stats, 0, sizeof(int) * 4, s);
    if (e != cudaSuccess) return cuda_status(e, "d2ic_grid_layout: clear");
    if (grid->n_elem > 0) {
        grid_place<<<(unsigned)((32 * (size_t)grid->n_elem + 255) / 256), 256, 0, s>>>(
            G, grid->n_elem, elem_off, elem_choff, grid->elements, rc, chunk_of, chunk_begin, chunk_nodes, chunk_elem,
            chunk_box, stats + 2);
        D2IC_CHECK_LAUNCH("grid_place");
    }
    if (n_pix > 0) {
        const Img ref{ref_coeff, grid->W, grid->H, cpitch, pad};
        const unsigned nb = (unsigned)((n_pix + 255) / 256);
        if (kind == D2IC_INTERP_CUBIC)
            grid_records<D2IC_INTERP_CUBIC><<<nb, 256, 0, s>>>(n_pix, rc, chunk_of, chunk_begin, chunk_box, chunk_nodes,
                                                               grid->nodes, 10, ref, (uint4 *)pix);
        else
            grid_records<D2IC_INTERP_LINEAR><<<nb, 256, 0, s>>>(n_pix, rc, chunk_of, chunk_begin, chunk_box,
                                                                chunk_nodes, grid->nodes, 10, ref, (uint4 *)pix);
        D2IC_CHECK_LAUNCH("grid_records");
    }
    if (n_chunks > 0) {
        grid_chunk_meta<<<(unsigned)((n_chunks + 255) / 256), 256, 0, s>>>(G, n_chunks, chunk_elem, chunk_nodes,
                                                                           elem_choff, chunk_slot, group_need);
        D2IC_CHECK_LAUNCH("grid_chunk_meta");
    }
    grid_node_stats<<<(unsigned)((grid->n_nodes + 255) / 256), 256, 0, s>>>(G, grid->n_nodes, grid->elements,
                                                                            elem_choff, stats);
    D2IC_CHECK_LAUNCH("grid_node_stats");
    return D2IC_OK;
}

extern "C" int d2ic_grid_springs(const d2ic_grid_t *grid, const float *rho, int max_deg, int *nbr_index,
                                 float *nbr_weight, void *stream) {
    int st = grid_check(grid, "d2ic_grid_springs");
    if (st) return st;
    D2IC_REQUIRE(rho && nbr_index && nbr_weight && max_deg >= 0 && max_deg <= 8, "d2ic_grid_springs: bad arguments");
    if (max_deg == 0) return D2IC_OK;
    grid_springs<<<(unsigned)((grid->n_nodes + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        grid_geo(grid), grid->n_nodes, grid->elements, grid->nodes, rho, max_deg, nbr_index, nbr_weight);
    D2IC_CHECK_LAUNCH("grid_springs");
    return D2IC_OK;
}
