/*
 * d2ic_gb300 — C ABI of the GB300 (sm_103a) global finite-element DIC hot path.
 *
 * Plain C: pointers, sizes and a CUDA stream handle passed as `void *`
 * (a cudaStream_t; NULL = legacy default stream).  Every device pointer is
 * borrowed for the duration of the call; the library never frees caller
 * memory.  Functions return D2IC_OK (0) or a negative status; the message of
 * the last failure on the calling thread is d2ic_last_error_string().
 * Nothing here throws across the ABI.
 *
 * The entry points replace the reference's JAX kernels behind the solver
 * plugin interface `SolverBase.compile/solve` (d2ic/solver_base.py:8-26).
 * Each declaration names the reference code it replaces.
 */
#ifndef D2IC_GB300_H
#define D2IC_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define D2IC_API __attribute__((visibility("default")))
#else
#define D2IC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define D2IC_OK             0
#define D2IC_BAD_ARG       -1   /* maps to ValueError on the Python side      */
#define D2IC_OOM           -2
#define D2IC_NAN_DETECTED  -3   /* reported in per-frame status, not raised   */
#define D2IC_MAX_ITERS     -4   /* reported in per-frame status, not raised   */
#define D2IC_WAIT_TIMEOUT  -5   /* a bounded device-side wait gave up         */
#define D2IC_CUDA_ERROR    -6
#define D2IC_UNSUPPORTED   -7
#define D2IC_INTERNAL      -8   /* an engine self-check failed (an index outside its table) */
#define D2IC_RUNNING        1   /* per-frame status: not finished at the end of a slice */

/* interpolation kinds (GlobalCGSolver(interpolation=...)) */
#define D2IC_INTERP_CUBIC   0   /* cubic B-spline, edge-replicating boundary  */
#define D2IC_INTERP_LINEAR  1   /* bilinear, edge clamped                     */

/* sizes of the engine's fixed-shape pieces */
#define D2IC_NODE_GROUP    32   /* nodes per reduction group (one warp)       */
#define D2IC_NPART          5   /* double-float pairs per group partial       */
#define D2IC_MAX_FRAMES  4096   /* frames per batched launch                  */
#define D2IC_CHUNK_MAX    256   /* pixels per chunk (one element per chunk)   */
#define D2IC_TILE_MAX_FLOATS 736 /* largest staged coefficient tile (w x h)  */

/* One pixel of the element-major pixel list: 16 bytes, read with one 128-bit load. */
typedef struct d2ic_pixrec {
    uint32_t pos;     /* column | (row << 16) of the pixel                     */
    float    I1;      /* reference-image sample at the pixel centre            */
    float    xi;      /* local element coordinates of the pixel centre         */
    float    eta;
} d2ic_pixrec_t;

/*
 * Everything one frame's solve reads and writes.  All pointers are device
 * pointers.  The workspace fields are set by d2ic_frame_bind_workspace().
 */
typedef struct d2ic_frame {
    /* TMA tensor map (a CUtensorMap, 128 bytes) of `coeff`, written by
     * d2ic_frame_encode_tiles(); it is read by the kernels from the device copy
     * of the descriptor, which must therefore be 64-byte aligned (sizeof is a
     * multiple of 64, so every element of a 64-byte aligned array is) */
    uint64_t     coeff_map[16];
    /* deformed image: B-spline coefficients (cubic) or the image itself (linear),
     * with a `pad`-wide halo; pixel (i,j) lives at coeff[(i+pad)*cpitch + j+pad] */
    const float *coeff;
    /* element-major pixel list, cut into chunks of <= D2IC_CHUNK_MAX pixels of one element */
    const d2ic_pixrec_t *pix;
    const int   *chunk_begin;      /* n_chunks + 1                                      */
    const int   *chunk_nodes;      /* 4 * n_chunks, the chunk's element nodes (Q4 order) */
    const int   *chunk_box;        /* 2 * n_chunks: (col0 | row0 << 16, col1 | row1 << 16),
                                      inclusive pixel box of the chunk                  */
    const int   *chunk_slot;       /* n_chunks: byte a = rank of the chunk among the chunks
                                      of its local node a (ascending chunk order), i.e.
                                      the node_grad slot the chunk's partial goes to     */
    const int   *group_need;       /* n_groups: chunks with a node in group g (nodes
                                      D2IC_NODE_GROUP*g ... +D2IC_NODE_GROUP-1)          */
    const int   *nbr_index;        /* max_deg * n_nodes spring neighbours, column-major,
                                      -1 padded after the last neighbour                */
    const float *nbr_weight;       /* same layout: w_ij * (rho_i + rho_j) / 2           */
    const float *u0;               /* 2 * n_nodes initial displacement                  */
    float       *u_out;            /* 2 * n_nodes solution                              */
    float       *hist;             /* 3 * max_iter CG history [J, |g|, alpha], NaN-filled */
    int         *n_iters;          /* 1: iterations taken                               */
    int         *status;           /* 1: D2IC_OK / D2IC_NAN_DETECTED / D2IC_MAX_ITERS   */
    int         *n_evals;          /* 1: objective evaluations (pixel passes) performed */
    /* workspace */
    float       *node_ws;          /* 14 * n_nodes floats                               */
    float       *node_grad;        /* 4 * node_chunk_k * n_nodes: per-node slots of the
                                      chunks' partials (gx, gy, and for the chunk's node 0
                                      its sum of r^2 as a double-float hi, lo), column-major
                                      (slot k of node n at k * n_nodes + n), unused slots 0 */
    float       *group_part;       /* 2 * D2IC_NPART * (n_groups + n_super) double-float
                                      partials of the groups, then of the supergroups of
                                      16 groups (n_super = ceil(n_groups / 16))          */
    int         *group_cnt;        /* n_groups + n_super + 1 completion counters (all 0
                                      between rounds)                                   */
    int         *chunk_tile;       /* n_chunks: origin (col | row << 16, int16 each) of the
                                      chunk's coefficient tile for the next pass        */
    double       tol;
    float        alpha_reg;
    int          max_iter;
    int          W, H, cpitch, pad;
    int          n_pix, n_chunks, n_nodes, max_deg;
    int          n_groups;         /* set by d2ic_frame_bind_workspace                  */
    int          node_chunk_k;
    int          tile_w, tile_h;   /* staged coefficient tile (0 = taps read from global
                                      memory); set by d2ic_frame_encode_tiles()         */
    int          reserved_[8];
} d2ic_frame_t;

/* ---- library ------------------------------------------------------------- */
D2IC_API const char *d2ic_last_error_string(void);
D2IC_API int d2ic_version(void);
/* sizeof(d2ic_frame_t), for bindings that mirror the descriptor to check their layout. */
D2IC_API size_t d2ic_frame_descriptor_bytes(void);
/* SM count and the persistent engine's resident blocks per SM on `device`. */
D2IC_API int d2ic_device_info(int device, int *num_sms, int *engine_blocks_per_sm);

/* ---- image preparation (replaces the per-call sampling setup inside
 *      im_jax.flat_nd_cubic_interpolate, d2ic/solver_global_cg.py:512-518) ---- */

/* Cubic B-spline coefficients of an HxW float image extended by edge
 * replication, written with a `pad`-wide halo into coeff ((H+2pad) x cpitch).
 * tmp: H x cpitch floats of scratch.  pad >= 16, cpitch >= W + 2 pad. */
D2IC_API int d2ic_bspline_prefilter(const float *img, int H, int W, int pad, int cpitch,
                           float *tmp, float *coeff, void *stream);
/* The same for n_images contiguous HxW images in one launch: image i's scratch at
 * tmp + i H cpitch and its coefficients at coeff + i (H + 2 pad) cpitch. */
D2IC_API int d2ic_bspline_prefilter_batch(const float *img, int n_images, int H, int W, int pad, int cpitch,
                                          float *tmp, float *coeff, void *stream);

/* Copy an image into the halo layout with edge replication (linear kind). */
D2IC_API int d2ic_pad_image(const float *img, int H, int W, int pad, int cpitch, float *out, void *stream);

/* The same two preparations for 8-bit camera frames (GlobalCGSolver.solve takes the frame as given,
 * jnp.asarray(def_image), d2ic/solver_global_cg.py:157-159): the pixels are read as uint8 and
 * widened on the device, so a frame crosses the host link at one byte per pixel. */
D2IC_API int d2ic_bspline_prefilter_u8(const unsigned char *img, int H, int W, int pad, int cpitch,
                                       float *tmp, float *coeff, void *stream);
D2IC_API int d2ic_pad_image_u8(const unsigned char *img, int H, int W, int pad, int cpitch, float *out,
                               void *stream);


/* Sample n points at image-index coordinates xy (x = col, y = row, i.e. the
 * reference's pixel-centre coordinates minus 0.5); value and d/dx, d/dy.
 * Replaces _cubic_sample / _bilinear_sample (d2ic/solver_global_cg.py:481-518). */
D2IC_API int d2ic_sample_points(const float *coeff, int H, int W, int pad, int cpitch, int kind,
                       const float *xy, int n, float *val, float *gx, float *gy, void *stream);

/* Build the 16-byte pixel records: pos from (col,row) pairs, I1 sampled from
 * the reference-image coefficients at the pixel centre, (xi,eta) copied. */
D2IC_API int d2ic_pack_pixels(const int *colrow, const float *xieta, int n,
                     const float *coeff1, int H, int W, int pad, int cpitch, int kind,
                     d2ic_pixrec_t *out, void *stream);

/* ---- adjoint linear solves: block-Jacobi PCG on the exact Hessian, K right-hand sides ---- */

/* Bytes of device scratch d2ic_pcg_solve needs (256-byte aligned base). */
D2IC_API size_t d2ic_pcg_work_bytes(int n_nodes, int K, int node_chunk_k);

/* X = H^-1 B for B, X (n_nodes, 2, K) FP64 (column index fastest), H assembled from chunk_hess
 * into the work buffer (as d2ic_hessian_assemble) and applied in FP32, Minv (n_nodes, 2, 2) FP64
 * inverse diagonal blocks (zero for inactive dofs), active (n_nodes) 0/1 mask.  Stops when every
 * column has ||R|| <= rtol ||B|| or after max_iter iterations (*iters_out); convergence is decided
 * on the device and read by the host once per batch of 8 iterations. */
D2IC_API int d2ic_pcg_solve(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                            const float *chunk_hess, float inv_np, float alpha_reg, const double *Minv,
                            const unsigned char *active, const double *B, double *X, int K, double rtol,
                            int max_iter, void *work, size_t work_bytes, int *iters_out, void *stream);

/* ---- pixel-asset setup (replaces the Newton inverse map of build_pixel_assets,
 *      d2ic/pixel_assets.py:240-294) ---- */

/* (xi, eta) of each pixel in its Q4 element by at most `iters` Newton steps from
 * (0, 0), FP64 with correctly rounded operations in the host restatement's order
 * (bit-identical results).  pixel_coords: 2 * n_pix; pixel_nodes: 4 * n_pix
 * node indices; nodes: 2 * n_nodes; xi, eta: n_pix each.  Device pointers. */
D2IC_API int d2ic_local_coordinates(const double *pixel_coords, const int *pixel_nodes, const double *nodes,
                                    long long n_pix, int iters, double *xi, double *eta, void *stream);

/* Element of each pixel on a tensor-grid mesh of axis-aligned cells (the
 * pixel-to-element map of build_pixel_assets, d2ic/pixel_assets.py:135-237, for
 * the grids mask_to_mesh builds): the lowest element index whose closed cell
 * rectangle contains the pixel centre, -1 if none.  pixel_coords: 2 * n_pix (x, y);
 * gx: nx ascending grid columns; gy: ny ascending grid rows; cell: (ny - 1) *
 * (nx - 1) element index per cell, row-major, -1 for no element; elts: n_pix.
 * FP64 comparisons only, so the result equals the host search exactly.  Device
 * pointers. */
D2IC_API int d2ic_structured_assign(const double *pixel_coords, long long n_pix, const double *gx, int nx,
                                    const double *gy, int ny, const long long *cell, long long *elts, void *stream);

/* ---- frame layout built on the device from the ROI mask, for the tensor-grid meshes of
 *      mask_to_mesh (replaces build_pixel_assets, d2ic/pixel_assets.py:21-131,135-294,330-409, and the
 *      host layout of the engine: the same pixels, element map, Newton coordinates, chunks, node slots
 *      and spring tables, bit for bit) ---- */
typedef struct d2ic_grid {
    const double *gx, *gy;          /* nx, ny grid lines, ascending (device)                       */
    int nx, ny;
    const int *cell;                /* (ny - 1) x (nx - 1): element of the cell, -1 for none (device) */
    const int *elem_cell;           /* n_elem: ix | iy << 16, the element's cell (device)            */
    const int *elements;            /* n_elem x 4 nodes, Q4 order (device)                           */
    const double *nodes;            /* n_nodes x 2 coordinates, node iy * nx + ix (device)           */
    const unsigned char *roi;       /* H x W ROI mask (device), NULL for every pixel                 */
    int n_elem, n_nodes, H, W;
    int i0, i1, j0, j1;             /* the padded node bbox [i0, i1) x [j0, j1) of the host sampler  */
} d2ic_grid_t;

/* Pass 1: the ROI pixels each element owns (lowest element index whose closed cell holds the pixel
 * centre).  grid: HOST pointer to the descriptor; elem_count: n_elem ints (device). */
D2IC_API int d2ic_grid_count(const d2ic_grid_t *grid, int *elem_count, void *stream);
/* Bytes of scratch d2ic_grid_layout needs. */
D2IC_API size_t d2ic_grid_scratch_bytes(long long n_pix, int n_chunks);
/* Pass 2: the layout.  elem_off (n_elem + 1) pixel offsets and elem_choff (n_elem + 1) chunk offsets
 * are the exclusive prefix sums of the counts and of ceil(count / chunk_max) (device).  Writes the
 * pixel records, chunk_begin (n_chunks + 1), chunk_nodes, chunk_box, chunk_slot, group_need
 * (ceil(n_nodes / 32)) and stats[4] = {most chunks at one node, largest spring degree, error, 0};
 * error != 0 when an element has more than 32 chunks. */
D2IC_API int d2ic_grid_layout(const d2ic_grid_t *grid, const int *elem_off, const int *elem_choff, long long n_pix,
                              int n_chunks, int kind, const float *ref_coeff, int cpitch, int pad, void *scratch,
                              size_t scratch_bytes, d2ic_pixrec_t *pix, int *chunk_begin, int *chunk_nodes,
                              int *chunk_box, int *chunk_slot, int *group_need, int *stats, void *stream);
/* Pass 3: spring tables (max_deg x n_nodes, column-major, -1 / 0 padded) with rho: n_nodes node
 * regularisation weights (device). */
D2IC_API int d2ic_grid_springs(const d2ic_grid_t *grid, const float *rho, int max_deg, int *nbr_index,
                               float *nbr_weight, void *stream);

/* ---- local Gauss-Newton refinement (replaces LocalGaussNewtonSolver,
 *      d2ic/solver_local_gn.py:34-414) ---- */

/* Central-difference gradient images of an HxW image, zero on the first/last
 * column (gx) and row (gy) (_compute_image_gradient_jax, :204-210). */
D2IC_API int d2ic_central_gradient(const float *img, int H, int W, float *gx, float *gy, void *stream);

/* Bytes of the per-node slot scratch of one sweep (zero it once; unused slots must stay 0). */
D2IC_API size_t d2ic_local_gn_slot_bytes(int n_nodes, int node_chunk_k);

/* One Jacobi sweep u -> u_next (_local_sweeps body, :283-313; jacobi_nodal_step_spring,
 * :316-414): frame_dev carries the deformed image's sampling array (coeff) and the
 * pixel/chunk layout; coeff_gx/coeff_gy the gradient images' sampling arrays in the
 * same layout; has_pix: 1 for nodes with pixels; nbr_index/nbr_weight: raw spring
 * table (max_deg x n_nodes, column-major, -1 after the last neighbour);
 * node_reg_weight: rho_i.  chunk_r2 (n_chunks doubles) and step_part (one double
 * per 256 nodes) receive the sums for the sweep's RMS history. */
D2IC_API int d2ic_local_gn_sweep(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                                 int interp_kind, const float *coeff_gx, const float *coeff_gy, const float *u,
                                 float *slots, double *chunk_r2, const int *has_pix, const int *nbr_index,
                                 const float *nbr_weight, int max_deg, const float *node_reg_weight, float lam,
                                 float max_step, float alpha_reg, float omega, float *u_next, double *step_part,
                                 void *stream);

/* ---- result maps (replaces compute_discrepancy_map_ref, d2ic/discrepancy.py:86-127) ---- */

/* Bilinear grey-level residual I_def(x + u(x)) - I_ref(x) at every ROI pixel of
 * the frame's pixel list, written at (row, col) of the HxW `map` (NaN elsewhere
 * and where the bilinear stencil leaves the image), with per-chunk FP64 sums of
 * r^2 and valid counts for the RMS.  frame_dev: device descriptor (pix,
 * chunk_begin, chunk_nodes, n_chunks, W, H); ref, def: HxW images; u: 2 * n_nodes. */
D2IC_API int d2ic_discrepancy_map(const d2ic_frame_t *frame_dev, int n_chunks, const float *ref, const float *def,
                                  const float *u, int H, int W, float *map, double *chunk_sums, int *chunk_counts,
                                  void *stream);

/* ---- global CG engine (replaces _cg_solve / _J_TOTAL_VG / J_total,
 *      d2ic/solver_global_cg.py:289-469, behind GlobalCGSolver.solve :151-198) ---- */

/* Bytes of per-frame workspace, and binding of a workspace block to a frame
 * descriptor (host-side; `ws` is a device pointer aligned to 256 bytes). */
D2IC_API size_t d2ic_frame_workspace_bytes(int n_nodes, int n_chunks, int node_chunk_k);
D2IC_API int d2ic_frame_bind_workspace(d2ic_frame_t *frame, void *ws);

/* Stage each chunk's window of the coefficient image in shared memory with a
 * 2-D TMA copy of tile_w x tile_h floats (tile_w a multiple of 4,
 * tile_w * tile_h <= D2IC_TILE_MAX_FLOATS, cubic frames only): encodes
 * frame->coeff_map for frame->coeff, W, H, cpitch and pad, which must be set.
 * tile_w = 0 turns staging off (taps read through L1).  Host-side.  Pixels
 * that fall outside their chunk's tile read global memory, with the same
 * arithmetic, so results do not depend on the tile shape.  Returns
 * D2IC_UNSUPPORTED (staging off) when the driver lacks tensor-map encoding. */
D2IC_API int d2ic_frame_encode_tiles(d2ic_frame_t *frame, int tile_w, int tile_h);

/* Bytes of launch-wide control scratch for a batched launch of n_frames. */
D2IC_API size_t d2ic_cg_control_bytes(int n_frames);

/* Solve n_frames independent frames in ONE persistent cooperative launch.
 * frames: device array of n_frames descriptors.  control: device scratch of
 * d2ic_cg_control_bytes(n_frames) bytes (the call clears it on `stream`).
 * grid_blocks: 0 = all resident blocks.  Per-frame results land in each
 * descriptor's u_out / hist / n_iters / status. */
D2IC_API int d2ic_cg_solve_batched(const d2ic_frame_t *frames, int n_frames, void *control,
                          size_t control_bytes, int interp_kind, int grid_blocks, void *stream);

/* Continuous batching: run at most max_rounds objective evaluations ("rounds")
 * of the frames in `frames`, keeping every frame's CG state in `control`
 * between calls.  Before a call the host sets one command word per frame at
 * control + d2ic_cg_command_offset(): D2IC_CMD_INIT admits a new frame (u0,
 * image coefficients and outputs must be ready), D2IC_CMD_RUN continues (or
 * leaves finished frames alone), D2IC_CMD_IDLE parks an empty slot, D2IC_CMD_HOLD
 * keeps an admitted frame's state but leaves it out of this call (set it only
 * after the call that consumed the frame's D2IC_CMD_INIT; the frame reports
 * D2IC_RUNNING and continues where it stopped under D2IC_CMD_RUN).  A frame
 * that finishes during the call gets its outputs and final status written;
 * unfinished frames report D2IC_RUNNING.  Serves the batched/served form of
 * GlobalCGSolver.solve (d2ic/solver_global_cg.py:151-198) for many frames. */
#define D2IC_CMD_INIT 0
#define D2IC_CMD_RUN  1
#define D2IC_CMD_IDLE 2
#define D2IC_CMD_HOLD 3
D2IC_API size_t d2ic_cg_command_offset(void);
D2IC_API int d2ic_cg_slice(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes,
                           int interp_kind, int grid_blocks, int max_rounds, void *stream);

/* d2ic_cg_slice that may end before max_rounds: with D2IC_STOP_ON_FINISH after the first round in
 * which a frame finishes (its outputs are then written at once), with D2IC_STOP_ON_IRQ after a round
 * that ends while the 32-bit word at control + d2ic_cg_irq_offset() is non-zero.  The host writes that
 * word (a copy on another stream) while the slice runs, to admit new frames without waiting for the
 * slice; every launch clears it.  Lets a lightly loaded server run long slices. */
#define D2IC_STOP_ON_FINISH 1
#define D2IC_STOP_ON_IRQ    2
D2IC_API size_t d2ic_cg_irq_offset(void);
D2IC_API int d2ic_cg_slice_ex(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes,
                              int interp_kind, int grid_blocks, int max_rounds, int stop_flags, void *stream);


/* As d2ic_cg_solve_batched, and writes 6 %globaltimer stamps per round into
 * trace[6*r .. 6*r+5] for r < trace_rounds: block 0's round start, end of the
 * pixel-pass barrier and end of its node pass; start and end of the control
 * step (by the block that ran it); block 0's exit from the control barrier
 * (diagnostics; no counterpart in the reference). */
D2IC_API int d2ic_cg_solve_traced(const d2ic_frame_t *frames, int n_frames, void *control, size_t control_bytes,
                                  int interp_kind, int grid_blocks, unsigned long long *trace, int trace_rounds,
                                  void *stream);

/* Solve one frame without allocating any device memory: for callers that
 * cannot call cudaMalloc (a host runtime without a device allocator, a plugin
 * whose host owns all device memory).  `frame` is a HOST pointer; its inputs
 * and outputs are used as given and its workspace fields are ignored: the
 * descriptor copy, control block and CG workspace come from one fixed
 * file-scope device array of D2IC_NOALLOC_SCRATCH_BYTES, which every GPU that
 * loads the library holds until the process exits.  A frame needing more
 * (about (57.5 + 16 node_chunk_k) B per node + 4 B per chunk + under 4 KB of
 * descriptor, control block and alignment) is rejected with D2IC_BAD_ARG.
 * The descriptor is written into the array by a small kernel that receives it
 * as a launch argument, so `frame` may be reused or freed when the call returns.
 * The first call on a device looks up the array's device address (set-up), so
 * make it before any stream capture.  All calls share the one array and the
 * last call's contents stay in it: calls whose work overlaps on the GPU race.
 * No counterpart in the reference. */
#define D2IC_NOALLOC_SCRATCH_BYTES (32u << 20)
D2IC_API int d2ic_cg_solve_noalloc(const d2ic_frame_t *frame, int interp_kind, void *stream);

/* Objective and gradient at u for one frame (the value_and_grad of J_total,
 * d2ic/solver_global_cg.py:323).  frame: device pointer; control: as above for
 * one frame.  Writes J (1 double) and grad (2*n_nodes floats). */
D2IC_API int d2ic_eval_objective(const d2ic_frame_t *frame, const float *u, void *control, size_t control_bytes,
                        int interp_kind, double *J_out, float *grad_out, void *stream);

/* ---- implicit derivative of the converged solve (the hand-written replacement
 *      for jax.jvp through _cg_solve in doc/11_Advanced_Use_Uncertainty_Propagation.ipynb,
 *      cells 14/22/30).  frame_dev: the solved frame's descriptor (device); u: the
 *      converged displacement (2*n_nodes).  Vectors of K right-hand sides are laid
 *      out (node, component, k) with k fastest. ---- */

/* Per chunk, the 10 distinct 2x2 blocks (xx, xy, yy) of sum_p N_a N_b M_p with
 * M_p = grad I2 grad I2^T (+ r hess I2 when exact): 32 floats per chunk. */
D2IC_API int d2ic_hessian_chunks(const d2ic_frame_t *frame_dev, int n_chunks, const float *u, int exact,
                                 float *chunk_hess, void *stream);
/* Y = H V for K vectors: chunk blocks / Np + alpha_reg * spring Hessian.  slots:
 * node_chunk_k * n_nodes * 2 * K floats of scratch. */
D2IC_API int d2ic_hessian_matvec(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, const float *chunk_hess,
                                 const float *V, int K, float inv_np, float alpha_reg, float *slots, float *Y,
                                 void *stream);
/* The same operator assembled once per linearisation point: per node at most D2IC_HOP_MAX
 * (column node, symmetric 2x2 block) entries, chunk blocks / Np plus alpha_reg times the spring
 * Hessian, merged in slot order (no atomics).  op: device buffer of d2ic_hessian_op_bytes(), 256-byte
 * aligned.  Returns D2IC_BAD_ARG if a node couples to more than D2IC_HOP_MAX nodes (a Q4 grid node
 * couples to at most 9). */
#define D2IC_HOP_MAX 16
D2IC_API size_t d2ic_hessian_op_bytes(int n_nodes, int node_chunk_k);
D2IC_API int d2ic_hessian_assemble(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                                   const float *chunk_hess, float inv_np, float alpha_reg, void *op, size_t op_bytes,
                                   void *stream);
/* Y = H V with the assembled operator, V and Y (n_nodes, 2, K), K fastest: one coalesced row of V per
 * neighbour and 32 columns, no scratch. */
D2IC_API int d2ic_hessian_apply(const void *op, int n_nodes, int node_chunk_k, const float *V, int K, float *Y,
                                void *stream);
/* Column k of out (n_nodes x 2 x K) = scale * (d grad_u J / dI2) dI, dI given by its
 * B-spline coefficients (halo layout of the frame).  slots: node_chunk_k * n_nodes * 2 floats. */
D2IC_API int d2ic_mixed_term(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, const float *u,
                             const float *dcoeff, float scale, float *slots, float *out, int K, int k, void *stream);
/* The same for n_images coefficient images in one launch (image i at dcoeff + i coeff_stride
 * floats) into columns k0 .. k0 + n_images - 1; slots: n_images * node_chunk_k * n_nodes * 2
 * floats, zero where no chunk writes (zeroed once by the caller). */
D2IC_API int d2ic_mixed_term_batch(const d2ic_frame_t *frame_dev, int n_chunks, int n_nodes, int node_chunk_k,
                                   const float *u, const float *dcoeff, int n_images, long long coeff_stride,
                                   float scale, float *slots, float *out, int K, int k0, void *stream);
/* Adjoint of d2ic_mixed_term: gcoeff (halo layout, zeroed by the caller) += scale *
 * (d grad_u J / dI2 coefficients)^T lambda, by atomic scatter (backward of the bicubic sampling). */
D2IC_API int d2ic_mixed_term_T(const d2ic_frame_t *frame_dev, int n_chunks, const float *u, const float *lam,
                               float scale, float *gcoeff, void *stream);
/* Transpose of d2ic_bspline_prefilter: image-space gradient from a coefficient-space one.
 * tmp: H x cpitch floats. */
D2IC_API int d2ic_bspline_prefilter_T(const float *gcoeff, int H, int W, int pad, int cpitch, float *tmp, float *gimg,
                                      void *stream);

/* ---- synthetic speckle frames (no counterpart in the reference, which reads camera images from
 *      disk): the benchmark streams' stand-in for recorded frames ---- */

/* Raw speckle field at every pixel centre y of an HxW frame: sum over dots (cx, cy, sigma, amp;
 * float4 each, bucketed by cell of `cell_px` pixels, gw x gh cells row-major, dots of cell c at
 * cell_start[c] .. cell_start[c+1]-1) of amp exp(-|x - c|^2 / (2 sigma^2)) for
 * |x - c| <= cutoff_sigmas sigma, at x = phi^-1(y) given as 6 doubles in HOST memory (x = m0 + m1 yx
 * + m2 yy, y = m3 + m4 yx + m5 yy); dots, cell_start and out are device pointers.  cell_px must be at
 * least the largest cut-off radius. */
D2IC_API int d2ic_render_speckle(const float *dots, const int *cell_start, float cell_px, int gw, int gh,
                                 float cutoff_sigmas, const double *inv_affine, int H, int W, float *out,
                                 void *stream);
/* Grey levels 20 + (raw - lo) scale plus N(0, sigma^2) noise from a counter-based generator seeded by
 * `seed`; out is float32, or uint8 rounded and clamped to [0, 255] when out_u8 != 0. */
D2IC_API int d2ic_speckle_finish(const float *raw, long long n, float lo, float scale, float sigma,
                                 unsigned long long seed, int out_u8, void *out, void *stream);

/* ---- initial motion (replaces _match_centers_jax, d2ic/solver_translation_zncc.py:118-168,
 *      and _project_centers_to_nodes_idw, d2ic/dic_init_motion.py:64-91) ---- */
D2IC_API int d2ic_zncc_match(const float *ref, int Hr, int Wr, const float *def, int Hd, int Wd,
                    const float *centers, int n_centers, int win, int search,
                    float *u_out, float *score_out, void *stream);
D2IC_API int d2ic_idw_project(const float *nodes, int n_nodes, const float *centers, const float *disp,
                     int n_centers, float power, float *u_out, void *stream);

/* ---- strain (replaces compute_green_lagrange_strain_nodes_lsq + green_lagrange_to_voigt,
 *      d2ic/strain.py:11-114) ---- */
D2IC_API int d2ic_strain_gl(const float *u, const float *nodes, const int *nbr_index, const int *nbr_degree,
                   int n_nodes, int max_deg, float gauge_length, float eps,
                   float *voigt_out, float *F_out, void *stream);

/* Linearised strain for K displacement directions (the strain sensitivity of the implicit adjoint;
 * the derivative of d2ic/strain.py:11-92 with respect to u): u (n_nodes, 2) FP64 is the
 * linearisation point, du (K, n_nodes, 2) FP64 the directions, nodes (n_nodes, 2) FP64;
 * dvoigt_out (K, n_nodes, 3) FP64 = [dE00, dE11, (dE01 + dE10) / 2] with dE = (dG^T F + F^T dG) / 2,
 * F = I + G(u), dG = G(du), G the same weighted least-squares gradient as d2ic_strain_gl.
 * work: d2ic_strain_gl_jvp_work_doubles(n_nodes, max_deg) doubles of device scratch.
 * No counterpart in the reference (its strain is differentiated by JAX autodiff). */
D2IC_API size_t d2ic_strain_gl_jvp_work_doubles(int n_nodes, int max_deg);
D2IC_API int d2ic_strain_gl_jvp(const double *u, const double *du, int K, const double *nodes, const int *nbr_index,
                       const int *nbr_degree, int n_nodes, int max_deg, double gauge_length, double eps,
                       double *work, double *dvoigt_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* D2IC_GB300_H */
