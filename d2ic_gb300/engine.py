"""GPU layout of a frame and launches of the CG engine.

Data layout in HBM (per reference image + mesh, built once by
:class:`FrameLayout`):

* ``pix``   (Np, 16 B): element-major pixel records ``{col | row << 16, I1,
  xi, eta}``, read with one 128-bit load; pixels of one element are
  contiguous (in the reference's pixel order) and cut into chunks of at most
  256 pixels;
* ``chunk_begin`` (Nc+1), ``chunk_nodes`` (Nc, 4): chunk extents and the 4
  nodes of the chunk's element;
* ``chunk_box`` (Nc, 2): inclusive pixel box of each chunk, which bounds the
  chunk's shared-memory coefficient tile;
* ``chunk_slot`` (Nc,): for each of the chunk's 4 nodes, the slot (rank of the
  chunk among the node's chunks) where the pixel pass stores the chunk's
  gradient partial for that node; the node pass sums its K slots in order --
  the transpose of the chunk -> node gather without atomics;
* ``nbr_index`` / ``nbr_weight`` (max_deg, Nn): the spring table, column-major,
  weights pre-multiplied by (rho_i + rho_j)/2 in FP32.

Per frame being solved (:class:`FrameSlot`): the deformed image's
B-spline coefficients with a 16-pixel halo (row pitch a multiple of 32
floats), the CG workspace, initial/final displacement, history and status.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import ptr

PAD = 16


def _pitch(W: int) -> int:
    return ((W + 2 * PAD + 31) // 32) * 32


def interp_kind(interpolation: str) -> int:
    v = str(interpolation).lower()
    if v == "bilinear":
        v = "linear"
    if v == "cubic":
        return _lib.INTERP_CUBIC
    if v == "linear":
        return _lib.INTERP_LINEAR
    raise ValueError(f"Unsupported interpolation: {interpolation}")


def as_device_image(img, device, keep_u8: bool = False) -> torch.Tensor:
    """float32 contiguous (H, W) image on ``device`` (host arrays are copied).

    ``keep_u8``: 8-bit camera frames stay 8-bit (one byte per pixel over the host link); the
    coefficient preparation widens them on the device."""
    if isinstance(img, torch.Tensor):
        if keep_u8 and img.dtype == torch.uint8:
            t = img.to(device=device, non_blocking=img.device.type == "cpu" and img.is_pinned())
        else:
            t = img.to(device=device, dtype=torch.float32)
    else:
        a = np.asarray(img)
        if not (keep_u8 and a.dtype == np.uint8):
            a = a.astype(np.float32, copy=False)
        t = torch.from_numpy(np.ascontiguousarray(a)).to(device, non_blocking=False)
    if t.dim() != 2:
        raise ValueError(f"expected a 2D image, got shape {tuple(t.shape)}")
    return t.contiguous()


def prepare_coefficients(img_dev: torch.Tensor, kind: int, out: torch.Tensor | None = None,
                         tmp: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """Halo'd sampling array of an image: B-spline coefficients (cubic) or the padded image (linear)."""
    H, W = img_dev.shape
    cp = _pitch(W)
    dev = img_dev.device
    if out is None:
        out = torch.empty((H + 2 * PAD, cp), dtype=torch.float32, device=dev)
    s = _lib.stream_handle(stream)
    u8 = img_dev.dtype == torch.uint8
    if not u8 and img_dev.dtype != torch.float32:
        raise ValueError(f"images are float32 or uint8, got {img_dev.dtype}")
    if kind == _lib.INTERP_CUBIC:
        if tmp is None:
            tmp = torch.empty((H, cp), dtype=torch.float32, device=dev)
        _lib.call("d2ic_bspline_prefilter_u8" if u8 else "d2ic_bspline_prefilter", ptr(img_dev), H, W, PAD, cp,
                  ptr(tmp), ptr(out), s)
    else:
        _lib.call("d2ic_pad_image_u8" if u8 else "d2ic_pad_image", ptr(img_dev), H, W, PAD, cp, ptr(out), s)
    return out


def sample_points(coeff: torch.Tensor, H: int, W: int, kind: int, xy_index: torch.Tensor, stream=None):
    """Value and gradient at image-index coordinates (x = col, y = row)."""
    n = xy_index.shape[0]
    dev = coeff.device
    xy = xy_index.to(device=dev, dtype=torch.float32).contiguous()
    v = torch.empty(n, dtype=torch.float32, device=dev)
    gx = torch.empty_like(v)
    gy = torch.empty_like(v)
    _lib.call("d2ic_sample_points", ptr(coeff), H, W, PAD, coeff.shape[1], kind, ptr(xy), n, ptr(v), ptr(gx),
              ptr(gy), _lib.stream_handle(stream))
    return v, gx, gy


def _xi_eta(pix) -> np.ndarray:
    xe = getattr(pix, "xi_eta", None)
    if xe is not None:
        return np.asarray(xe, dtype=np.float64)
    # Q4: N1 + N2 - N0 - N3 = xi and N2 + N3 - N0 - N1 = eta exactly
    N = np.asarray(pix.pixel_shapeN, dtype=np.float64)
    return np.stack([N[:, 1] + N[:, 2] - N[:, 0] - N[:, 3], N[:, 2] + N[:, 3] - N[:, 0] - N[:, 1]], axis=1)


def _elements_of(pix) -> np.ndarray:
    e = getattr(pix, "pixel_elts", None)
    if e is not None:
        return np.asarray(e, dtype=np.int64)
    _, inv = np.unique(np.asarray(pix.pixel_nodes, dtype=np.int64), axis=0, return_inverse=True)
    return inv.reshape(-1)


def _grid_struct(nodes, elements, gc, roi_mask, H: int, W: int, bbox_pad: float, dev):
    """d2ic_grid_t of a tensor-grid mesh (``gc`` from pixel_assets.grid_cells) and the device
    tensors it points to (keep them alive while the struct is used)."""
    from .pixel_assets import _bbox
    gx, gy, cell, elem_cell = gc
    T = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt))).to(dev)
    keep = dict(gx=T(gx, np.float64), gy=T(gy, np.float64), cell=T(cell, np.int32), ec=T(elem_cell, np.int32),
                el=T(elements, np.int32), nodes=T(nodes, np.float64))
    if roi_mask is not None:
        rm = np.asarray(roi_mask, dtype=bool)
        if rm.shape != (H, W):
            raise ValueError(f"roi_mask shape {rm.shape} does not match ref_image shape {(H, W)}")
        keep["roi"] = T(rm, np.uint8)
    g = _lib.Grid()
    g.gx, g.gy, g.nx, g.ny = ptr(keep["gx"]), ptr(keep["gy"]), int(gx.size), int(gy.size)
    g.cell, g.elem_cell, g.elements, g.nodes = ptr(keep["cell"]), ptr(keep["ec"]), ptr(keep["el"]), ptr(keep["nodes"])
    g.roi = ptr(keep["roi"]) if "roi" in keep else None
    g.n_elem, g.n_nodes, g.H, g.W = int(elements.shape[0]), int(nodes.shape[0]), int(H), int(W)
    g.i0, g.i1, g.j0, g.j1 = _bbox(nodes, H, W, bbox_pad)
    return g, keep


def _grid_counts(g, n_elem: int, dev) -> np.ndarray:
    """ROI pixels owned by each element (d2ic_grid_count)."""
    counts = torch.zeros(max(n_elem, 1), dtype=torch.int32, device=dev)
    _lib.call("d2ic_grid_count", ctypes.byref(g), ptr(counts), _lib.stream_handle())
    return counts[:n_elem].cpu().numpy().astype(np.int64)


def grid_element_counts(mesh, roi_mask, image_shape, bbox_pad: float = 2.0, binning: float = 1.0, device=None):
    """ROI pixels of each element of a tensor-grid mesh, counted on the device."""
    from .pixel_assets import grid_cells
    dev = torch.device(device if device is not None else "cuda")
    nodes = np.asarray(mesh.nodes_xy, dtype=np.float64) / float(binning)
    elements = np.asarray(mesh.elements, dtype=np.int64)
    gc = grid_cells(nodes, elements)
    if gc is None:
        raise ValueError("grid_element_counts needs a tensor-grid mesh with one element per cell")
    H, W = (int(v) for v in image_shape)
    g, keep = _grid_struct(nodes, elements, gc, roi_mask, H, W, bbox_pad, dev)
    return _grid_counts(g, int(elements.shape[0]), dev)


class FrameLayout:
    """Device-resident static data of one (reference image, mesh) pair."""

    def __init__(self, pix, n_nodes: int, ref_image, interpolation: str = "cubic", device=None,
                 chunk_max: int = _lib.CHUNK_MAX):
        if not 1 <= int(chunk_max) <= _lib.CHUNK_MAX:
            raise ValueError(f"chunk_max must be in [1, {_lib.CHUNK_MAX}]")
        chunk_max = int(chunk_max)
        from .pixel_assets import GridPixelData
        if isinstance(pix, GridPixelData) and pix.device_ok():
            built = FrameLayout.from_grid(pix.mesh, pix.roi_mask, ref_image, interpolation, device, chunk_max,
                                          bbox_pad=pix.bbox_pad, binning=pix.binning)
            self.__dict__.update(built.__dict__)
            return
        self.device = torch.device(device if device is not None else "cuda")
        self.kind = interp_kind(interpolation)
        self.n_nodes = int(n_nodes)
        ref = as_device_image(ref_image, self.device)
        self.H, self.W = ref.shape
        if self.H >= 65536 or self.W >= 65536:
            raise ValueError("image sides must be < 65536")
        self.cpitch = _pitch(self.W)
        pc = np.asarray(pix.pixel_coords_ref, dtype=np.float64)
        pn = np.asarray(pix.pixel_nodes, dtype=np.int64)
        Np = pc.shape[0]
        self.n_pix = Np
        elts = _elements_of(pix)
        order = np.argsort(elts, kind="stable")                  # element-major, pixel order inside
        e_sorted = elts[order]
        # element runs -> chunks of <= chunk_max pixels (equal split of long runs)
        if Np:
            starts = np.flatnonzero(np.r_[True, e_sorted[1:] != e_sorted[:-1]])
            lens = np.diff(np.r_[starts, Np])
            nch = (lens + chunk_max - 1) // chunk_max
            run = np.repeat(np.arange(starts.size), nch)
            k = np.arange(nch.sum()) - np.repeat(np.cumsum(nch) - nch, nch)
            cb = starts[run] + (lens[run] * k) // nch[run]
            chunk_begin = np.r_[cb, Np].astype(np.int32)
            chunk_nodes = pn[order[cb]].astype(np.int32)
        else:
            chunk_begin = np.zeros(1, np.int32)
            chunk_nodes = np.zeros((0, 4), np.int32)
        self.n_chunks = int(chunk_begin.size - 1)
        # inclusive pixel box of each chunk (bounds of its shared-memory coefficient tile)
        colrow = np.stack([np.floor(pc[:, 0] - 0.5), np.floor(pc[:, 1] - 0.5)], axis=1).astype(np.int64)[order]
        if self.n_chunks:
            cstart = chunk_begin[:-1].astype(np.int64)
            bx0 = np.minimum.reduceat(colrow[:, 0], cstart)
            by0 = np.minimum.reduceat(colrow[:, 1], cstart)
            bx1 = np.maximum.reduceat(colrow[:, 0], cstart)
            by1 = np.maximum.reduceat(colrow[:, 1], cstart)
            chunk_box = np.stack([bx0 | (by0 << 16), bx1 | (by1 << 16)], axis=1).astype(np.int64)
            chunk_box = chunk_box.astype(np.uint32).view(np.int32)
            # Pixel order inside full 16-column chunks (h rows, h a multiple of 8): the two
            # half-warps of each 32-pixel step read rows r and r + 4 instead of r and r + 1, so that
            # with the 28-float tile pitch of such chunks their taps fall 16 banks apart.  Only the
            # order of a chunk's partial sums changes.
            lens_c = np.diff(chunk_begin).astype(np.int64)
            w_c, h_c = bx1 - bx0 + 1, by1 - by0 + 1
            full = (w_c == 16) & (h_c % 8 == 0) & (lens_c == 16 * h_c)
            if self.kind == _lib.INTERP_CUBIC and full.any():
                cid = np.repeat(np.arange(self.n_chunks), lens_c)
                sel = full[cid]
                r = colrow[sel, 1] - by0[cid[sel]]
                c = colrow[sel, 0] - bx0[cid[sel]]
                dest = cstart[cid[sel]] + 32 * ((r & 3) + ((r >> 3) << 2)) + 16 * ((r >> 2) & 1) + c
                src = np.flatnonzero(sel)
                if np.bincount(dest, minlength=Np).max(initial=0) > 1:
                    raise AssertionError("pixel permutation inside chunks is not one-to-one")
                new = order.copy()
                new[dest] = order[src]
                order = new
                colrow = np.stack([np.floor(pc[:, 0] - 0.5), np.floor(pc[:, 1] - 0.5)],
                                  axis=1).astype(np.int64)[order]
        else:
            chunk_box = np.zeros((0, 2), np.int32)
        # node gradient slots: the chunk's partial for its local node a goes to slot rank(chunk) of
        # that node, ranks in ascending chunk order; K = most chunks meeting at one node
        flat = chunk_nodes.reshape(-1).astype(np.int64)
        o = np.argsort(flat, kind="stable")
        cnt = np.bincount(flat, minlength=self.n_nodes)
        K = max(int(cnt.max(initial=0)), 1)
        if K > 255:
            raise ValueError(f"a node touches {K} chunks; at most 255 are supported")
        rank = np.empty(flat.size, dtype=np.int64)
        rank[o] = np.arange(flat.size) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        r4 = rank.reshape(-1, 4)
        chunk_slot = (r4[:, 0] | (r4[:, 1] << 8) | (r4[:, 2] << 16) | (r4[:, 3] << 24)).astype(np.uint32).view(np.int32)
        self.node_chunk_k = K
        # chunks with a node in each group of NODE_GROUP consecutive nodes (the group's reducer
        # waits for that many completion counts per pass)
        ng = (self.n_nodes + _lib.NODE_GROUP - 1) // _lib.NODE_GROUP
        cg = np.sort(chunk_nodes.astype(np.int64).reshape(-1, 4) // _lib.NODE_GROUP, axis=1)
        first = np.ones(cg.shape, dtype=bool)
        first[:, 1:] = cg[:, 1:] != cg[:, :-1]
        group_need = np.bincount(cg[first], minlength=ng).astype(np.int32)
        # spring table: entries beyond the degree are padding; column-major for coalesced node-pass loads
        nbi = np.asarray(pix.node_neighbor_index, dtype=np.int64).reshape(self.n_nodes, -1)
        md = nbi.shape[1]
        deg = np.asarray(pix.node_neighbor_degree, dtype=np.int64)
        valid = np.arange(md)[None, :] < deg[:, None]
        nid = np.where(valid, nbi, 0)
        rho = np.asarray(pix.node_reg_weight, dtype=np.float32)
        w = np.asarray(pix.node_neighbor_weight, dtype=np.float32).reshape(self.n_nodes, -1)
        wc = (w * np.float32(0.5) * (rho[:, None] + rho[nid])).astype(np.float32)
        self.max_deg = md
        nbr_index = np.where(valid, nbi, -1).astype(np.int32).T.copy()
        nbr_weight = np.where(valid, wc, np.float32(0)).astype(np.float32).T.copy()
        # pixel records (I1 sampled on the device from the reference image)
        colrow = colrow.astype(np.int32)
        xieta = _xi_eta(pix).astype(np.float32)[order]
        dev = self.device
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        self.chunk_begin = T(chunk_begin)
        self.chunk_nodes = T(chunk_nodes)
        self.chunk_box = T(chunk_box) if self.n_chunks else torch.zeros((1, 2), dtype=torch.int32, device=dev)
        self.chunk_slot = T(chunk_slot) if self.n_chunks else torch.zeros((1,), dtype=torch.int32, device=dev)
        self.group_need = T(group_need)
        self.nbr_index = T(nbr_index) if md else torch.full((1,), -1, dtype=torch.int32, device=dev)
        self.nbr_weight = T(nbr_weight) if md else torch.zeros((1,), dtype=torch.float32, device=dev)
        self.pixel_order = order
        self.pix = torch.empty((max(Np, 1), 4), dtype=torch.int32, device=dev)
        ref_coeff = prepare_coefficients(ref, self.kind)
        if Np:
            cr = T(colrow)
            xe = T(xieta)
            _lib.call("d2ic_pack_pixels", ptr(cr), ptr(xe), Np, ptr(ref_coeff), self.H, self.W, PAD, self.cpitch,
                      self.kind, ptr(self.pix), _lib.stream_handle())
        self.ref_image = ref
        del ref_coeff
        self.tile_w, self.tile_h = self._tile_shape(self.kind, chunk_box, self.W, self.H)

    @staticmethod
    def _tile_shape(kind: int, chunk_box: np.ndarray, W: int, H: int):
        """Shared-memory coefficient tile per chunk (cubic): a chunk's pixel box plus the 4x4
        stencil (3), a 2-pixel margin each side (4), one pixel of spread between the element's
        nodes (1) and, in x, up to 3 columns lost to the 16-byte TMA alignment.  Sized for the
        largest box when that fits in TILE_MAX_FLOATS, else for the 90th percentile of the boxes'
        widths and heights (a few partly covered elements, e.g. on an ellipse boundary, can make one
        chunk's box much larger than the rest): a chunk whose box exceeds the tile reads the pixels
        outside it from global memory with the same arithmetic, so the tile changes no result."""
        if kind != _lib.INTERP_CUBIC or chunk_box.shape[0] == 0 or W + 2 * PAD >= 32768 or H + 2 * PAD >= 32768:
            return 0, 0
        b0 = chunk_box[:, 0].astype(np.int64) & 0xFFFFFFFF
        b1 = chunk_box[:, 1].astype(np.int64) & 0xFFFFFFFF
        cws = (b1 & 0xFFFF) - (b0 & 0xFFFF) + 1
        chs = (b1 >> 16) - (b0 >> 16) + 1

        def shape(cw, ch):
            return (int(cw) + 11 + 3) // 4 * 4, int(ch) + 8

        tw, th = shape(cws.max(), chs.max())
        if tw * th <= _lib.TILE_MAX_FLOATS:
            return tw, th
        tw, th = shape(np.percentile(cws, 90, method="higher"), np.percentile(chs, 90, method="higher"))
        return (tw, th) if tw * th <= _lib.TILE_MAX_FLOATS else (0, 0)

    @classmethod
    def from_grid(cls, mesh, roi_mask, ref_image, interpolation: str = "cubic", device=None,
                  chunk_max: int = _lib.CHUNK_MAX, bbox_pad: float = 2.0, binning: float = 1.0,
                  node_reg_weight=None) -> "FrameLayout":
        """The layout of a tensor-grid mesh built on the device from the ROI mask (d2ic_grid_count,
        d2ic_grid_layout, d2ic_grid_springs): the same tensors, bit for bit, as building the host
        pixel assets (build_pixel_assets) and then the layout from them."""
        from .pixel_assets import grid_cells
        dev = torch.device(device if device is not None else "cuda")
        chunk_max = int(chunk_max)
        if not 1 <= chunk_max <= _lib.CHUNK_MAX:
            raise ValueError(f"chunk_max must be in [1, {_lib.CHUNK_MAX}]")
        nodes = np.asarray(mesh.nodes_xy, dtype=np.float64) / float(binning)
        elements = np.asarray(mesh.elements, dtype=np.int64)
        gc = grid_cells(nodes, elements)
        if gc is None:
            raise ValueError("from_grid needs a tensor-grid mesh with one element per cell")
        self = cls.__new__(cls)
        self.device = dev
        self.kind = interp_kind(interpolation)
        self.n_nodes = int(nodes.shape[0])
        ref = as_device_image(ref_image, dev)
        self.H, self.W = (int(v) for v in ref.shape)
        if self.H >= 65536 or self.W >= 65536:
            raise ValueError("image sides must be < 65536")
        self.cpitch = _pitch(self.W)
        T = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dt))).to(dev)
        g, keep = _grid_struct(nodes, elements, gc, roi_mask, self.H, self.W, bbox_pad, dev)
        s = _lib.stream_handle()
        Ne = int(elements.shape[0])
        cnt = _grid_counts(g, Ne, dev)
        nch = (cnt + chunk_max - 1) // chunk_max
        off = np.r_[0, np.cumsum(cnt)]
        choff = np.r_[0, np.cumsum(nch)]
        Np, n_chunks = int(off[-1]), int(choff[-1])
        if Np >= 2 ** 31:
            raise ValueError("too many ROI pixels for one frame")
        self.n_pix, self.n_chunks = Np, n_chunks
        self.element_pixel_counts = cnt
        t_off, t_choff = T(off, np.int32), T(choff, np.int32)
        ref_coeff = prepare_coefficients(ref, self.kind)
        self.pix = torch.empty((max(Np, 1), 4), dtype=torch.int32, device=dev)
        chunk_begin = torch.zeros(n_chunks + 1, dtype=torch.int32, device=dev)
        chunk_nodes = torch.empty((max(n_chunks, 1), 4), dtype=torch.int32, device=dev)
        chunk_box = torch.zeros((max(n_chunks, 1), 2), dtype=torch.int32, device=dev)
        chunk_slot = torch.zeros(max(n_chunks, 1), dtype=torch.int32, device=dev)
        ng = (self.n_nodes + _lib.NODE_GROUP - 1) // _lib.NODE_GROUP
        self.group_need = torch.empty(ng, dtype=torch.int32, device=dev)
        stats = torch.zeros(4, dtype=torch.int32, device=dev)
        nb = int(_lib.load().d2ic_grid_scratch_bytes(Np, n_chunks))
        scratch = torch.empty(nb + 256, dtype=torch.uint8, device=dev)
        sp = (ptr(scratch) + 255) & ~255
        _lib.call("d2ic_grid_layout", ctypes.byref(g), ptr(t_off), ptr(t_choff), Np, n_chunks, self.kind,
                  ptr(ref_coeff), self.cpitch, PAD, sp, nb, ptr(self.pix), ptr(chunk_begin), ptr(chunk_nodes),
                  ptr(chunk_box), ptr(chunk_slot), ptr(self.group_need), ptr(stats), s)
        st = stats.cpu().numpy()
        if st[2]:
            raise ValueError("from_grid: an element has more than 32 chunks; use a larger chunk size")
        self.node_chunk_k = max(int(st[0]), 1)
        if self.node_chunk_k > 255:
            raise ValueError(f"a node touches {self.node_chunk_k} chunks; at most 255 are supported")
        md = int(st[1])
        self.max_deg = md
        rho = (torch.ones(self.n_nodes, dtype=torch.float32, device=dev) if node_reg_weight is None
               else T(node_reg_weight, np.float32))
        if md:
            self.nbr_index = torch.empty((md, self.n_nodes), dtype=torch.int32, device=dev)
            self.nbr_weight = torch.empty((md, self.n_nodes), dtype=torch.float32, device=dev)
            _lib.call("d2ic_grid_springs", ctypes.byref(g), ptr(rho), md, ptr(self.nbr_index), ptr(self.nbr_weight), s)
        else:
            self.nbr_index = torch.full((1,), -1, dtype=torch.int32, device=dev)
            self.nbr_weight = torch.zeros((1,), dtype=torch.float32, device=dev)
        self.chunk_begin = chunk_begin
        self.chunk_nodes = chunk_nodes[:n_chunks] if n_chunks else torch.zeros((0, 4), dtype=torch.int32, device=dev)
        self.chunk_box = chunk_box if n_chunks else torch.zeros((1, 2), dtype=torch.int32, device=dev)
        self.chunk_slot = chunk_slot if n_chunks else torch.zeros((1,), dtype=torch.int32, device=dev)
        self.pixel_order = None
        self.ref_image = ref
        box = chunk_box[:n_chunks].cpu().numpy() if n_chunks else np.zeros((0, 2), np.int32)
        self.tile_w, self.tile_h = cls._tile_shape(self.kind, box, self.W, self.H)
        torch.cuda.current_stream(dev).synchronize()        # the scratch and staging tensors go out of scope
        return self

    # bytes read per pixel per objective evaluation by the P phase (pixel record + ~1 coefficient)
    PIX_BYTES = 16 + 4


class FrameSlot:
    """Per-solve device buffers and the frame descriptor."""

    def __init__(self, layout: FrameLayout, max_iter: int):
        self.layout = layout
        dev = layout.device
        L = layout
        self.max_iter = int(max_iter)
        self.coeff = torch.empty((L.H + 2 * PAD, L.cpitch), dtype=torch.float32, device=dev)
        self.tmp = torch.empty((L.H, L.cpitch), dtype=torch.float32, device=dev) if L.kind == _lib.INTERP_CUBIC else None
        self.u0 = torch.zeros((L.n_nodes, 2), dtype=torch.float32, device=dev)
        self.u_out = torch.zeros((L.n_nodes, 2), dtype=torch.float32, device=dev)
        self.hist = torch.full((max(self.max_iter, 1), 3), float("nan"), dtype=torch.float32, device=dev)
        self.info = torch.zeros(3, dtype=torch.int32, device=dev)          # n_iters, status, n_evals
        nb = _lib.load().d2ic_frame_workspace_bytes(L.n_nodes, L.n_chunks, L.node_chunk_k)
        self.ws = torch.empty(nb, dtype=torch.uint8, device=dev)
        self.desc = self._descriptor(1e-6, 0.0)

    def _descriptor(self, tol: float, alpha_reg: float) -> _lib.Frame:
        L = self.layout
        f = _lib.Frame()
        f.coeff = ptr(self.coeff)
        f.pix = ptr(L.pix)
        f.chunk_begin = ptr(L.chunk_begin)
        f.chunk_nodes = ptr(L.chunk_nodes)
        f.chunk_box = ptr(L.chunk_box)
        f.chunk_slot = ptr(L.chunk_slot)
        f.group_need = ptr(L.group_need)
        f.node_chunk_k = L.node_chunk_k
        f.nbr_index = ptr(L.nbr_index)
        f.nbr_weight = ptr(L.nbr_weight)
        f.u0 = ptr(self.u0)
        f.u_out = ptr(self.u_out)
        f.hist = ptr(self.hist)
        f.n_iters = ptr(self.info)
        f.status = ptr(self.info) + 4
        f.n_evals = ptr(self.info) + 8
        f.tol = float(tol)
        f.alpha_reg = float(alpha_reg)
        f.max_iter = self.max_iter
        f.W, f.H, f.cpitch, f.pad = L.W, L.H, L.cpitch, PAD
        f.n_pix, f.n_chunks, f.n_nodes, f.max_deg = L.n_pix, L.n_chunks, L.n_nodes, L.max_deg
        _lib.call("d2ic_frame_bind_workspace", ctypes.byref(f), ptr(self.ws))
        rc = _lib.load().d2ic_frame_encode_tiles(ctypes.byref(f), L.tile_w, L.tile_h)
        if rc not in (_lib.OK, _lib.UNSUPPORTED):      # unsupported: taps through L1, same results
            _lib.check(rc)
        return f

    def set_params(self, tol: float, alpha_reg: float):
        self.desc.tol = float(tol)
        self.desc.alpha_reg = float(alpha_reg)

    def load_image(self, def_image, stream=None):
        img = as_device_image(def_image, self.layout.device, keep_u8=True)
        prepare_coefficients(img, self.layout.kind, self.coeff, self.tmp, stream)

    def set_u0(self, u0):
        if u0 is None:
            self.u0.zero_()
        elif isinstance(u0, torch.Tensor):
            self.u0.copy_(u0.reshape(-1, 2))
        else:
            self.u0.copy_(torch.from_numpy(np.ascontiguousarray(np.asarray(u0, dtype=np.float32).reshape(-1, 2))))


def descriptors_to_device(descs, device) -> torch.Tensor:
    """Pack frame descriptors into a device byte tensor (one d2ic_frame_t per frame)."""
    n = len(descs)
    arr = (_lib.Frame * n)(*descs)
    buf = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8)
    return buf.to(device)


class Engine:
    """Launch wrapper for batched solves: control scratch sized for up to ``max_frames``."""

    def __init__(self, device, max_frames: int = 1):
        self.device = torch.device(device)
        self.max_frames = int(max_frames)
        self.control = torch.empty(_lib.load().d2ic_cg_control_bytes(self.max_frames), dtype=torch.uint8,
                                   device=self.device)

    def solve(self, desc_dev: torch.Tensor, n_frames: int, kind: int, grid_blocks: int = 0, stream=None):
        if n_frames > self.max_frames:
            raise ValueError(f"{n_frames} frames > engine capacity {self.max_frames}")
        _lib.call("d2ic_cg_solve_batched", ptr(desc_dev), n_frames, ptr(self.control), self.control.numel(), kind,
                  grid_blocks, _lib.stream_handle(stream))

    def commands(self, n_frames: int) -> torch.Tensor:
        """The per-frame command words inside the control block (int32 view)."""
        off = _lib.load().d2ic_cg_command_offset()
        return self.control[off: off + 4 * n_frames].view(torch.int32)

    def run_slice(self, desc_dev: torch.Tensor, n_frames: int, kind: int, max_rounds: int, grid_blocks: int = 0,
                  stream=None, stop_flags: int = 0):
        """Advance every admitted frame by at most ``max_rounds`` objective evaluations; with
        ``stop_flags`` (D2IC_STOP_ON_FINISH | D2IC_STOP_ON_IRQ) the slice may end earlier."""
        if n_frames > self.max_frames:
            raise ValueError(f"{n_frames} frames > engine capacity {self.max_frames}")
        if stop_flags:
            _lib.call("d2ic_cg_slice_ex", ptr(desc_dev), n_frames, ptr(self.control), self.control.numel(), kind,
                      grid_blocks, int(max_rounds), int(stop_flags), _lib.stream_handle(stream))
        else:
            _lib.call("d2ic_cg_slice", ptr(desc_dev), n_frames, ptr(self.control), self.control.numel(), kind,
                      grid_blocks, int(max_rounds), _lib.stream_handle(stream))

    def irq_word(self) -> torch.Tensor:
        """The control block's interrupt word (int32 view): non-zero ends a D2IC_STOP_ON_IRQ slice."""
        off = int(_lib.load().d2ic_cg_irq_offset())
        return self.control[off:off + 4].view(torch.int32)

    def solve_traced(self, desc_dev: torch.Tensor, n_frames: int, kind: int, rounds: int = 4096, grid_blocks: int = 0):
        """Solve; per-round durations in microseconds, columns: warp 0 of block 0's pixel work, its
        node-group work, from there to the end of the round, the (last) frame control step, from
        that step to the end of the round, and the whole round."""
        tr = torch.zeros(7 * rounds, dtype=torch.int64, device=self.device)
        _lib.call("d2ic_cg_solve_traced", ptr(desc_dev), n_frames, ptr(self.control), self.control.numel(), kind,
                  grid_blocks, ptr(tr), rounds, _lib.stream_handle())
        t = tr.cpu().numpy().reshape(-1, 7).astype(np.float64)
        t = t[t[:, 5] > 0]
        return np.stack([t[:, 1] - t[:, 0], t[:, 2] - t[:, 1], t[:, 5] - t[:, 2], t[:, 4] - t[:, 3],
                         t[:, 5] - t[:, 4], t[:, 5] - t[:, 0]], axis=1) / 1e3

    def eval_objective(self, desc_dev: torch.Tensor, u: torch.Tensor, kind: int, stream=None):
        J = torch.zeros(1, dtype=torch.float64, device=self.device)
        g = torch.empty_like(u)
        _lib.call("d2ic_eval_objective", ptr(desc_dev), ptr(u), ptr(self.control), self.control.numel(), kind,
                  ptr(J), ptr(g), _lib.stream_handle(stream))
        return J, g
