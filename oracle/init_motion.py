"""Oracle ZNCC integer-translation search and IDW projection (FP64).

Test infrastructure only (see oracle/__init__.py).

Reference: d2ic/solver_translation_zncc.py:89-168, d2ic/dic_init_motion.py:64-91.
"""
from __future__ import annotations

import numpy as np


def zncc_scores(template, windows):
    """ZNCC of a template against a stack of windows (d2ic/solver_translation_zncc.py:89-98).

    Both sides zero-mean and divided by (population std + 1e-12); score is the
    mean of the product.
    """
    t = template - template.mean()
    t = t / (t.std() + 1e-12)
    w = windows - windows.mean(axis=(1, 2), keepdims=True)
    w = w / (w.std(axis=(1, 2), keepdims=True) + 1e-12)
    return (w * t).mean(axis=(1, 2))


def match_centers(centers, ref_image, def_image, win, search):
    """Best integer translation per centre (d2ic/solver_translation_zncc.py:118-168).

    Centre rounded half-to-even; template and search patch must lie inside the
    images, else displacement 0 and score NaN; the first maximum over offsets
    in row-major (ky, kx) order wins.  Returns ``(u (Nc,2) f64, scores (Nc,))``.
    """
    ref = np.asarray(ref_image, dtype=np.float64)
    dfm = np.asarray(def_image, dtype=np.float64)
    r = win // 2
    hr, wr = ref.shape[:2]
    hd, wd = dfm.shape[:2]
    npa = 2 * search + 1
    ps = win + 2 * search
    c = np.asarray(centers, dtype=np.float64)
    out = np.zeros((c.shape[0], 2))
    scores = np.full(c.shape[0], np.nan)
    for n in range(c.shape[0]):
        x = int(np.rint(c[n, 0]))
        y = int(np.rint(c[n, 1]))
        tpl_ok = (y - r >= 0) and (y + r < hr) and (x - r >= 0) and (x + r < wr)
        xs, ys, xe, ye = x - search, y - search, x + search, y + search
        patch_ok = (ys - r >= 0) and (ye + r < hd) and (xs - r >= 0) and (xe + r < wd)
        if not (tpl_ok and patch_ok):
            continue
        tpl = ref[y - r:y - r + win, x - r:x - r + win]
        patch = dfm[ys - r:ys - r + ps, xs - r:xs - r + ps]
        sw = np.lib.stride_tricks.sliding_window_view(patch, (win, win)).reshape(npa * npa, win, win)
        s = zncc_scores(tpl, sw)
        best = int(np.argmax(s))
        ky, kx = divmod(best, npa)
        out[n] = [xs + kx - x, ys + ky - y]
        scores[n] = s[best]
    return out, scores


def apply_score_min(u, scores, score_min):
    """Reject matches below ``score_min`` (d2ic/solver_translation_zncc.py:74-77)."""
    if score_min is None:
        return u, scores
    valid = scores >= float(score_min)
    return np.where(valid[:, None], u, 0.0), np.where(valid, scores, np.nan)


def project_centers_to_nodes_idw(nodes, centers, disp, power=2.0):
    """Inverse-distance weighting of centre displacements onto nodes (d2ic/dic_init_motion.py:64-91).

    Centres whose displacement has a NaN are dropped; a node closer than 1e-6
    to a centre takes that (first) centre's value.
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    c = np.asarray(centers, dtype=np.float64)
    d = np.asarray(disp, dtype=np.float64)
    valid = ~np.isnan(d).any(axis=1)
    c, d = c[valid], d[valid]
    out = np.zeros_like(nodes)
    if c.size == 0:
        return out
    for i, p in enumerate(nodes):
        dist = np.linalg.norm(c - p, axis=1)
        close = dist < 1e-6
        if close.any():
            out[i] = d[close][0]
            continue
        w = 1.0 / np.power(dist + 1e-12, power)
        w /= w.sum()
        out[i] = (w[:, None] * d).sum(axis=0)
    return out
