"""On-disk formats: per-frame npz (d2ic/batch_mesh_based.py:174-185) and fields_sequence.npz
(doc/03_0_tutorial_sequentialDIC.py:213-239), written from host and torch inputs."""
from __future__ import annotations

import numpy as np
import pytest


def _results(n_frames, with_maps):
    import torch

    from d2ic_gb300.dataclasses import DICDiagnostics, DICResult
    rng = np.random.default_rng(5)
    out = []
    for k in range(n_frames):
        maps = {"discrepancy_ref": torch.from_numpy(rng.normal(size=(6, 7)))} if with_maps else {}
        out.append(DICResult(u_nodal=torch.from_numpy(rng.normal(size=(9, 2)).astype(np.float32)),
                             strain=rng.normal(size=(9, 3)), diagnostics=DICDiagnostics(info={}), pixel_maps=maps))
    return out


def test_frame_npz_fields(tmp_path):
    from d2ic_gb300 import save_frame_npz
    r = _results(1, True)[0]
    z = np.load(save_frame_npz(tmp_path / "frame_0000.npz", r))
    assert sorted(z.files) == ["discrepancy_ref", "strain", "u_nodal"]
    assert np.array_equal(z["u_nodal"], r.u_nodal.numpy()) and z["u_nodal"].dtype == np.float32
    assert np.array_equal(z["strain"], r.strain)
    assert np.array_equal(z["discrepancy_ref"], r.pixel_maps["discrepancy_ref"].numpy())
    r2 = _results(1, False)[0]
    assert "discrepancy_ref" not in np.load(save_frame_npz(tmp_path / "f.npz", r2)).files


def test_fields_sequence(tmp_path):
    from d2ic_gb300 import save_fields_sequence
    nodes = np.arange(18, dtype=np.float64).reshape(9, 2)
    res = _results(3, True)
    p = save_fields_sequence(tmp_path, nodes, res, ref_path="ref.tif", def_paths=["a.tif", "b.tif", "c.tif"])
    assert p.name == "fields_sequence.npz"
    z = np.load(p)
    assert np.array_equal(z["nodes_xy"], nodes)
    assert z["u_nodal"].shape == (3, 9, 2) and z["strain"].shape == (3, 9, 3)
    assert np.array_equal(z["u_nodal"][2], res[2].u_nodal.numpy())
    assert z["discrepancy_ref"].shape == (3, 6, 7) and z["discrepancy_ref"].dtype == np.float32
    assert str(z["ref_path"]) == "ref.tif" and list(z["def_paths"]) == ["a.tif", "b.tif", "c.tif"]
    # one frame without a map: no map stack, like the tutorial
    res[1].pixel_maps.clear()
    z = np.load(save_fields_sequence(tmp_path / "seq.npz", nodes, res))
    assert "discrepancy_ref" not in z.files
    with pytest.raises(ValueError):
        save_fields_sequence(tmp_path, nodes, [])
