"""Scene files through the device: load_ply of files written by the oracle's
restatement of the reference's format (any property order, comments, unknown
properties) equals the oracle's reading of them bit for bit; save_ply writes
the oracle's bytes; save -> load round trips exactly at 1M primitives."""
import os
import types

import numpy as np
import pytest
import torch

import oracle as orc
from ubs import ply

pytestmark = pytest.mark.gpu
DEV = "cuda"


def scene(n, D, seed=0):
    rng = np.random.default_rng(seed)
    return {"xyz": rng.standard_normal((n, 3)), "mean": rng.standard_normal((n, D - 3)),
            "rgb": rng.random((n, 3)), "opacity": rng.standard_normal((n, 1)),
            "beta": rng.standard_normal((n, D - 2)), "scale": rng.standard_normal((n, D)),
            "l_triangle": rng.standard_normal((n, D * (D - 1) // 2))}


@pytest.mark.parametrize("D", [6, 7])
def test_load_matches_oracle_reading(tmp_path, D):
    p = scene(3001, D, D)
    names = orc.ply_attribute_names(D - 2, D - 3, D, D * (D - 1) // 2)
    rng = np.random.default_rng(0)
    shuffled = list(rng.permutation(names)) + ["f_dc_0", "extra"]
    data = orc.ply_bytes(p, names=shuffled, comments=("x",))
    path = str(tmp_path / "s.ply")
    open(path, "wb").write(data)
    got = ply.load_ply(path, DEV)
    want = orc.ply_parse(data)
    for k in ply.NAMES:
        assert np.array_equal(got[k].cpu().numpy(), want[k].astype(np.float32)), k


@pytest.mark.parametrize("D", [6, 7])
def test_save_writes_oracle_bytes(tmp_path, D):
    p = scene(1000, D, 10 + D)
    path = str(tmp_path / "sub" / "o.ply")
    ply.save_ply(path, {k: torch.from_numpy(v.astype(np.float32)).to(DEV) for k, v in p.items()})
    assert open(path, "rb").read() == orc.ply_bytes(p)


def test_round_trip_one_million(tmp_path):
    from ubs import scene as S
    p = S.synthetic_params(1_000_000, 6, seed=3, device=DEV)
    path = str(tmp_path / "big.ply")
    old_chunk = ply.CHUNK_BYTES
    ply.CHUNK_BYTES = 7 << 20  # several chunks, the last one partial
    try:
        ply.save_ply(path, p)
        q = ply.load_ply(path, DEV)
    finally:
        ply.CHUNK_BYTES = old_chunk
    n, names, off = ply.read_header(path)
    assert n == 1_000_000 and len(names) == 35
    assert os.path.getsize(path) == off + 1_000_000 * 35 * 4
    for k in ply.NAMES:
        assert torch.equal(q[k], p[k].reshape(p[k].shape[0], -1)), k


def test_model_drop_ins(tmp_path):
    p = scene(500, 7, 4)
    m = types.SimpleNamespace()
    for k, v in p.items():
        setattr(m, "_" + k, torch.nn.Parameter(torch.from_numpy(v.astype(np.float32)).to(DEV)))
    path = str(tmp_path / "m.ply")
    ply.save_model_ply(m, path)
    m2 = types.SimpleNamespace()
    ply.load_model_ply(m2, path)
    for k in ply.NAMES:
        a, b = getattr(m, "_" + k), getattr(m2, "_" + k)
        assert isinstance(b, torch.nn.Parameter) and b.requires_grad
        assert torch.equal(a, b), k


def test_empty_scene(tmp_path):
    p = {k: torch.empty(0, w, device=DEV) for k, w in
         (("xyz", 3), ("mean", 3), ("rgb", 3), ("opacity", 1), ("beta", 4), ("scale", 6),
          ("l_triangle", 15))}
    path = str(tmp_path / "e.ply")
    ply.save_ply(path, p)
    q = ply.load_ply(path, DEV)
    assert all(q[k].shape == p[k].shape for k in ply.NAMES)
