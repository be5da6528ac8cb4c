"""Golden vectors for MCMC densification from the reference's own BetaModel.

BetaModel.relocate_gs / add_new_gs (scene/beta_model.py:553-658) move dead
primitives onto opacity-sampled live ones and append new ones, splitting the
sampled primitives' opacity and resetting their Adam moments.  This script
loads scene/beta_model.py from a checkout of the reference on the CPU, with
stub modules standing in for the packages absent here (plyfile, matplotlib,
the viewer) that these methods never touch, builds a small model with a
torch.optim.Adam carrying non-zero moments, runs relocate_gs and add_new_gs,
records the indices torch.multinomial drew (by wrapping _sample_alives) and
stores inputs, drawn indices and outputs in mcmc.npz next to this script.

Usage:  python tests/golden/make_mcmc_golden.py /path/to/reference
"""
import importlib.util
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("UBS_REFERENCE_ROOT")
if not REF:
    sys.exit("usage: %s /path/to/reference (or set UBS_REFERENCE_ROOT)" % sys.argv[0])
NAMES = ["xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle"]


def load_beta_model():
    for name in ("matplotlib", "matplotlib.pyplot", "plyfile"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib"].colormaps = {}
    sys.modules["plyfile"].PlyData = sys.modules["plyfile"].PlyElement = object
    pkg = types.ModuleType("scene")
    pkg.__path__ = [os.path.join(REF, "scene")]
    sys.modules["scene"] = pkg
    viewer = types.ModuleType("scene.beta_viewer")
    viewer.BetaRenderTabState = object
    sys.modules["scene.beta_viewer"] = viewer
    sys.path.insert(0, REF)
    sys.path.insert(0, os.path.join(REF, "submodules"))
    spec = importlib.util.spec_from_file_location("scene.beta_model",
                                                  os.path.join(REF, "scene", "beta_model.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.BetaModel


def make_model(BetaModel, g, N, D):
    m = object.__new__(BetaModel)
    m.input_dim = D
    m.setup_functions()
    shapes = {"xyz": 3, "mean": D - 3, "rgb": 3, "opacity": 1, "beta": D - 2, "scale": D,
              "l_triangle": D * (D - 1) // 2}
    # values on a 2^-8 grid (exact in float32) keep the fixture small
    q = lambda t: torch.round(t * 256) / 256  # noqa: E731
    raw = {k: q(torch.randn(N, c, generator=g)) for k, c in shapes.items()}
    # a spread of opacities with some at or below the 0.005 death threshold
    raw["opacity"] = q(torch.randn(N, 1, generator=g) * 2.5 - 1.0)
    raw["opacity"][: N // 10] = -7.0
    for k in NAMES:
        setattr(m, "_" + k, torch.nn.Parameter(raw[k].clone()))
    groups = [{"params": [getattr(m, "_" + k)], "lr": 1e-3, "name": k} for k in NAMES]
    m.optimizer = torch.optim.Adam(groups, lr=0.0, eps=1e-15)
    for k in NAMES:  # non-zero moments and a step count, as mid-training
        p = getattr(m, "_" + k)
        st = m.optimizer.state[p]
        st["step"] = torch.tensor(7.0)
        st["exp_avg"] = q(torch.randn(p.shape, generator=g)) * 2.0 ** -10
        st["exp_avg_sq"] = q(torch.rand(p.shape, generator=g)) * 2.0 ** -20
    return m


def snapshot(m, prefix, out):
    for k in NAMES:
        p = getattr(m, "_" + k)
        st = m.optimizer.state[p]
        out[prefix + k] = p.detach().numpy().copy()
        out[prefix + "m_" + k] = st["exp_avg"].numpy().copy()
        out[prefix + "v_" + k] = st["exp_avg_sq"].numpy().copy()


def main():
    BetaModel = load_beta_model()
    drawn = []
    orig = BetaModel._sample_alives

    def recording(self, probs, num, alive_indices=None):
        idx, ratio = orig(self, probs, num, alive_indices)
        drawn.append(idx.clone())
        return idx, ratio

    BetaModel._sample_alives = recording
    out = {}
    for D in (6, 7):
        g = torch.Generator().manual_seed(D)
        torch.manual_seed(100 + D)
        m = make_model(BetaModel, g, 120, D)
        tag = "d%d_" % D
        snapshot(m, tag + "in_", out)
        dead = (m.get_opacity <= 0.005).squeeze(-1)
        out[tag + "dead"] = dead.numpy()
        drawn.clear()
        with torch.no_grad():  # as train.py:129-170 calls them
            m.relocate_gs(dead_mask=dead)
        out[tag + "reloc_src"] = drawn[0].numpy().astype(np.int64)
        snapshot(m, tag + "reloc_", out)
        drawn.clear()
        with torch.no_grad():
            n_new = m.add_new_gs(cap_max=10_000)
        out[tag + "add_src"] = drawn[0].numpy().astype(np.int64)
        out[tag + "n_new"] = np.int64(n_new)
        snapshot(m, tag + "add_", out)
    np.savez_compressed(os.path.join(HERE, "mcmc.npz"), **out)
    print("wrote mcmc.npz", {k: v.shape for k, v in out.items() if "src" in k or "dead" in k})


if __name__ == "__main__":
    main()
