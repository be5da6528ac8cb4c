"""MCMC densification kernels (ubs.mcmc) against the oracle, which is pinned
to the reference's own BetaModel.relocate_gs / add_new_gs
(tests/golden/mcmc.npz): with the reference's draws given, copies and Adam
moments match bit for bit and split opacities within 1e-5 (FP32 sigmoid, pow
and log with the device's fast intrinsics); the device sampler is checked
for its distribution; the whole relocation runs inside a CUDA graph."""
import os
import types

import numpy as np
import pytest
import torch

import oracle as orc
from ubs import mcmc

pytestmark = pytest.mark.gpu
DEV = "cuda"
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mcmc.npz")


def model_from(z, prefix):
    m = types.SimpleNamespace()
    groups = []
    for k in orc.MCMC_NAMES:
        p = torch.nn.Parameter(torch.from_numpy(z[prefix + k]).to(DEV))
        setattr(m, "_" + k, p)
        groups.append({"params": [p], "lr": 1e-3, "name": k})
    m.optimizer = torch.optim.Adam(groups, lr=0.0, eps=1e-15)
    for k in orc.MCMC_NAMES:
        st = m.optimizer.state[getattr(m, "_" + k)]
        st["step"] = torch.tensor(7.0)
        st["exp_avg"] = torch.from_numpy(z[prefix + "m_" + k]).to(DEV)
        st["exp_avg_sq"] = torch.from_numpy(z[prefix + "v_" + k]).to(DEV)
    return m


def check(m, z, prefix):
    for k in orc.MCMC_NAMES:
        p = getattr(m, "_" + k)
        want = z[prefix + k]
        got = p.detach().cpu().numpy()
        assert got.shape == want.shape, k
        if k == "opacity":
            assert np.allclose(got, want, rtol=1e-5, atol=1e-5), np.abs(got - want).max()
        else:
            assert np.array_equal(got, want), k
        st = m.optimizer.state[p]
        assert np.array_equal(st["exp_avg"].cpu().numpy(), z[prefix + "m_" + k]), k
        assert np.array_equal(st["exp_avg_sq"].cpu().numpy(), z[prefix + "v_" + k]), k
        assert any(g["params"][0] is p for g in m.optimizer.param_groups)


@pytest.mark.parametrize("D", [6, 7])
def test_reference_draws_reproduce_the_reference(D):
    z = np.load(GOLD)
    t = "d%d_" % D
    m = model_from(z, t + "in_")
    dead = torch.from_numpy(z[t + "dead"]).to(DEV)
    st = mcmc.relocate_gs(m, dead, src=torch.from_numpy(z[t + "reloc_src"]))
    check(m, z, t + "reloc_")
    n = mcmc.add_new_gs(m, 10_000, src=torch.from_numpy(z[t + "add_src"]))
    assert n == int(z[t + "n_new"])
    check(m, z, t + "add_")
    assert int(st.item()) == 0


def synthetic(N, seed, dead_frac=0.3):
    g = torch.Generator().manual_seed(seed)
    m = types.SimpleNamespace()
    shapes = {"xyz": 3, "mean": 3, "rgb": 3, "opacity": 1, "beta": 4, "scale": 6,
              "l_triangle": 15}
    vals = {k: torch.randn(N, c, generator=g) for k, c in shapes.items()}
    vals["xyz"][:, 0] = torch.arange(N, dtype=torch.float32)  # identifies a row's origin
    op = torch.randn(N, 1, generator=g) * 2
    op[torch.rand(N, generator=g) < dead_frac] = -8.0
    vals["opacity"] = op
    groups = []
    for k in orc.MCMC_NAMES:
        p = torch.nn.Parameter(vals[k].to(DEV))
        setattr(m, "_" + k, p)
        groups.append({"params": [p], "lr": 1e-3, "name": k})
    m.optimizer = torch.optim.Adam(groups, lr=0.0, eps=1e-15)
    for k in orc.MCMC_NAMES:
        p = getattr(m, "_" + k)
        st = m.optimizer.state[p]
        st["step"] = torch.tensor(3.0)
        st["exp_avg"] = torch.full_like(p, 0.5)
        st["exp_avg_sq"] = torch.full_like(p, 0.25)
    return m, vals


def test_device_draws_relocate_dead_onto_live():
    N = 5000
    m, vals = synthetic(N, 1)
    op0 = vals["opacity"][:, 0].numpy()
    dead = 1 / (1 + np.exp(-op0.astype(np.float64))) <= 0.005
    torch.manual_seed(0)
    mcmc.relocate_gs(m)  # threshold on the device
    xyz = m._xyz.detach().cpu().numpy()
    src = xyz[dead, 0].astype(np.int64)
    assert not dead[src].any()                      # every source is live
    # the rest of each dead row is its source's
    for k in ("mean", "rgb", "beta", "scale", "l_triangle"):
        got = getattr(m, "_" + k).detach().cpu().numpy()
        assert np.array_equal(got[dead], vals[k].numpy()[src]), k
        assert np.array_equal(got[~dead & ~np.isin(np.arange(N), src)],
                              vals[k].numpy()[~dead & ~np.isin(np.arange(N), src)]), k
    # then the oracle, given these draws, agrees everywhere
    params = {k: vals[k].numpy() for k in orc.MCMC_NAMES}
    moments = {k: (np.full(vals[k].shape, 0.5, np.float32), np.full(vals[k].shape, 0.25,
                                                                      np.float32))
               for k in orc.MCMC_NAMES}
    op, mom = orc.mcmc_relocate(params, moments, dead, src)
    assert np.allclose(m._opacity.detach().cpu().numpy(), op["opacity"], rtol=1e-5, atol=1e-5)
    for k in orc.MCMC_NAMES:
        st = m.optimizer.state[getattr(m, "_" + k)]
        assert np.array_equal(st["exp_avg"].cpu().numpy(), mom[k][0]), k


def test_draw_distribution_follows_opacity():
    """200k draws over 16 primitives: frequencies against sigmoid(opacity) /
    sum (chi-square, 15 degrees of freedom, bound at p ~ 1e-4)."""
    m, vals = synthetic(16, 2, dead_frac=0.0)
    # add_new_gs draws 2% at a time; the C entry point takes any count
    import ctypes
    from ubs import _lib as L
    params = mcmc._params(m)
    moments = [(None, None)] * len(params)
    n_add = 200_000
    grown = [torch.empty((16 + n_add,) + tuple(p.shape[1:]), device=DEV) for p in params]
    s_old, s_new = mcmc._set(params, moments), mcmc._set(grown, moments)
    ws = L.workspace(L.query("ubs_mcmc_workspace_bytes", 16, n_add), DEV)
    st = torch.zeros(1, dtype=torch.int32, device=DEV)
    L.call("ubs_mcmc_add", ctypes.byref(s_old), ctypes.byref(s_new), 16, n_add, 12345, None,
           L.ptr(st), L.ptr(ws), ws.numel(), L.stream(DEV))
    src = grown[0][16:, 0].cpu().numpy().astype(np.int64)
    freq = np.bincount(src, minlength=16)
    w = 1 / (1 + np.exp(-vals["opacity"][:, 0].double().numpy()))
    expect = n_add * w / w.sum()
    chi2 = float(((freq - expect) ** 2 / expect).sum())
    assert chi2 < 45.0, (chi2, freq, expect)


def test_relocation_runs_inside_a_cuda_graph():
    N = 3000
    m, vals = synthetic(N, 3)
    dead_ref = torch.sigmoid(vals["opacity"][:, 0]) <= 0.005
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g):
            mcmc.relocate_gs(m, generator=torch.Generator().manual_seed(5))
    torch.cuda.current_stream().wait_stream(s)
    g.replay()
    torch.cuda.synchronize()
    xyz = m._xyz.detach().cpu().numpy()
    src = xyz[dead_ref.numpy(), 0].astype(np.int64)
    assert not dead_ref.numpy()[src].any()
    assert (torch.sigmoid(m._opacity) > 0.0049).all()


def test_perturb_xyz_given_noise_matches_oracle():
    N = 4000
    m, vals = synthetic(N, 4)
    g = torch.Generator().manual_seed(9)
    noise = torch.randn(N, 3, generator=g)
    with torch.no_grad():  # O(1) positions, so FP32 keeps the small displacement
        m._xyz.copy_(torch.randn(N, 3, generator=g))
    before = m._xyz.detach().cpu().numpy().astype(np.float64)
    mcmc.perturb_xyz(m, 1.6e-4 * 5.0, noise=noise)
    want = orc.mcmc_perturb_xyz(before, vals["opacity"].numpy(), vals["scale"].numpy(),
                                vals["l_triangle"].numpy(), noise.numpy(), 1.6e-4 * 5.0)
    got = m._xyz.detach().cpu().numpy()
    d_got, d_want = got - before, want - before
    scale = np.abs(d_want).max()
    assert np.abs(d_got - d_want).max() <= 1e-4 * scale + 1e-6


def test_perturb_xyz_device_noise_is_standard_normal():
    N = 100_000
    m, _ = synthetic(N, 5)
    with torch.no_grad():
        m._opacity.fill_(-30.0)                   # (1 - o)^100 = 1
        m._scale.fill_(float(np.log(np.e - 1)))   # softplus -> 1
        m._l_triangle.zero_()                     # R = I: Sigma = I
        m._xyz.zero_()
    torch.manual_seed(1)
    mcmc.perturb_xyz(m, 1.0)
    z = m._xyz.detach().cpu().numpy().astype(np.float64).ravel()
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert abs(((z ** 4).mean()) - 3.0) < 0.1   # normal kurtosis


def test_bad_given_draws():
    m, _ = synthetic(50, 6)
    with pytest.raises(ValueError):
        mcmc.add_new_gs(m, 10_000, src=torch.tensor([0, 1, 2]))
    dead = torch.zeros(50, dtype=torch.bool, device=DEV)
    dead[:2] = True
    st = mcmc.relocate_gs(m, dead, src=torch.tensor([10, 999]))
    assert int(st.item()) != 0


def test_relocate_without_live_primitives_changes_nothing():
    """As the reference's early return: nothing to draw from."""
    m, vals = synthetic(300, 9, dead_frac=1.0)
    before = {k: getattr(m, "_" + k).detach().clone() for k in orc.MCMC_NAMES}
    mcmc.relocate_gs(m, torch.ones(300, dtype=torch.bool, device=DEV))
    for k in orc.MCMC_NAMES:
        assert torch.equal(getattr(m, "_" + k), before[k]), k
