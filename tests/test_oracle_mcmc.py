"""Pin the oracle's MCMC densification against the reference's own
BetaModel.relocate_gs / add_new_gs (tests/golden/make_mcmc_golden.py ran
them on the CPU and recorded the indices torch.multinomial drew).  CPU only."""
import os

import numpy as np
import pytest

import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mcmc.npz")


def load(z, prefix):
    params = {k: z[prefix + k] for k in orc.MCMC_NAMES}
    moments = {k: (z[prefix + "m_" + k], z[prefix + "v_" + k]) for k in orc.MCMC_NAMES}
    return params, moments


def check(got, want, op_tol):
    (p, m), (wp, wm) = got, want
    for k in orc.MCMC_NAMES:
        assert p[k].shape == wp[k].shape, k
        if k == "opacity":  # FP32 sigmoid / pow / log: an ulp or two
            assert np.allclose(p[k], wp[k], rtol=op_tol, atol=op_tol), k
        else:
            assert np.array_equal(p[k], wp[k]), k
        assert np.array_equal(m[k][0], wm[k][0]) and np.array_equal(m[k][1], wm[k][1]), k


@pytest.mark.parametrize("D", [6, 7])
def test_relocate_and_add_match_reference(D):
    z = np.load(GOLD)
    t = "d%d_" % D
    params, moments = load(z, t + "in_")
    dead = z[t + "dead"]
    src = z[t + "reloc_src"]
    assert len(src) == dead.sum() and not dead[src].any()
    got = orc.mcmc_relocate(params, moments, dead, src)
    check(got, load(z, t + "reloc_"), 2e-6)
    n_new = int(z[t + "n_new"])
    assert n_new == orc.mcmc_add_count(len(dead), 10_000)
    got2 = orc.mcmc_add(*load(z, t + "reloc_"), z[t + "add_src"])
    check(got2, load(z, t + "add_"), 2e-6)


def test_split_opacity_conserves_coverage():
    """(1 - o')^(count + 1) = 1 - o: the copies together cover what the source did."""
    raw = np.linspace(-4, 4, 41).astype(np.float32)
    for c in (1, 2, 5):
        new = orc.mcmc_split_opacity(raw, np.full(raw.shape, c))
        o = 1 / (1 + np.exp(-raw.astype(np.float64)))
        o2 = 1 / (1 + np.exp(-new.astype(np.float64)))
        keep = (o2 > 0.0051) & (o2 < 0.999)
        assert np.allclose((1 - o2[keep]) ** (c + 1), 1 - o[keep], rtol=1e-4)


def test_add_count():
    assert orc.mcmc_add_count(1000, 10_000) == 20
    assert orc.mcmc_add_count(1000, 1010) == 10
    assert orc.mcmc_add_count(1000, 900) == 0
