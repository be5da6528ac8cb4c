"""The training loop of the reference (train.py:95-171) assembled from this
library's pieces: fused render, the L1 + SSIM loss, backward, FusedAdam, and
every few iterations MCMC relocation, addition and position noise, which
replace the parameter tensors under the optimizer.  The loop must keep
training (finite, falling loss), keep the optimizer attached to the grown
parameters, and match torch.optim.Adam in the same loop."""
import types

import pytest
import torch

from ubs import mcmc
from ubs import scene as S
from ubs.loss import l1_ssim_loss
from ubs.optim import FusedAdam
from ubs.render import Renderer, Views

pytestmark = pytest.mark.gpu
DEV = "cuda"
W, H = 96, 72
NAMES = ("xyz", "mean", "rgb", "opacity", "beta", "scale", "l_triangle")
LRS = {"xyz": 1.6e-4, "mean": 2e-3, "rgb": 2.5e-3, "opacity": 5e-2, "beta": 5e-3,
       "scale": 5e-3, "l_triangle": 1e-3}


def make_model(opt_cls, seed=0):
    p = S.synthetic_params(4000, 6, seed=seed, xyz_range=1.0, device=DEV)
    with torch.no_grad():
        p["scale"][:, :3] += 1.0
        p["opacity"][:400] = -8.0  # some dead primitives for the relocation
    m = types.SimpleNamespace(input_dim=6)
    for k in NAMES:
        setattr(m, "_" + k, torch.nn.Parameter(p[k].contiguous()))
    groups = [{"params": [getattr(m, "_" + k)], "lr": LRS[k], "name": k} for k in NAMES]
    m.optimizer = opt_cls(groups, lr=0.0, eps=1e-15)
    return m


def params_of(m):
    return {"xyz": m._xyz, "mean": m._mean, "scale": m._scale, "l_triangle": m._l_triangle,
            "opacity": m._opacity.view(-1), "beta": m._beta, "rgb": m._rgb}


def run(opt_cls, iters=12):
    torch.manual_seed(0)
    m = make_model(opt_cls)
    cams = [S.orbit_view(i, 3.0, W, H, 80.0, 80.0, device=DEV) for i in range(4)]
    g = torch.Generator().manual_seed(1)
    targets = [torch.rand(1, H, W, 3, generator=g).to(DEV) for _ in cams]
    r = Renderer(dim=6)
    losses, sizes = [], []
    for it in range(iters):
        v = it % len(cams)
        views = Views([cams[v]], device=DEV)
        colors, _ = r.render(params_of(m), views, None)
        loss = l1_ssim_loss(colors.view(1, H, W, 3), targets[v], 0.2, channels_last=True)
        loss.backward()
        losses.append(float(loss))
        if it % 4 == 3:  # densification block of train.py:156-171
            with torch.no_grad():
                dead = (torch.sigmoid(m._opacity) <= 0.005).squeeze(-1)
            mcmc.relocate_gs(m, dead, generator=torch.Generator().manual_seed(it))
            mcmc.add_new_gs(m, cap_max=10_000, generator=torch.Generator().manual_seed(it))
            mcmc.perturb_xyz(m, 1.0 * LRS["xyz"], generator=torch.Generator().manual_seed(it))
        m.optimizer.step()
        m.optimizer.zero_grad(set_to_none=True)
        sizes.append(m._xyz.shape[0])
    return m, losses, sizes


def test_loop_trains_and_keeps_the_optimizer_attached():
    m, losses, sizes = run(FusedAdam)
    assert all(torch.isfinite(torch.tensor(losses)))
    assert sizes[-1] > sizes[0]                      # add_new_gs grew the scene
    for group in m.optimizer.param_groups:           # the grown tensors are optimized
        p = group["params"][0]
        assert p is getattr(m, "_" + group["name"])
        st = m.optimizer.state[p]
        # the iterations that densified replaced the parameters before the
        # step, so those tensors had no gradient to step on (as in train.py)
        assert st["exp_avg"].shape == p.shape and float(st["step"]) == 9
    with torch.no_grad():                            # no dead primitives left behind
        assert (torch.sigmoid(m._opacity) > 0.0049).all()
    # the same views again: the loss went down over the run
    assert sum(losses[-4:]) < sum(losses[:4])


def test_fused_adam_follows_torch_adam():
    """FusedAdam and torch.optim.Adam in the same loop: the same losses until
    the first densification (later, the blend backward's float atomics make
    opacity-driven draws free to differ between runs) and the same growth."""
    _, lf, sf = run(FusedAdam)
    _, lt, st = run(torch.optim.Adam)
    assert sf == st
    for a, b in zip(lf[:4], lt[:4]):
        assert abs(a - b) <= 1e-5 * max(1.0, abs(b))
    assert all(torch.isfinite(torch.tensor(lt)))
