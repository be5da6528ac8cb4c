"""HostFedStep: steps fed from pinned host memory with the next step's copies
overlapping the current step's compute.  Each step's loss must be the loss of
the inputs fed for that step, whatever ran on the other buffer set."""
import pytest
import torch

from ubs import scene as S
from ubs.render import HostFedStep, Renderer, Views

pytestmark = pytest.mark.gpu
DEV = "cuda"
W, H = 128, 96


def test_each_step_sees_its_own_inputs():
    base = S.synthetic_params(20_000, 6, seed=1, xyz_range=1.0, device=DEV)
    cam = S.orbit_view(2, 3.0, W, H, 100.0, 100.0, device=DEV)
    views = Views([cam], device=DEV)
    g = torch.Generator().manual_seed(0)
    feeds_host = []
    for i in range(6):  # six different parameter sets and targets
        hp = {k: (v.detach().cpu() + 0.01 * i * torch.randn(v.shape, generator=g)).pin_memory()
              for k, v in base.items()}
        tgt = torch.rand(W * H, 3, generator=g).pin_memory()
        feeds_host.append((hp, tgt))
    names = list(base)

    def make_inputs():
        q = {k: torch.nn.Parameter(v.detach().clone()) for k, v in base.items()}
        t = torch.zeros(W * H, 3, device=DEV)
        return q, [q[k] for k in names] + [t], lambda c, a: (c - t).abs().mean()

    hf = HostFedStep(Renderer(dim=6), views, None, make_inputs)
    for _ in range(2):  # the same sequence twice: rings and events wrap
        for hp, tgt in feeds_host:
            hf.step([hp[k] for k in names] + [tgt])
        got = hf.losses()
        r = Renderer(dim=6)
        for (hp, tgt), loss in zip(feeds_host, got):
            with torch.no_grad():
                c, _ = r.render({k: v.to(DEV) for k, v in hp.items()}, views, None)
            want = float((c - tgt.to(DEV)).abs().mean())
            assert abs(loss - want) <= 1e-6 * max(1.0, abs(want)), (loss, want)
    hf.check()
