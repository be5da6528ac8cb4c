"""FusedAdam against torch.optim.Adam (the reference's optimizer,
scene/beta_model.py:239-276: seven parameter groups, eps 1e-15, the xyz
learning rate rescheduled every iteration): parameters and moments after
several steps agree to FP32 rounding, the state can be replaced the way the
reference's densification code does, and a captured launch follows prepare()."""
import pytest
import torch

from ubs import scene as S
from ubs.optim import FusedAdam

pytestmark = pytest.mark.gpu
DEV = "cuda"
LRS = {"xyz": 1.6e-4, "mean": 2e-3, "rgb": 2.5e-3, "opacity": 5e-2, "beta": 5e-3,
       "scale": 5e-3, "l_triangle": 1e-3}


def groups(params):
    return [{"params": [params[k]], "lr": lr, "name": k} for k, lr in LRS.items()]


def twin_params(n=5000, seed=0):
    base = S.synthetic_params(n, 6, seed=seed, device=DEV)
    a = {k: torch.nn.Parameter(v.clone()) for k, v in base.items()}
    b = {k: torch.nn.Parameter(v.clone()) for k, v in base.items()}
    return a, b


def rel(x, y):
    return float((x - y).abs().max() / y.abs().max().clamp_min(1e-30))


def test_fused_adam_matches_torch_adam():
    pa, pb = twin_params()
    ref = torch.optim.Adam(groups(pa), lr=0.0, eps=1e-15)
    ours = FusedAdam(groups(pb), lr=0.0, eps=1e-15)
    g = torch.Generator(device=DEV).manual_seed(0)
    for it in range(6):
        for k in pa:
            grad = torch.randn(pa[k].shape, generator=g, device=DEV) * (0.1 if it % 2 else 10.0)
            pa[k].grad = grad.clone()
            pb[k].grad = grad.clone()
        for opt in (ref, ours):  # the reference reschedules xyz every iteration
            opt.param_groups[0]["lr"] = LRS["xyz"] * (0.9 ** it)
        ref.step()
        ours.step()
        torch.cuda.synchronize()
        for k in pa:
            assert rel(pb[k].data, pa[k].data) < 1e-6, (it, k)
            sa, sb = ref.state[pa[k]], ours.state[pb[k]]
            assert rel(sb["exp_avg"], sa["exp_avg"]) < 1e-6, (it, k)
            assert rel(sb["exp_avg_sq"], sa["exp_avg_sq"]) < 1e-6, (it, k)
            assert float(sb["step"]) == float(sa["step"])


def test_state_replacement_like_densification():
    """Replacing a parameter and its moments (beta_model.py:406-419) is picked up."""
    pa, pb = twin_params(2000, 1)
    ours = FusedAdam(groups(pb), lr=0.0, eps=1e-15)
    ref = torch.optim.Adam(groups(pa), lr=0.0, eps=1e-15)
    for opt, params in ((ref, pa), (ours, pb)):
        for v in params.values():
            v.grad = torch.ones_like(v)
        opt.step()
        # replace the opacity tensor, resetting its moments
        group = next(gr for gr in opt.param_groups if gr["name"] == "opacity")
        old = group["params"][0]
        state = opt.state.pop(old)
        state["exp_avg"] = torch.zeros_like(old)
        state["exp_avg_sq"] = torch.zeros_like(old)
        new = torch.nn.Parameter(old.detach().clone() * 0.5)
        group["params"][0] = new
        opt.state[new] = state
        params["opacity"] = new
        for v in params.values():
            v.grad = torch.full_like(v, 0.3)
        opt.step()
    torch.cuda.synchronize()
    for k in pa:
        assert rel(pb[k].data, pa[k].data) < 1e-6, k


def test_captured_launch_follows_prepare():
    pa, pb = twin_params(3000, 2)
    ref = torch.optim.Adam(groups(pa), lr=0.0, eps=1e-15)
    ours = FusedAdam(groups(pb), lr=0.0, eps=1e-15)
    for params in (pa, pb):
        for v in params.values():
            v.grad = torch.full_like(v, 0.5)
    ref.step()
    ours.step()  # initialises the state and the table outside the graph
    ours.prepare()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph):
            ours.launch()
    torch.cuda.current_stream().wait_stream(side)
    graph.replay()  # step 2 (prepared above)
    ref.step()
    for it in range(3):
        for opt in (ref, ours):
            opt.param_groups[0]["lr"] = LRS["xyz"] * (0.5 + it)
        ours.prepare()
        graph.replay()
        ref.step()
    torch.cuda.synchronize()
    for k in pa:
        assert rel(pb[k].data, pa[k].data) < 1e-6, k


def test_graphed_step_with_fused_adam_matches_eager_training():
    """Render + L1 + backward + Adam as one graph, three iterations, against
    the same iterations eagerly with torch.optim.Adam."""
    from ubs.render import GraphedStep, Renderer, Views
    base = S.synthetic_params(4000, 6, seed=7, xyz_range=1.0, device=DEV)
    base["scale"][:, :3] += 1.5
    pa = {k: torch.nn.Parameter(v.clone()) for k, v in base.items()}
    pb = {k: torch.nn.Parameter(v.clone()) for k, v in base.items()}
    cam = S.orbit_view(3, 3.0, 200, 150, 180.0, 180.0, device=DEV)
    target = torch.rand(200 * 150, 3, generator=torch.Generator().manual_seed(2)).to(DEV)
    loss_fn = lambda c, a: (c - target).abs().mean()  # noqa: E731
    ref_opt = torch.optim.Adam(groups(pa), lr=0.0, eps=1e-15)
    r_ref = Renderer(dim=6)
    views = Views([cam], device=DEV)

    def eager_iter():
        for v in pa.values():
            v.grad = None
        c, a = r_ref.render(pa, views)
        loss_fn(c, a).backward()
        ref_opt.step()

    opt = FusedAdam(groups(pb), lr=0.0, eps=1e-15)
    gs = GraphedStep(Renderer(dim=6), pb, views, None, loss_fn, optimizer=opt, warmup=2)
    for _ in range(2):  # the warm-up iterations of the graphed step
        eager_iter()
    for _ in range(3):
        gs.replay()
        eager_iter()
    gs.check()
    torch.cuda.synchronize()
    for k in pa:
        assert rel(pb[k].data, pa[k].data) < 1e-5, k


@pytest.mark.parametrize("n_tensors", [5, 80])
def test_ragged_unaligned_and_many_tensors(n_tensors):
    """Odd sizes (scalar tails), parameters that are views 4 bytes into their
    storage (no 16-byte accesses), and more tensors than the flattened
    launch takes (the per-tensor grid)."""
    g = torch.Generator(device=DEV).manual_seed(3)
    sizes = [(i * 7919) % 20011 + 1 for i in range(n_tensors)]
    pa, pb = [], []
    for i, n in enumerate(sizes):
        base = torch.randn(n + 1, generator=g, device=DEV)
        if i % 2:  # a view one float into its storage
            a = torch.nn.Parameter(base.clone()[1:])
            b = torch.nn.Parameter(base.clone()[1:])
        else:
            a = torch.nn.Parameter(base[:n].clone())
            b = torch.nn.Parameter(base[:n].clone())
        pa.append(a)
        pb.append(b)
    ga = [{"params": [p], "lr": 1e-3 * (1 + i % 3)} for i, p in enumerate(pa)]
    gb = [{"params": [p], "lr": 1e-3 * (1 + i % 3)} for i, p in enumerate(pb)]
    ref = torch.optim.Adam(ga, lr=0.0, eps=1e-15)
    ours = FusedAdam(gb, lr=0.0, eps=1e-15)
    for it in range(4):
        for a, b in zip(pa, pb):
            grad = torch.randn(a.shape, generator=g, device=DEV)
            a.grad = grad.clone()
            b.grad = grad.clone()
        ref.step()
        ours.step()
    torch.cuda.synchronize()
    for a, b in zip(pa, pb):
        assert rel(b.data, a.data) < 1e-6
        assert rel(ours.state[b]["exp_avg_sq"], ref.state[a]["exp_avg_sq"]) < 1e-6
