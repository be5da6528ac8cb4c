"""The continuous-batching server returns, for every request, the image the
request gets when rendered alone (max abs difference 1e-5, the blend
tolerance), whatever batch and stream it shared; also when undersized
intersection estimates force batches to be re-run."""
import pytest
import torch

from ubs import scene as S
from ubs.render import Renderer, Views
from ubs.serve import Request, ServeConfig, Server, latency_stats, poisson_trace

pytestmark = pytest.mark.gpu
DEV = "cuda"
RES = [(160, 120), (320, 240), (256, 144)]


def scenes():
    out = {}
    for name, n, d, seed in (("small6", 20000, 6, 1), ("mid6", 50000, 6, 2), ("dyn7", 30000, 7, 3)):
        p = S.synthetic_params(n, d, seed=seed, xyz_range=1.0, device=DEV)
        p["scale"][:, :3] += 1.0
        out[name] = p
    return out


def alone(p, cam):
    r = Renderer(dim=p["scale"].shape[1])
    with torch.no_grad():
        colors, _ = r.render(p, Views([cam], device=DEV), torch.zeros(1, 3, device=DEV))
    return colors.view(cam.height, cam.width, 3).cpu()


def trace(n, seed):
    tr = poisson_trace(1000.0, 10.0, ["small6", "mid6", "dyn7"], RES, seed=seed, radius=3.0,
                       focal_per_width=0.9, device=DEV)[:n]
    for i, r in enumerate(tr):
        r.camera.timestamp = (i % 7) / 7.0
    return tr


@pytest.mark.parametrize("margin", [1.5, 0.02])
def test_served_images_equal_alone(margin):
    sc = scenes()
    cfg = ServeConfig(max_slots=3, max_batch_views=4, mem_budget=4 << 30, margin=margin,
                      keep_images=True)
    srv = Server(sc, cfg)
    tr = trace(30, seed=5)
    done = srv.run(tr, realtime=False)
    assert sorted(d.rid for d in done) == list(range(len(tr)))
    assert max(d.batch_size for d in done) > 1  # requests were batched together
    if margin < 1:
        assert srv.reruns > 0
    by_id = {r.rid: r for r in tr}
    for d in done:
        r = by_id[d.rid]
        ref = alone(sc[r.scene], r.camera)
        assert d.image.shape == ref.shape
        assert float((d.image - ref).abs().max()) <= 1e-5, d.rid


def test_realtime_trace_latency():
    sc = scenes()
    srv = Server(sc, ServeConfig(max_slots=3, max_batch_views=4))
    srv.calibrate({k: S.orbit_view(0, 3.0, 320, 240, 288.0, 288.0, device=DEV) for k in sc})
    tr = poisson_trace(200.0, 0.5, list(sc), RES, seed=9, radius=3.0, focal_per_width=0.9,
                       device=DEV)
    done = srv.run(tr, realtime=True)
    st = latency_stats(done)
    assert st["requests"] == len(tr) and 0 < st["p50_ms"] <= st["p99_ms"] < 1000


def test_scene_loaded_from_ply_serves_the_same_images(tmp_path):
    """Server.load_scene (the reference's PLY file, unpacked on the device)
    serves exactly what the same scene served from memory does."""
    from ubs import ply
    p = S.synthetic_params(20000, 7, seed=4, xyz_range=1.0, device=DEV)
    p["scale"][:, :3] += 1.0
    path = str(tmp_path / "scene.ply")
    ply.save_ply(path, p)
    cfg = ServeConfig(max_slots=2, max_batch_views=4, mem_budget=2 << 30, keep_images=True)
    a = Server({"s": p}, cfg)
    b = Server({}, cfg)
    b.load_scene("s", path)
    tr = poisson_trace(1000.0, 10.0, ["s"], RES, seed=6, radius=3.0, focal_per_width=0.9,
                       device=DEV)[:8]
    da = {d.rid: d.image for d in a.run(tr, realtime=False)}
    db = {d.rid: d.image for d in b.run(tr, realtime=False)}
    assert sorted(da) == sorted(db) == list(range(8))
    for rid in da:
        assert torch.equal(da[rid], db[rid]), rid
