"""Selection and caching of the launch-geometry autotuner (host logic, a fake
timer; no GPU)."""
from ubs.autotune import TileAutotuner


def make(costs, **kw):
    """Tuner whose timer returns costs[(tile, fwd, bwd)] for the variant
    applied last; records the applied variants and the configs timed."""
    state = {"variant": (0, 0), "applied": [], "timed": []}

    def apply_variant(f, b):
        state["variant"] = (f, b)
        state["applied"].append((f, b))

    def timer(fn, warmup, reps):
        cfg = (fn(),) + state["variant"]  # the step returns its tile size here
        state["timed"].append(cfg)
        return costs[cfg]

    return TileAutotuner(timer=timer, apply_variant=apply_variant, **kw), state


def step(ts):
    return ts


def test_tile_then_variants_and_cache():
    costs = {(8, 0, 0): 5.0, (16, 0, 0): 4.0, (32, 0, 0): 6.0,
             (16, 1, 0): 3.5, (16, 2, 0): 4.2, (16, 0, 1): 3.9, (16, 0, 2): 4.5,
             (16, 1, 1): 3.3}
    tuner, st = make(costs)
    assert tuner.pick("k", step) == 16
    assert tuner.choice("k") == (16, 1, 1)
    assert st["variant"] == (1, 1)  # the winner is left applied
    # every config measured once, the combination last
    assert sorted(st["timed"]) == sorted(costs) and st["timed"][-1] == (16, 1, 1)
    n = len(st["timed"])
    assert tuner.pick("k", step) == 16 and len(st["timed"]) == n  # cached: no new timing
    assert tuner.timings("k")[(32, 0, 0)] == 6.0


def test_large_tiles_have_no_variants():
    costs = {(8, 0, 0): 5.0, (16, 0, 0): 4.0, (32, 0, 0): 2.0}
    tuner, st = make(costs)
    assert tuner.pick("k", step) == 32
    assert tuner.choice("k") == (32, 0, 0) and len(st["timed"]) == 3


def test_combination_slower_than_a_single_variant_is_not_chosen():
    costs = {(8, 0, 0): 5.0, (16, 0, 0): 4.0, (32, 0, 0): 6.0,
             (16, 1, 0): 3.0, (16, 2, 0): 4.2, (16, 0, 1): 3.5, (16, 0, 2): 4.5,
             (16, 1, 1): 3.8}
    tuner, st = make(costs)
    tuner.pick("k", step)
    assert tuner.choice("k") == (16, 1, 0) and st["variant"] == (1, 0)
