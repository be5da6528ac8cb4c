"""Autotuner of the fused render's launch geometry: tile size and the blend
kernels' occupancy variant (blocks per SM).

The tile size sets the whole launch geometry of the blend: a tile of TS x TS
pixels is one CTA of TS*TS/2 threads (two pixels each), its batch of staged
records is TS*TS entries, and with the shared memory that batch needs it
fixes how many CTAs fit on an SM.  It also changes the intersection count
(smaller tiles: more buckets, fewer wasted pixels per record).  For tiles up
to 16 x 16 the blend kernels are compiled in variants (ubs_set_blend_variant,
for the forward and the backward separately: the forward's trade records per
staged batch against CTAs per SM, the backward's its register bound and how a
batch's per-record gradient sums are accumulated).  Which point is fastest depends on the
resolution mix and the scene's footprint sizes, so it is measured: each
candidate runs the caller's step a few times after a warm-up, timed with CUDA
events on the launching stream, and the winner is cached under a
caller-chosen key (for example the scene and the view shapes).

Search: the tile sizes at the default variant; then, at the best tile size
when it has variants, each forward variant with the default backward and
each backward variant with the default forward (they are different kernels
of the step), then the best forward and backward together.  The winning
variant is left set process-wide.
"""
from typing import Callable, Dict, Hashable, Optional, Sequence, Tuple

CANDIDATES = (8, 16, 32)
FWD_VARIANTS = (0, 1, 2)
BWD_VARIANTS = (0, 1, 2)
VARIANT_MAX_TILE = 16  # tiles of at most 16 x 16 pixels have occupancy variants

Config = Tuple[int, int, int]  # (tile size, forward variant, backward variant)


def set_blend_variant(forward: int, backward: int) -> None:
    """Select the blend kernels' occupancy variant (process-wide)."""
    from . import _lib as L
    L.call("ubs_set_blend_variant", int(forward), int(backward))


def get_blend_variant() -> Tuple[int, int]:
    import ctypes
    from . import _lib as L
    f, b = ctypes.c_int32(), ctypes.c_int32()
    L.call("ubs_get_blend_variant", ctypes.byref(f), ctypes.byref(b))
    return int(f.value), int(b.value)


def cuda_event_timer(fn: Callable[[], None], warmup: int, reps: int) -> float:
    """Milliseconds per call of fn: warm-up calls, then reps calls between two
    CUDA events on the current stream."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


class TileAutotuner:
    def __init__(self, candidates: Sequence[int] = CANDIDATES,
                 fwd_variants: Sequence[int] = FWD_VARIANTS,
                 bwd_variants: Sequence[int] = BWD_VARIANTS, warmup: int = 2, reps: int = 5,
                 timer: Optional[Callable] = None, apply_variant: Optional[Callable] = None):
        self.candidates = tuple(candidates)
        self.fwd_variants = tuple(fwd_variants)
        self.bwd_variants = tuple(bwd_variants)
        self.warmup = warmup
        self.reps = reps
        self.timer = timer or cuda_event_timer
        self.apply_variant = apply_variant or set_blend_variant
        self.cache: Dict[Hashable, Tuple[Config, Dict[Config, float]]] = {}

    def _time(self, cfg: Config, step, times: Dict[Config, float]) -> float:
        if cfg not in times:
            ts, f, b = cfg
            self.apply_variant(f, b)
            times[cfg] = self.timer(lambda: step(ts), self.warmup, self.reps)
        return times[cfg]

    def pick(self, key: Hashable, step: Callable[[int], None]) -> int:
        """Fastest tile size for `key`, leaving its best blend variant set;
        `step(tile_size)` runs one render (forward or forward + backward)
        with that tile size."""
        if key not in self.cache:
            times: Dict[Config, float] = {}
            for ts in self.candidates:
                self._time((ts, 0, 0), step, times)
            ts = min(times, key=times.get)[0]
            if ts <= VARIANT_MAX_TILE:
                for f in self.fwd_variants:
                    self._time((ts, f, 0), step, times)
                for b in self.bwd_variants:
                    self._time((ts, 0, b), step, times)
                f = min(self.fwd_variants, key=lambda v: times[(ts, v, 0)])
                b = min(self.bwd_variants, key=lambda v: times[(ts, 0, v)])
                self._time((ts, f, b), step, times)
            best = min(times, key=times.get)
            self.cache[key] = (best, times)
        best = self.cache[key][0]
        self.apply_variant(best[1], best[2])
        return best[0]

    def choice(self, key: Hashable) -> Config:
        """(tile size, forward variant, backward variant) picked for `key`."""
        return self.cache[key][0]

    def timings(self, key: Hashable) -> Dict[Config, float]:
        return dict(self.cache[key][1])
