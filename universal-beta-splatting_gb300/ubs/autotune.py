"""Tile-size autotuner for the fused render.

The tile size sets the whole launch geometry of the blend: a tile of TS x TS
pixels is one CTA of TS*TS/2 threads (two pixels each), its batch of staged
records is TS*TS entries, and with the shared memory that batch needs it
fixes how many CTAs fit on an SM.  It also changes the intersection count
(smaller tiles: more buckets, fewer wasted pixels per record).  Which size is
fastest depends on the resolution mix and the scene's footprint sizes, so it
is measured: each candidate runs the caller's step a few times after a
warm-up, timed with CUDA events on the launching stream, and the fastest is
cached under a caller-chosen key (for example the scene and the view shapes).
"""
from typing import Callable, Dict, Hashable, Sequence, Tuple

import torch

CANDIDATES = (8, 16, 32)


class TileAutotuner:
    def __init__(self, candidates: Sequence[int] = CANDIDATES, warmup: int = 2, reps: int = 5):
        self.candidates = tuple(candidates)
        self.warmup = warmup
        self.reps = reps
        self.cache: Dict[Hashable, Tuple[int, Dict[int, float]]] = {}

    def pick(self, key: Hashable, step: Callable[[int], None]) -> int:
        """Fastest tile size for `key`; `step(tile_size)` runs one render
        (forward or forward + backward) with that tile size."""
        if key in self.cache:
            return self.cache[key][0]
        times = {}
        for ts in self.candidates:
            for _ in range(self.warmup):
                step(ts)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(self.reps):
                step(ts)
            e1.record()
            e1.synchronize()
            times[ts] = e0.elapsed_time(e1) / self.reps
        best = min(times, key=times.get)
        self.cache[key] = (best, times)
        return best

    def timings(self, key: Hashable) -> Dict[int, float]:
        return dict(self.cache[key][1])
