"""FusedAdam: torch.optim.Adam's update in one kernel launch per step.

The reference optimises its seven parameter groups with
torch.optim.Adam(groups, lr=0.0, eps=1e-15) (scene/beta_model.py:239-276) and
reschedules the xyz group's learning rate every iteration (:278-284).  This
optimizer has the same constructor, parameter groups and per-parameter state
(`step` as a float, `exp_avg`, `exp_avg_sq`), so the reference's code that edits
optimizer state when it adds, prunes or relocates primitives
(beta_model.py:406-470) works on it unchanged; the update itself is one
launch of `ubs_adam_step` over every parameter with a gradient.

Only what the reference uses is supported: FP32 CUDA parameters, no weight
decay, no amsgrad, no maximize.

For CUDA-graph capture, `step()` splits into `prepare()` (host: advance the
step counts and upload each tensor's step size and bias correction) and
`launch()` (the kernel on the current stream): capture `launch()` and call
`prepare()` before every replay.
"""
import ctypes
from typing import List

import torch

from . import _lib as L


class FusedAdam(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, weight_decay=0.0):
        if weight_decay != 0.0:
            raise ValueError("FusedAdam: weight decay is not supported")
        super().__init__(params, dict(lr=lr, betas=tuple(betas), eps=eps))
        self._key = None          # data pointers the device table was built for
        self._table_dev = None
        self._table_host = None
        self._hyper_dev = None
        self._hyper_host = None   # ring of pinned buffers
        self._hyper_events = None
        self._ring = 0
        self._entries: List = []

    # ---------------------------------------------------------------- state
    def _active(self):
        """(param, group) of every parameter with a gradient, in group order."""
        out = []
        for group in self.param_groups:
            for p in group["params"]:
                if p.grad is None:
                    continue
                if not (p.is_cuda and p.dtype == torch.float32 and p.grad.dtype == torch.float32):
                    raise TypeError("FusedAdam handles float32 CUDA parameters")
                if not (p.is_contiguous() and p.grad.is_contiguous()):
                    raise ValueError("FusedAdam needs contiguous parameters and gradients")
                st = self.state[p]
                if len(st) == 0:
                    st["step"] = 0.0
                    st["exp_avg"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                    st["exp_avg_sq"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                out.append((p, group))
        return out

    def _ensure_table(self, active):
        key = tuple((p.data_ptr(), p.grad.data_ptr(), self.state[p]["exp_avg"].data_ptr(),
                     self.state[p]["exp_avg_sq"].data_ptr(), p.numel()) for p, _ in active)
        if key == self._key:
            return
        n = len(active)
        dev = active[0][0].device
        nbytes = int(L.query("ubs_adam_table_bytes", n))
        self._table_host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        for i, (p, _) in enumerate(active):
            st = self.state[p]
            L.call("ubs_adam_table_entry", ctypes.c_void_p(self._table_host.data_ptr()), i,
                   L.ptr(p), L.ptr(p.grad), L.ptr(st["exp_avg"]), L.ptr(st["exp_avg_sq"]),
                   p.numel(), i)
        self._table_dev = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self._table_dev.copy_(self._table_host, non_blocking=True)
        self._hyper_dev = torch.empty(2 * n, dtype=torch.float32, device=dev)
        self._hyper_host = [torch.empty(2 * n, dtype=torch.float32, pin_memory=True)
                            for _ in range(2)]
        self._hyper_np = [h.numpy() for h in self._hyper_host]
        self._hyper_events = [None, None]
        self._entries = active
        self._max_numel = max(p.numel() for p, _ in active)
        self._total_numel = sum(p.numel() for p, _ in active)
        self._key = key

    # ----------------------------------------------------------------- step
    @torch.no_grad()
    def prepare(self):
        """Host part of a step: advance the step counts and upload the step
        sizes and bias corrections (ordered before the next launch on the
        current stream)."""
        active = self._active()
        if not active:
            self._entries = []
            return
        self._ensure_table(active)
        slot = self._ring
        self._ring ^= 1
        ev = self._hyper_events[slot]
        if ev is not None:
            ev.synchronize()  # the copy that last read this pinned buffer is done
        hyper = self._hyper_np[slot]
        for i, (p, group) in enumerate(active):
            st = self.state[p]
            t = float(st["step"]) + 1.0
            st["step"] = t
            b1, b2 = group["betas"]
            # as torch.optim.Adam forms them (in double, then rounded to float)
            hyper[2 * i] = (group["lr"] / (1.0 - b1 ** t)) * -1
            hyper[2 * i + 1] = (1.0 - b2 ** t) ** 0.5
        self._hyper_dev.copy_(self._hyper_host[slot], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record()
        self._hyper_events[slot] = ev

    @torch.no_grad()
    def launch(self):
        """The update kernel on the current stream (capturable)."""
        if not self._entries:
            return
        group = self._entries[0][1]
        b1, b2 = group["betas"]
        if any(g["betas"] != group["betas"] or g["eps"] != group["eps"]
               for _, g in self._entries):
            raise ValueError("FusedAdam: all groups must share betas and eps")
        L.call("ubs_adam_step", len(self._entries), L.ptr(self._table_dev),
               L.ptr(self._hyper_dev), int(self._max_numel), int(self._total_numel),
               float(1 - b1), float(b2),
               float(1 - b2), float(group["eps"]), L.stream(self._table_dev.device))

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        self.prepare()
        self.launch()
        return loss
