"""Streaming host-resident ensembles through the GPU filter.

An ensemble that lives in host memory (the reference's callers hold VALL on
the host) is filtered batch after batch: every step copies its inputs from
pinned host memory to the device, runs forward and/or adjoint filtering, and
copies the result back.  Three streams (host to device, compute, device to
host) let step s+1's upload and step s-1's download run while step s is
filtered; uploads and downloads use separate streams because the host link
moves data in both directions at once (about 330 GB/s in total against about
200 GB/s one way).  Events order each device field set's reuse: the upload
of step s waits for the download of step s - nsets.  With two sets that
wait chains every other step's download and upload between two filterings
(on GB300 at the batched ensemble's 14.8 GB per direction, about 147 ms of
copies against about 100 ms of filtering); three sets (the default) leave
the filtering as the only serial chain whenever the link keeps up.
"""
from __future__ import annotations

from typing import List, Sequence

import torch

from .mgbf import MGBFBatch


class HostStream:
    """Pipelined host -> GPU -> host filtering of a batch's variable groups."""

    def __init__(self, batch: MGBFBatch, dtype=torch.float32, device=None, ops: Sequence[str] = ("fwd", "adj"),
                 nsets: int = 3):
        if nsets < 2:
            raise ValueError("HostStream needs at least two device field sets")
        self.batch = batch
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = dtype
        self.ops = tuple(ops)
        self.nsets = nsets
        self.sets = [[torch.empty(batch.field_shape(q), dtype=dtype, device=self.device)
                      for q in range(len(batch.groups))] for _ in range(nsets)]
        self.s_h2d = torch.cuda.Stream(self.device)
        self.s_cmp = torch.cuda.Stream(self.device)
        self.s_d2h = torch.cuda.Stream(self.device)
        self.ev_h2d = [torch.cuda.Event() for _ in range(nsets)]
        self.ev_cmp = [torch.cuda.Event() for _ in range(nsets)]
        self.ev_d2h = [torch.cuda.Event() for _ in range(nsets)]
        self.step = 0

    def bytes_per_step(self) -> int:
        return sum(f.numel() * f.element_size() for f in self.sets[0])

    def submit(self, host_in: List[torch.Tensor], host_out: List[torch.Tensor]) -> None:
        """Queue one step: host_in -> device, filter, device -> host_out.
        Host tensors should be pinned for asynchronous copies; read host_out
        only after finish()."""
        i = self.step % self.nsets
        dev = self.sets[i]
        with torch.cuda.stream(self.s_h2d):
            if self.step >= self.nsets:
                self.s_h2d.wait_event(self.ev_d2h[i])  # the set's previous download is done
            for d, h in zip(dev, host_in):
                d.copy_(h, non_blocking=True)
            self.ev_h2d[i].record(self.s_h2d)
        with torch.cuda.stream(self.s_cmp):
            self.s_cmp.wait_event(self.ev_h2d[i])
            for op in self.ops:
                self.batch.apply(dev, adjoint=(op == "adj"))
            self.ev_cmp[i].record(self.s_cmp)
        with torch.cuda.stream(self.s_d2h):
            self.s_d2h.wait_event(self.ev_cmp[i])
            for d, h in zip(dev, host_out):
                h.copy_(d, non_blocking=True)
            self.ev_d2h[i].record(self.s_d2h)
        self.step += 1

    def finish(self) -> None:
        """Wait for every queued step."""
        for s in (self.s_h2d, self.s_cmp, self.s_d2h):
            s.synchronize()
