"""Host-to-device input staging that overlaps with the integration kernels.

A caller whose inputs live in (pinned) host memory would otherwise copy a
whole batch to the GPU before the first kernel starts.  HostUpload issues the
copy on a side stream (optionally in batch chunks, one event per chunk).
transform_data_from_host (functions.py) queues the integration of the
trajectories first (it needs no image), then the copy of the images, and
samples once the copy has landed, so the copy runs under the integration.
Everything stays stream-ordered (no host synchronisation), so it can also be
captured in a CUDA graph.
"""
from __future__ import annotations

import threading

import torch

_streams = {}
_lock = threading.Lock()


def copy_stream(device) -> torch.cuda.Stream:
    """One side stream per device for host-to-device copies."""
    device = torch.device(device)
    idx = device.index if device.index is not None else torch.cuda.current_device()
    with _lock:
        st = _streams.get(idx)
        if st is None:
            st = torch.cuda.Stream(device=torch.device('cuda', idx))
            _streams[idx] = st
    return st


def chunk_bounds(n: int, chunks: int):
    """[(a, b), ...]: n rows in at most `chunks` nearly equal consecutive parts."""
    chunks = max(1, min(int(chunks), n)) if n > 0 else 1
    base, extra = divmod(n, chunks)
    out, a = [], 0
    for k in range(chunks):
        b = a + base + (1 if k < extra else 0)
        out.append((a, b))
        a = b
    return out


class HostUpload:
    """Copy a host tensor to `device` in `chunks` slices of its first axis on
    the copy stream.  `tensor` is the device tensor (usable once the matching
    event has been waited for); wait(k) makes the current stream wait for
    chunk k, wait() for all of them, and returns the tensor.  With
    start=False only the device tensor is allocated; start() (or the first
    wait()) enqueues the copies, so a caller can launch work that does not
    need the data first."""

    def __init__(self, host: torch.Tensor, device, chunks: int = 1, dtype=torch.float32,
                 start: bool = True):
        if host.is_cuda:
            raise ValueError('HostUpload takes a host tensor')
        device = torch.device(device)
        host = host.detach()
        if host.dtype != dtype:
            host = host.to(dtype)
        host = host.contiguous()
        if not host.is_pinned():
            # a pageable source would make the copy synchronous
            host = host.pin_memory()
        self.host = host
        cur = torch.cuda.current_stream(device)
        self._cs = copy_stream(device)
        n = host.shape[0] if host.dim() > 0 else 1
        self.bounds = chunk_bounds(n, chunks) if host.dim() > 0 else [(0, 1)]
        self.events = []
        self.started = False
        with torch.cuda.stream(self._cs):
            # allocated on the copy stream: the allocator hands it a block
            # whose earlier users are ordered before the copy, so the copy
            # need not wait for the current stream's queued kernels
            self.tensor = torch.empty(host.shape, dtype=dtype, device=device)
            if start:   # in the same stream context (one switch per upload)
                self._enqueue()
        # consumers run on the current stream: the block is reused only after
        # their queued work is done
        self.tensor.record_stream(cur)

    def _enqueue(self):
        # the copies and their events, on the copy stream (the current one)
        self.started = True
        host, cs = self.host, self._cs
        if len(self.bounds) == 1:
            self.tensor.copy_(host, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(cs)
            self.events.append(ev)
            return
        for a, b in self.bounds:
            self.tensor[a:b].copy_(host[a:b], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(cs)
            self.events.append(ev)

    def start(self):
        """Enqueue the copies (once)."""
        if self.started:
            return
        with torch.cuda.stream(self._cs):
            self._enqueue()

    def wait(self, k: int | None = None) -> torch.Tensor:
        self.start()
        cur = torch.cuda.current_stream(self.tensor.device)
        for ev in (self.events if k is None else [self.events[k]]):
            cur.wait_event(ev)
        return self.tensor
