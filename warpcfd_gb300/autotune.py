"""Autotuner of the batched form: picks the block size of the batched field and assembly
kernels for a batch by timing one batched outer iteration per candidate on the batch's
own cases, then puts every case back as it was.

The field and assembly kernels compute each face or cell on its own, so the choice moves
time, never results; the Krylov cluster size (which fixes the order of the reductions) is
not tuned here.  Choices are cached per (cell-count bucket, case count, mesh kind) for the
life of the process, so a batch is timed once and later batches of the same shape reuse
the answer.
"""
from __future__ import annotations

import math

import torch

CANDIDATES = (128, 256, 512)
_cache: dict = {}


def _key(batch):
    d = batch.dims
    return (int(math.log2(max(d.max_cells, 1))), len(batch), d.faces_per_cell, d.ell_width, d.cluster_size)


def tune_field_block(batch, candidates=CANDIDATES, repeats: int = 2, key=None) -> int:
    """Best field block size for ``batch`` (a CaseBatch), timed on the current stream;
    the batch's cases are restored bit for bit afterwards and its dims keep the choice.
    ``key`` overrides the cache key (default: cell-count bucket, case count, cell type,
    width, cluster size)."""
    key = _key(batch) if key is None else key
    if key in _cache:
        batch.dims.field_block = _cache[key]
        return _cache[key]
    snaps = [s.snapshot() for s in batch.solvers]
    stats = batch.stats.clone()
    best, best_ms = candidates[0], float("inf")
    stream = torch.cuda.current_stream()
    for fb in candidates:
        batch.dims.field_block = fb
        batch.step()  # first use of this configuration, untimed
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(repeats):
            batch.step()
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1) / repeats
        if ms < best_ms:
            best, best_ms = fb, ms
    for s, snap in zip(batch.solvers, snaps):
        s.restore(snap)
    batch.stats.copy_(stats)
    batch.dims.field_block = best
    _cache[key] = best
    return best


def cached_choices() -> dict:
    return dict(_cache)
