"""NVTX ranges around the solver's phases (sector build, Lanczos, refinement,
reduced quantities, Green's functions, batched sweeps).  They name the
phases in an Nsight Systems timeline or an ``ncu --nvtx`` capture; without a
profiler attached a range costs two driver calls."""
from __future__ import annotations

import contextlib


@contextlib.contextmanager
def nvtx(name: str):
    import torch
    if not torch.cuda.is_available():
        yield
        return
    torch.cuda.nvtx.range_push(name)
    try:
        yield
    finally:
        torch.cuda.nvtx.range_pop()
