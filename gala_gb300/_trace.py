"""NVTX ranges around the library's public GPU calls.

Each decorated call opens a range named ``gala_gb300.<name>``, so an Nsight
Systems or Nsight Compute timeline shows which API call issued which kernels.
Without a profiler attached the ranges cost a few microseconds per call.
"""
from __future__ import annotations

import functools


def traced(name: str):
    label = f"gala_gb300.{name}"

    def deco(fn):
        @functools.wraps(fn)
        def wrapper(*args, **kwargs):
            import torch

            with torch.cuda.nvtx.range(label):
                return fn(*args, **kwargs)

        return wrapper

    return deco
