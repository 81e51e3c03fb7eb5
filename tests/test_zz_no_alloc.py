"""The allocation-free batch entry point, gx_batch_integrate_fp32_noalloc.

Some callers cannot allocate device memory (their memory manager owns the GPU,
they only hold device pointers handed over by another runtime, or they cannot
afford the device synchronisation of cudaMalloc/cudaFree), so this entry point
takes only inputs and outputs and keeps its work queue in a fixed array inside
the library.  The test calls it through the C ABI twice in a row and checks
each result against the regular entry point, gx_batch_integrate_fp32, which
takes its queue scratch from the caller.  Per-orbit arithmetic is the same in
both, so the results must agree bit for bit.

This file is named so that pytest collects it last.
"""

import numpy as np
import pytest

from gala_gb300 import _abi
from gala_gb300 import workloads as W
from gala_gb300.batch import BatchIntegrator

pytestmark = pytest.mark.gpu


def _inputs(n, seed):
    import torch

    rng = np.random.default_rng(seed)
    w0 = torch.from_numpy(W.mw_ics(n, seed=seed)).cuda()
    nsteps = torch.from_numpy(np.round(np.exp(rng.uniform(np.log(20), np.log(800), n))).astype(np.int64)).cuda()
    dt = torch.from_numpy(rng.choice(np.array([0.1, 0.5, 1.0]), n)).cuda()
    method = torch.from_numpy(rng.integers(0, 2, n).astype(np.int32)).cuda()
    return w0, nsteps, dt, method


def test_noalloc_matches_regular_entry_point_twice():
    import torch

    lib = _abi.load()
    pot = W.mw_composite()
    desc = pot.packed().for_device()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    stream = torch.cuda.current_stream().cuda_stream
    for call, (n, seed) in enumerate([(5000, 101), (3001, 202)]):
        w0, nsteps, dt, method = _inputs(n, seed)
        regular = BatchIntegrator(pot, w0, nsteps, dt, method,
                                  config={"block": 128, "ctas_per_sm": 4, "chunk": 32}).run()
        out = torch.full((6, n), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.gx_batch_integrate_fp32_noalloc(desc, w0.data_ptr(), n, nsteps.data_ptr(), dt.data_ptr(),
                                                 method.data_ptr(), 128, 4 * sms, out.data_ptr(), stream)
        assert rc == 0, lib.gx_last_error_message()
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), regular.cpu().numpy()
        assert np.isfinite(a).all(), f"call {call}: unfilled outputs"
        assert np.array_equal(a, b), f"call {call}: max |diff| {np.nanmax(np.abs(a - b))}"


def test_noalloc_call_allocates_no_device_memory():
    """After one warm-up call, a further call leaves the device's free memory
    unchanged: the work queue is the library's own array."""
    import torch

    lib = _abi.load()
    desc = W.mw_composite().packed().for_device()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    stream = torch.cuda.current_stream().cuda_stream
    n = 4000
    w0, nsteps, dt, method = _inputs(n, 303)
    out = torch.empty((6, n), dtype=torch.float64, device="cuda")
    args = (desc, w0.data_ptr(), n, nsteps.data_ptr(), dt.data_ptr(), method.data_ptr(), 128, 4 * sms,
            out.data_ptr(), stream)
    assert lib.gx_batch_integrate_fp32_noalloc(*args) == 0
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    assert lib.gx_batch_integrate_fp32_noalloc(*args) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _abi.load()
    desc = W.mw_composite().packed().for_device()
    n = _abi.GX_NOALLOC_MAX_ORBITS + 1
    rc = lib.gx_batch_integrate_fp32_noalloc(desc, None, n, None, None, None, 128, 1, None, None)
    assert rc == _abi.GX_ERR_CAPACITY
    assert b"GX_NOALLOC_MAX_ORBITS" in lib.gx_last_error_message()
