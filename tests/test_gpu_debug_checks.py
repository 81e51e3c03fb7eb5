"""The debug build (libgala_gb300_debug.so, -DGX_DEBUG_CHECKS): caller-supplied
indices that fail the kernels' own range checks are skipped in both builds and
recorded in the debug build, and the persistent queues account for every
orbit they complete (gx_debug_read).  Every bad index used here is one the
kernels test before any access, so nothing is read or written out of bounds."""
import numpy as np
import pytest

from gala_gb300 import _abi
from gala_gb300 import workloads as W
from gala_gb300.batch import BatchIntegrator

pytestmark = pytest.mark.gpu

CODE_ORDER, CODE_SYSTEM, CODE_OFFSET, CODE_COUNT = 1, 2, 3, 4


def _read(lib, reset=True):
    import ctypes as C

    out = (C.c_int64 * 9)()
    assert lib.gx_debug_read(C.cast(out, C.c_void_p), int(reset)) == 0
    return dict(zip(["code", "line", "index", "bound", "fails", "done", "id_sum", "id_sq", "steps"], list(out)))


@pytest.fixture
def debug_lib(monkeypatch):
    """The debug library as the process's library for one test."""
    dbg = _abi.load_debug()
    assert dbg.gx_debug_enabled() == 1 and _abi.load().gx_debug_enabled() == 0
    _read(dbg)  # clear
    monkeypatch.setattr(_abi, "_lib", dbg)
    return dbg


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
def test_batch_queue_records_a_bad_order_id_and_accounts_for_every_orbit(debug_lib, monkeypatch, precision):
    import torch

    n = 1000  # not a multiple of the chunk: the order ends in -1 padding
    mw = W.mw_composite()
    rng = np.random.default_rng(5)
    w0 = W.mw_ics(n, seed=75)
    steps = rng.integers(10, 200, n)
    dt = np.full(n, 0.5)
    method = (np.arange(n) % 2).astype(np.int32)
    cfg = dict(block=128, ctas_per_sm=2, chunk=32)
    b = BatchIntegrator(mw, w0, steps, dt, method, config=cfg, precision=precision)
    b._prepare()
    pad = torch.nonzero(b.order == -1).flatten()
    assert pad.numel() > 0
    b.order[pad[0]] = n + 5
    got = b.run().clone()
    torch.cuda.synchronize()
    rec = _read(debug_lib)
    assert rec["code"] == CODE_ORDER and rec["index"] == n + 5 and rec["bound"] == n and rec["fails"] == 1
    k = np.arange(1, n + 1, dtype=np.int64)
    assert rec["done"] == n and rec["id_sum"] == k.sum() and rec["id_sq"] == (k * k).sum()
    assert rec["steps"] == int(steps.sum())
    # the release library skips the same entry silently and integrates the same orbits
    monkeypatch.setattr(_abi, "_lib", None)
    ref = BatchIntegrator(mw, w0, steps, dt, method, config=cfg, precision=precision).run()
    torch.testing.assert_close(got, ref, rtol=0, atol=0)


def test_dop853_fp32_order_entry_out_of_range_is_skipped(debug_lib):
    import torch

    from gala_gb300._device import ptr, stream_handle
    import gala_gb300 as g

    mw = W.mw_composite()
    n = 256
    w0 = torch.from_numpy(W.mw_ics(n, seed=76)).cuda()
    t = torch.from_numpy(g.parse_time_specification(dt=0.5, n_steps=50)).cuda()
    order = torch.arange(n, dtype=torch.int32, device="cuda")
    order[17] = n + 7  # orbit 17 is then never taken
    out = torch.zeros((6, n), dtype=torch.float64, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    _abi.call("gx_dop853_fp32", mw.packed().for_device(), None, ptr(w0), n, ptr(t), t.numel(), 1e-10, 1e-8, 0, 0.0,
              0, 0, 1, ptr(order), ptr(out), ptr(st), None, ptr(cnt), stream_handle())
    rec = _read(debug_lib)
    status = st.cpu().numpy()
    assert status[17] == 0 and np.all(np.delete(status, 17) == 1)
    assert rec["code"] == CODE_ORDER and rec["index"] == n + 7 and rec["fails"] == 1
    k = np.delete(np.arange(1, n + 1, dtype=np.int64), 17)
    assert rec["done"] == n - 1 and rec["id_sum"] == k.sum() and rec["id_sq"] == (k * k).sum()


def test_animate_release_count_overrun_is_recorded(debug_lib):
    """Release counts that sum past the particle array: the interval whose count
    overruns reports -1, the count is clamped, and the debug record names it."""
    from ._cases import stream_case
    from .test_gpu_mockstream import _animate_gpu

    c = stream_case(n_streams=1, n_steps=20)  # 2 particles released at each of the 21 times
    c["counts"] = c["counts"].copy()
    c["counts"][20] += 3  # the last release claims 6 particles more than the stream holds
    snap, w, status, _ = _animate_gpu(c, 5)
    rec = _read(debug_lib)
    assert status[0, 20] == -1 and np.all(status[0, :20] == 1)
    assert rec["code"] == CODE_COUNT and rec["index"] == 20 and rec["bound"] == 21 and rec["fails"] == 1
    assert np.isfinite(w).all()
