"""The host cancel flag (gala_gb300.cancel, gx_set_cancel_flag): a flag in
mapped host memory that the persistent kernels poll before taking work.

No test here waits on the device for anything the host does not also end: a
flag set before the launch means the kernels take no work and return; a flag
set during a launch only shortens it, and the launch ends either way."""
import time

import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import _abi
from gala_gb300 import workloads as W
from gala_gb300.batch import BatchIntegrator
from gala_gb300.cancel import CancelFlag

pytestmark = pytest.mark.gpu


def _batch(n, steps, precision):
    mw = W.mw_composite()
    w0 = W.mw_ics(n, seed=71)
    return BatchIntegrator(mw, w0, np.full(n, steps), np.full(n, 0.5), np.arange(n) % 2, precision=precision)


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
def test_flag_set_before_the_launch_takes_no_chunk(precision):
    import torch

    b = _batch(4096, 50, precision)
    flag = CancelFlag()
    flag.set()
    with flag.installed():
        b.run()
    torch.cuda.synchronize()
    assert b.chunks_taken() == 0
    assert not bool(b.completed().any())
    flag.clear()
    with flag.installed():  # a cleared flag changes nothing
        b.run()
    torch.cuda.synchronize()
    assert bool(b.completed().all())
    flag.close()


def test_cancel_during_a_batch_run_stops_taking_chunks():
    """Twice as many 32-orbit chunks as the grid has warps, every orbit the
    same length: setting the flag while the first chunks run leaves the second
    half untaken; the orbits that were integrated equal an uncancelled run."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cfg = dict(block=128, ctas_per_sm=2, chunk=32)
    warps = sms * cfg["ctas_per_sm"] * cfg["block"] // 32
    n = 2 * warps * cfg["chunk"]
    mw = W.mw_composite()
    w0 = W.mw_ics(n, seed=72)
    args = (mw, w0, np.full(n, 400_000), np.full(n, 0.5), np.zeros(n, dtype=np.int32))
    full = BatchIntegrator(*args, config=cfg)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    ref = full.run().clone()
    e1.record()
    torch.cuda.synchronize()
    t_full = e0.elapsed_time(e1)
    assert bool(full.completed().all())

    part = BatchIntegrator(*args, config=cfg)
    flag = CancelFlag()
    with flag.installed():
        e0.record()
        part.run()
        e1.record()
    time.sleep(min(0.25, t_full / 1e3 / 4))  # inside the first half of the run
    flag.set()
    torch.cuda.synchronize()
    t_part = e0.elapsed_time(e1)
    done = part.completed()
    taken = part.chunks_taken()
    n_chunks = n // cfg["chunk"]
    assert 0 < taken < n_chunks, (taken, n_chunks)
    assert t_part < 0.8 * t_full, (t_part, t_full)
    assert int(done.sum()) == taken * cfg["chunk"]
    torch.testing.assert_close(part.w_out[:, done], ref[:, done], rtol=0, atol=0)
    flag.close()


def test_flag_set_before_dop853_launches():
    """gx_dop853_fp32 and gx_dop853_integrate_hamiltonian take no orbit or
    batch: the status arrays keep their initial zeros."""
    import torch

    from gala_gb300._device import ptr, stream_handle

    mw = W.mw_composite()
    n = 300
    w0 = torch.from_numpy(W.mw_ics(n, seed=73)).cuda()
    t = torch.from_numpy(g.parse_time_specification(dt=0.5, n_steps=100)).cuda()
    out = torch.empty((6, n), dtype=torch.float64, device="cuda")
    st32 = torch.zeros(n, dtype=torch.int32, device="cuda")
    st64 = torch.zeros(3, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    frame = g.StaticFrame().c_frame()
    import ctypes as C

    flag = CancelFlag()
    flag.set()
    with flag.installed():
        _abi.call("gx_dop853_fp32", mw.packed().for_device(), None, ptr(w0), n, ptr(t), t.numel(), 1e-10, 1e-8,
                  0, 0.0, 0, 0, 1, None, ptr(out), ptr(st32), None, ptr(cnt), stream_handle())
        _abi.call("gx_dop853_integrate_hamiltonian", mw.packed().for_device(), C.byref(frame), ptr(w0), n, ptr(t),
                  t.numel(), 1e-10, 1e-10, 0, 0.0, 0, 0, 100, 1, ptr(out), ptr(st64), None, stream_handle())
    torch.cuda.synchronize()
    assert int(cnt.item()) == 0
    assert not bool(st32.any()) and not bool(st64.any())
    flag.clear()
    with flag.installed():
        _abi.call("gx_dop853_integrate_hamiltonian", mw.packed().for_device(), C.byref(frame), ptr(w0), n, ptr(t),
                  t.numel(), 1e-10, 1e-10, 0, 0.0, 0, 0, 100, 1, ptr(out), ptr(st64), None, stream_handle())
    torch.cuda.synchronize()
    assert bool((st64 == 1).all())
    flag.close()


def test_flag_set_before_an_animate_run_keeps_the_initial_state():
    """gx_mockstream_dop853_animate stops before its first interval: every
    interval's status is 0, the first snapshot is the initial state, the others
    are NaN, and the final state is the initial one."""
    from ._cases import stream_case
    from .test_gpu_mockstream import _animate_gpu

    c = stream_case(n_streams=2, n_steps=30)
    flag = CancelFlag()
    flag.set()
    with flag.installed():
        snap, w, status, stats = _animate_gpu(c, 5)
    assert np.all(status[:, 0] == 1) and np.all(status[:, 1:] == 0)
    assert np.isnan(snap[:, 1:]).all()
    live = 1 + 2 * int(c["counts"][0])
    assert np.isfinite(snap[:, 0, :live]).all() and np.isnan(snap[:, 0, live:]).all()
    np.testing.assert_array_equal(w[:, 1:], c["stream_w0"])
    np.testing.assert_array_equal(w[:, 0], c["w0"].T)
    assert not stats.any()
    flag.close()
