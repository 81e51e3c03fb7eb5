"""FP32 forms through the drop-in call: Hamiltonian.integrate_orbit with
Integrator_kwargs precision="fp32c".

* Leapfrog / Ruth4: FP32 forces with Kahan-compensated FP32 state against the
  FP64 oracle on the same time grid (strided snapshots).
* DOP853: FP32 stages and forces with FP64 time, error norm and accept/reject,
  per-orbit step control, against the FP64 oracle's DOP853.
Accuracy contract of the FP32 forms: final position within 1e-4 relative of the
FP64 oracle, median relative energy drift <= 1e-6.
"""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import workloads as W

from .conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["leapfrog", "ruth4"])
def test_fp32c_fixed_step_snapshots_match_oracle(oracle, method):
    mw = W.mw_composite()
    w0 = W.mw_ics(512, seed=31)
    t = g.parse_time_specification(dt=0.5, n_steps=2000)
    o = mw.integrate_orbit(w0, t=t, Integrator=method, Integrator_kwargs=dict(precision="fp32c", out_stride=10))
    w = o.w()
    assert w.shape == (6, 201, 512)
    assert np.array_equal(o.t, t[::10])
    ref = oracle.fixed(mw, w0, t, method)[:, ::10]
    assert np.array_equal(w[:, 0], w0)
    assert np.max(rel_err(w[:3], ref[:3])) <= 1e-4
    H = g.Hamiltonian(mw)
    dE = np.abs((H.energy(w[:, -1]) - H.energy(w0)) / H.energy(w0))
    dE_ref = np.abs((H.energy(ref[:, -1]) - H.energy(w0)) / H.energy(w0))
    # the FP32 form conserves energy like the FP64 integrator it restates
    assert np.median(np.abs(dE - dE_ref)) <= 1e-6


def test_fp32c_fixed_step_final_state_and_stride_one(oracle):
    pot = W.hernquist_potential()
    w0 = W.hernquist_ics(300, seed=32)
    t = g.parse_time_specification(dt=1.0, n_steps=500)
    last = pot.integrate_orbit(w0, t=t, Integrator="leapfrog", Integrator_kwargs=dict(precision="fp32c"),
                               save_all=False).w()
    full = pot.integrate_orbit(w0, t=t, Integrator="leapfrog", Integrator_kwargs=dict(precision="fp32c")).w()
    assert full.shape == (6, 501, 300)
    np.testing.assert_array_equal(last[:, 0], full[:, -1])
    ref = oracle.fixed(pot, w0, t, "leapfrog", save_all=False)
    assert np.max(rel_err(last[:3, 0], ref[:3])) <= 1e-5


def test_fp32_dop853_matches_fp64_oracle(oracle):
    """At atol 1e-10, rtol 1e-8 (FP32 stages resolve about 1e-8 relative per
    step; tighter tolerances only shrink the steps): median final position
    within 1e-4 of the FP64 oracle's DOP853 at gala's 1e-10, every orbit within
    1e-2, median energy drift <= 1e-6."""
    mw = W.mw_composite()
    n = 300
    w0 = W.mw_ics(n, seed=33)
    t = g.parse_time_specification(dt=0.5, n_steps=3000)
    o = mw.integrate_orbit(w0, t=t, Integrator="dop853",
                           Integrator_kwargs=dict(atol=1e-10, rtol=1e-8, precision="fp32c", out_stride=30))
    w = o.w()
    assert w.shape == (6, 101, n)
    assert np.array_equal(w[:, 0], w0)
    ref, st, _ = oracle.dop853(mw, w0, t, atol=1e-12, rtol=1e-10, out_stride=30)
    assert np.all(st == 1)
    err = rel_err(w[:3, -1], ref[:3, -1])
    assert np.median(err) <= 1e-4, np.median(err)
    assert np.max(rel_err(w[:3], ref[:3])) <= 1e-2
    H = g.Hamiltonian(mw)
    E0 = H.energy(w0)
    dE = np.abs((H.energy(w[:, -1]) - E0) / E0)
    assert np.median(dE) <= 1e-6, np.median(dE)


def test_fp32_dop853_step_control_follows_tolerance():
    """Looser tolerance -> fewer steps and every orbit finishes (status 1)."""
    import torch

    from gala_gb300 import _abi
    from gala_gb300._device import ptr

    mw = W.mw_composite()
    n = 256
    w0 = torch.from_numpy(W.mw_ics(n, seed=37)).cuda()
    t = torch.from_numpy(g.parse_time_specification(dt=0.5, n_steps=2000)).cuda()
    out = torch.empty((6, n), dtype=torch.float64, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    stats = torch.zeros((n, 4), dtype=torch.int64, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    steps = []
    for rtol in (1e-7, 1e-8):
        _abi.call("gx_dop853_fp32", mw.packed().for_device(), None, ptr(w0), n, ptr(t), t.numel(), rtol * 1e-2, rtol,
                  0, 0.0, 0, 0, 1, None, ptr(out), ptr(st), ptr(stats), ptr(cnt),
                  torch.cuda.current_stream().cuda_stream)
        assert torch.all(st == 1)
        s = stats.cpu().numpy()
        # gala's counter identities: nfcn = 2 + 11 nstep + naccpt (no dense output), nstep = naccpt + rejected
        assert np.all(s[:, 0] == 2 + 11 * s[:, 1] + s[:, 2])
        assert np.all(s[:, 1] >= s[:, 2] + s[:, 3])
        steps.append(s[:, 1].mean())
    assert steps[0] < 0.5 * steps[1]


def test_fp32_dop853_rotating_frame(oracle):
    pot = W.mw_composite()
    frame = g.ConstantRotatingFrame(Omega=[0.0, 0.0, 0.03])
    H = g.Hamiltonian(pot, frame=frame)
    w0 = W.mw_ics(128, seed=34)
    t = g.parse_time_specification(dt=0.5, n_steps=1000)
    w = H.integrate_orbit(w0, t=t, Integrator="dop853",
                          Integrator_kwargs=dict(precision="fp32c", out_stride=50, atol=1e-10, rtol=1e-8)).w()
    ref, st, _ = oracle.dop853(pot, w0, t, atol=1e-12, rtol=1e-10, out_stride=50, frame=frame)
    assert np.all(st == 1)
    err = rel_err(w[:3], ref[:3])
    assert np.median(err) <= 1e-5 and np.max(err) <= 1e-3, (np.median(err), np.max(err))


def test_fp32_dop853_failure_codes():
    mw = W.mw_composite()
    w0 = W.mw_ics(40, seed=35)
    t = g.parse_time_specification(dt=0.5, n_steps=2000)
    with pytest.raises(RuntimeError, match="code -2"):
        mw.integrate_orbit(w0, t=t, Integrator="dop853",
                           Integrator_kwargs=dict(precision="fp32c", nmax=50, atol=1e-10, rtol=1e-8))
    # err_if_fail=0 returns what was integrated
    o = mw.integrate_orbit(w0, t=t, Integrator="dop853",
                           Integrator_kwargs=dict(precision="fp32c", nmax=50, err_if_fail=0, atol=1e-10, rtol=1e-8),
                           save_all=False)
    assert o.w().shape == (6, 1, 40)


def test_fp32_forms_refuse_scf():
    S = np.zeros((1, 1, 1))
    S[0, 0, 0] = 1.0
    scf = g.SCFPotential(m=1e11, r_s=1.0, Snlm=S, Tnlm=S * 0)
    w0 = W.mw_ics(8, seed=36)
    for integ in ("leapfrog", "dop853"):
        with pytest.raises(TypeError):
            scf.integrate_orbit(w0, dt=1.0, n_steps=10, Integrator=integ, Integrator_kwargs=dict(precision="fp32c"))


def test_fp32_dop853_result_independent_of_processing_order():
    """Each orbit is its own system: the queue order (here the cost order used
    by integrate_orbit, and its reverse) changes no bits of any orbit."""
    import torch

    from gala_gb300 import _abi
    from gala_gb300._device import ptr
    from gala_gb300.hamiltonian import cost_order

    mw = W.mw_composite()
    n = 500
    w0 = torch.from_numpy(W.mw_ics(n, seed=38)).cuda()
    t = torch.from_numpy(g.parse_time_specification(dt=0.5, n_steps=800)).cuda()
    sh = torch.cuda.current_stream().cuda_stream
    order = cost_order(mw, w0, sh)
    assert sorted(order.cpu().tolist()) == list(range(n))
    outs = []
    for o in (None, order, torch.flip(order, [0]).contiguous()):
        out = torch.empty((6, 9, n), dtype=torch.float64, device="cuda")
        st = torch.zeros(n, dtype=torch.int32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        _abi.call("gx_dop853_fp32", mw.packed().for_device(), None, ptr(w0), n, ptr(t), t.numel(), 1e-10, 1e-8, 0,
                  0.0, 0, 1, 100, None if o is None else ptr(o), ptr(out), ptr(st), None, ptr(cnt), sh)
        assert torch.all(st == 1)
        outs.append(out.cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("name", ["kepler", "hernquist", "plummer", "miyamotonagai", "sphericalnfw",
                                  "flattenednfw", "triaxialnfw", "shifted_rotated"])
def test_fp32c_every_component_type(oracle, name):
    """The FP32 force of every closed-form component type (the run-time
    component loop, with the shift / rotation path): Ruth4 with FP32 forces
    and compensated state against the FP64 oracle on near-circular orbits."""
    from ._cases import potentials
    from .test_gpu_parity import _near_circular_ics

    pot = potentials()[name]
    w0 = _near_circular_ics(oracle, pot, 64, seed=67)
    t = g.parse_time_specification(dt=0.5, n_steps=500)
    w = pot.integrate_orbit(w0, t=t, Integrator="ruth4",
                            Integrator_kwargs=dict(precision="fp32c", out_stride=50)).w()
    ref = oracle.fixed(pot, w0, t, "ruth4")[:, ::50]
    err = rel_err(w[:3], ref[:3])
    assert np.median(err) <= 1e-5 and np.max(err) <= 1e-4, (name, np.median(err), np.max(err))
