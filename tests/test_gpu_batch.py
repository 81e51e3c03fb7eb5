"""Batched uneven workload (per-orbit n_steps, dt, integrator) on the GPU.

* FP64 batch kernel: gala's per-orbit arithmetic, checked orbit by orbit
  against the oracle (bit-exact for Hernquist, <= 1e-12 for the MW composite).
* FP32-compensated kernel: against the FP64 oracle, final position error
  <= 1e-4 relative and median energy drift <= 1e-6 (the accuracy contract of
  the FP32 form).
"""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import workloads as W
from gala_gb300.batch import SEARCH, BatchIntegrator

from .conftest import rel_err

pytestmark = pytest.mark.gpu


def _workload(n, seed, max_steps):
    rng = np.random.default_rng(seed)
    nsteps = np.round(np.exp(rng.uniform(np.log(50), np.log(max_steps), n))).astype(np.int64)
    dt = rng.choice(np.array([0.1, 0.5, 1.0]), n)
    method = rng.integers(0, 2, n).astype(np.int32)
    return nsteps, dt, method


def _oracle_final(oracle, pot, w0, nsteps, dt, method):
    out = np.empty_like(w0)
    for i in range(w0.shape[1]):
        t = g.parse_time_specification(dt=float(dt[i]), n_steps=int(nsteps[i]))
        out[:, i] = oracle.fixed(pot, w0[:, i:i + 1], t, "leapfrog" if method[i] == 0 else "ruth4",
                                 save_all=False)[:, 0]
    return out


@pytest.mark.parametrize("potname", ["hernquist", "mw"])
def test_fp64_batch_matches_oracle(oracle, potname):
    pot = W.hernquist_potential() if potname == "hernquist" else W.mw_composite()
    w0 = W.hernquist_ics(300, seed=3) if potname == "hernquist" else W.mw_ics(300, seed=3)
    nsteps, dt, method = _workload(300, 5, 600)
    b = BatchIntegrator(pot, w0, nsteps, dt, method, precision="fp64")
    w = b.run().cpu().numpy()
    ref = _oracle_final(oracle, pot, w0, nsteps, dt, method)
    if potname == "hernquist":
        assert np.array_equal(w, ref)
    else:
        assert np.max(rel_err(w, ref)) <= 1e-12


def test_fp32c_accuracy_contract(oracle):
    pot = W.mw_composite()
    n = 1024
    w0 = W.mw_ics(n, seed=7)
    nsteps, dt, method = _workload(n, 8, 4000)
    b = BatchIntegrator(pot, w0, nsteps, dt, method)
    w = b.run().cpu().numpy()
    ref = _oracle_final(oracle, pot, w0, nsteps, dt, method)
    pos_err = rel_err(w[:3], ref[:3])
    assert np.max(pos_err) <= 1e-4, np.max(pos_err)
    dE = b.energy_drift().cpu().numpy()
    assert np.median(dE) <= 1e-6, np.median(dE)
    # the FP64 diagnostic agrees with the oracle's energy of the final states
    E1 = oracle.hamiltonian_value(pot, w)
    np.testing.assert_allclose(b.E1.cpu().numpy(), E1, rtol=1e-13)


def test_graph_replay_matches_eager():
    pot = W.mw_composite()
    n = 2000
    w0 = W.mw_ics(n, seed=9)
    nsteps, dt, method = _workload(n, 10, 500)
    eager = BatchIntegrator(pot, w0, nsteps, dt, method).run().cpu().numpy()
    b = BatchIntegrator(pot, w0, nsteps, dt, method).capture()
    for _ in range(2):
        b.run()
    assert np.array_equal(b.w_out.cpu().numpy(), eager)


def test_autotune_returns_searched_config(tmp_path, monkeypatch):
    import gala_gb300.batch as B

    monkeypatch.setattr(B, "CACHE", tmp_path / "autotune.json")
    pot = W.mw_composite()
    w0 = W.mw_ics(4096, seed=11)
    nsteps, dt, method = _workload(4096, 12, 300)
    b = BatchIntegrator(pot, w0, nsteps, dt, method)
    best = b.autotune(work_fraction=0.05, reps=1)
    assert best in SEARCH["fp32c"]
    assert (tmp_path / "autotune.json").exists()
    # a new integrator of the same workload picks the cached choice
    assert BatchIntegrator(pot, w0, nsteps, dt, method).config == best


def test_zero_steps_and_single_method():
    pot = W.mw_composite()
    w0 = W.mw_ics(64, seed=13)
    nsteps = np.zeros(64, dtype=np.int64)
    nsteps[::2] = 100
    for prec in ("fp32c", "fp64"):
        b = BatchIntegrator(pot, w0, nsteps, np.full(64, 0.5), np.zeros(64, dtype=np.int32), precision=prec)
        w = b.run().cpu().numpy()
        assert np.array_equal(w[:, 1::2], w0[:, 1::2])
        assert not np.array_equal(w[:, ::2], w0[:, ::2])


def test_invalid_batch_arguments():
    pot = W.mw_composite()
    w0 = W.mw_ics(8, seed=14)
    with pytest.raises(ValueError):
        BatchIntegrator(pot, w0, np.ones(7, dtype=np.int64), np.ones(8), np.zeros(8, dtype=np.int32))
    with pytest.raises(ValueError):
        BatchIntegrator(pot, w0, np.ones(8, dtype=np.int64), np.ones(8), np.full(8, 3, dtype=np.int32))
    S = np.zeros((1, 1, 1))
    S[0, 0, 0] = 1.0
    scf = g.SCFPotential(m=1e11, r_s=1.0, Snlm=S, Tnlm=S * 0)
    with pytest.raises(TypeError):
        BatchIntegrator(scf, w0, np.ones(8, dtype=np.int64), np.ones(8), np.zeros(8, dtype=np.int32)).run()


@pytest.mark.parametrize("chunk", [32, 64])
def test_device_schedule_is_a_cost_ordered_chunking(chunk):
    """gx_batch_schedule: every orbit exactly once; every chunk holds one
    integrator; within each integrator the lists run from the most expensive
    orbit down (to the 0.54 % bins); chunk heads of the merged order do not
    increase in cost by more than a bin; the same chunk-head costs as the
    exact torch order to within a bin."""
    import torch

    from gala_gb300.batch import COST, schedule

    rng = np.random.default_rng(11)
    n = 10_001
    nsteps = torch.from_numpy(np.exp(rng.uniform(np.log(5), np.log(40_000), n)).astype(np.int64)).cuda()
    method = torch.from_numpy(rng.integers(0, 2, n).astype(np.int32)).cuda()
    b = BatchIntegrator(W.mw_composite(), W.mw_ics(n, seed=3), nsteps, torch.full((n,), 0.5, device="cuda"), method,
                        config=dict(block=128, ctas_per_sm=2, chunk=chunk))
    b._prepare(torch.cuda.current_stream().cuda_stream)
    order = b.order.cpu().numpy()
    assert order.size % chunk == 0
    real = order[order >= 0]
    assert np.array_equal(np.sort(real), np.arange(n))
    ns, me = nsteps.cpu().numpy(), method.cpu().numpy()
    cost = ns * np.where(me == 1, COST[1], COST[0])
    bin_ratio = 2.0 ** (1 / 128)
    heads = []
    for c in order.reshape(-1, chunk):
        ids = c[c >= 0]
        if ids.size == 0:
            continue
        assert np.unique(me[ids]).size == 1
        assert np.all(cost[ids][1:] <= cost[ids][:-1] * bin_ratio + 1)
        heads.append(cost[ids[0]])
    heads = np.array(heads, dtype=np.float64)
    assert np.all(heads[1:] <= heads[:-1] * bin_ratio + 1)
    ref = schedule(nsteps, method, chunk).cpu().numpy().reshape(-1, chunk)
    ref_heads = np.sort(np.array([cost[c[0]] for c in ref if c[0] >= 0], dtype=np.float64))[::-1]
    assert ref_heads.size == heads.size
    np.testing.assert_allclose(heads, ref_heads, rtol=bin_ratio - 1, atol=1)


def test_checkpoint_resume_is_bit_identical():
    """A run of k steps that keeps its state, then runs resumed from it (through
    host memory, as a checkpoint file would), give the bits of one run of n
    steps, orbit by orbit -- for Leapfrog (whose state is the half-step
    velocity) and Ruth4, with segments of zero steps among them."""
    import torch

    n = 3000
    pot = W.mw_composite()
    w0 = W.mw_ics(n, seed=91)
    nsteps, dt, method = _workload(n, 92, 600)
    k1 = nsteps // 3
    k2 = (nsteps - k1) // 2
    k1[:3], k2[:3] = 0, 0                  # first segments of zero steps
    k1[3:6], k2[3:6] = nsteps[3:6], 0      # everything in the first segment
    k3 = nsteps - k1 - k2
    full = BatchIntegrator(pot, w0, nsteps, dt, method).run().clone()
    a = BatchIntegrator(pot, w0, k1, dt, method, checkpoint=True)
    a.run()
    b = BatchIntegrator(pot, w0, k2, dt, method, state=a.state.cpu().numpy(), checkpoint=True)
    b.run()
    c = BatchIntegrator(pot, w0, k3, dt, method, state=b.state)
    out = c.run()
    torch.cuda.synchronize()
    assert torch.equal(out, full)
    # the energy diagnostic of the last segment refers to the original initial conditions
    ref = BatchIntegrator(pot, w0, nsteps, dt, method)
    ref.run()
    assert torch.equal(c.energy_drift(), ref.energy_drift())


def test_orbit_pairs_give_the_bits_of_single_orbits():
    """Main-region chunks of 64 orbits run two orbits per lane; lead blocks and
    32-orbit chunks run one.  Every orbit's bits are the same either way, also
    with zero-step orbits among them and through a checkpoint and resume."""
    import torch

    n = 40_000  # more than the lead region (4 x SMs blocks of 32), so both regions run
    pot = W.mw_composite()
    w0 = W.mw_ics(n, seed=95)
    nsteps, dt, method = _workload(n, 96, 300)
    nsteps[::97] = 0
    one = dict(block=128, ctas_per_sm=2, chunk=32)
    two = dict(block=128, ctas_per_sm=2, chunk=64)
    single = BatchIntegrator(pot, w0, nsteps, dt, method, config=one).run().clone()
    paired = BatchIntegrator(pot, w0, nsteps, dt, method, config=two)
    assert torch.equal(paired.run(), single)
    assert bool(paired.completed().all())
    k1 = nsteps // 2
    a = BatchIntegrator(pot, w0, k1, dt, method, config=two, checkpoint=True)
    a.run()
    b = BatchIntegrator(pot, w0, nsteps - k1, dt, method, config=two, state=a.state)
    out = b.run()
    torch.cuda.synchronize()
    # an orbit with no step in either segment returns its state's value (for
    # Leapfrog v_{1/2} + g h / 2, an FP32 compensated sum: to ~1e-7 of the
    # smallest velocity components); one run of no steps returns w0 itself
    stepped = torch.from_numpy(nsteps > 0).cuda()
    assert torch.equal(out[:, stepped], single[:, stepped])
    torch.testing.assert_close(out[:, ~stepped], single[:, ~stepped], rtol=1e-6, atol=1e-9)


def test_checkpoint_arguments():
    pot = W.mw_composite()
    w0 = W.mw_ics(64, seed=93)
    nsteps, dt, method = _workload(64, 94, 100)
    with pytest.raises(NotImplementedError):
        BatchIntegrator(pot, w0, nsteps, dt, method, precision="fp64", checkpoint=True)
    with pytest.raises(ValueError, match="shape"):
        BatchIntegrator(pot, w0, nsteps, dt, method, state=np.zeros((12, 63), dtype=np.float32))
