"""The oracle (C restatement of gala's hot path) pinned against gala itself.

Golden fixtures were produced by gala's own C/C++ (release flags, -Ofast); where
gala's sources are available the restatement is also compared bit-for-bit with
gala's code built without fast-math (same expression order, no contraction).
"""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import workloads as W

from .conftest import rel_err

# gala's -Ofast build reassociates some sums; the restatement (strict IEEE)
# agrees with it to this relative level on the fixtures' horizons.
OFAST_RTOL = 1e-11


def _pots():
    from ._cases import potentials

    return potentials()


def test_potentials_match_gala_golden(oracle, golden):
    d = golden("potentials.npz")
    q = d["q"]
    for name, pot in _pots().items():
        np.testing.assert_allclose(oracle.gradient(pot, q), d[f"{name}/gradient"], rtol=1e-13, atol=0)
        np.testing.assert_allclose(oracle.energy(pot, q), d[f"{name}/value"], rtol=1e-13, atol=0)
        if f"{name}/density" in d:
            np.testing.assert_allclose(oracle.density(pot, q), d[f"{name}/density"], rtol=1e-13, atol=0)
        np.testing.assert_allclose(oracle.hamiltonian_gradient(pot, d[f"{name}/w"]),
                                   d[f"{name}/hamiltonian_gradient"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("tag", ["fwd", "bwd"])
@pytest.mark.parametrize("method", ["leapfrog", "ruth4"])
def test_hernquist_fixed_step_golden(oracle, golden, method, tag):
    d = golden("hernquist_fixed.npz")
    w = oracle.fixed(g.HernquistPotential(m=1e11, c=0.5), d["w0"], d[f"t_{tag}"], method)
    assert np.max(rel_err(w[:, ::50, :], d[f"{method}_{tag}"])) <= OFAST_RTOL
    assert np.max(rel_err(w[:, -1, :], d[f"{method}_{tag}_final"])) <= OFAST_RTOL


@pytest.mark.parametrize("method", ["leapfrog", "ruth4"])
def test_mw_fixed_step_golden(oracle, golden, method):
    d = golden("mw_fixed.npz")
    w = oracle.fixed(W.mw_composite(), d["w0"], d["t"], method)
    assert np.max(rel_err(w[:, ::50, :], d[method])) <= OFAST_RTOL


def test_mw_dop853_golden(oracle, golden):
    d = golden("mw_dop853.npz")
    w, st, stats = oracle.dop853(W.mw_composite(), d["w0"], d["t"], atol=float(d["atol"]), rtol=float(d["rtol"]),
                                 nbatch=int(d["nbatch"]))
    assert np.all(st == d["status"])
    assert np.max(rel_err(w[:, ::50, :], d["w"])) <= OFAST_RTOL
    assert np.max(rel_err(w[:, -1, :], d["final"])) <= OFAST_RTOL


def test_rotating_frame_dop853_golden(oracle, golden):
    d = golden("mw_rotating_dop853.npz")
    frame = g.ConstantRotatingFrame(Omega=d["omega"])
    w, st, _ = oracle.dop853(W.mw_composite(), d["w0"], d["t"], atol=1e-12, rtol=1e-10, nbatch=8, frame=frame)
    assert np.all(st == d["status"])
    assert np.max(rel_err(w[:, ::50, :], d["w"])) <= OFAST_RTOL


def test_scf_matches_fortran(oracle, golden):
    """SCF restatement vs the original Fortran SCF code (rtol 1e-6, as gala's test)."""
    d = golden("scf_fortran.npz")
    for name in ["simple-hernquist", "multi-hernquist", "simple-nonsph", "random", "wang-zhao"]:
        pot = g.SCFPotential(m=1.0, r_s=1.0, Snlm=d[f"{name}/S"], Tnlm=d[f"{name}/T"])
        pot.G = 1.0
        np.testing.assert_allclose(oracle.gradient(pot, d["xyz"]), d[f"{name}/grad"], rtol=1e-6)
        np.testing.assert_allclose(oracle.energy(pot, d["xyz"]), d[f"{name}/pot"], rtol=1e-6)


def test_scf_s000_is_hernquist(oracle):
    """A pure S000 = 1 expansion is the Hernquist sphere (gala test_bfe.py:34-62)."""
    S = np.zeros((1, 1, 1))
    S[0, 0, 0] = 1.0
    scf = g.SCFPotential(m=1e11, r_s=2.0, Snlm=S, Tnlm=np.zeros_like(S))
    her = g.HernquistPotential(m=1e11, c=2.0)
    q = np.random.default_rng(0).normal(0, 5, size=(3, 50))
    np.testing.assert_allclose(oracle.energy(scf, q), oracle.energy(her, q), rtol=1e-12)
    np.testing.assert_allclose(oracle.gradient(scf, q), oracle.gradient(her, q), rtol=1e-10, atol=1e-22)
    np.testing.assert_allclose(oracle.density(scf, q), oracle.density(her, q), rtol=1e-10)


# ------------------------------------------------------- bit parity with gala
def test_bit_exact_vs_gala_strict(oracle, gala_ref_strict):
    """Same expression order, no contraction: identical bits to gala's code."""
    mw = W.mw_composite()
    w0 = W.mw_ics(30, seed=5)
    t = g.parse_time_specification(dt=0.5, n_steps=600)
    a, sa, _ = oracle.dop853(mw, w0, t, atol=1e-12, rtol=1e-10, nbatch=7)
    b, sb, _ = gala_ref_strict.dop853(mw, w0, t, atol=1e-12, rtol=1e-10, nbatch=7)
    assert np.array_equal(sa, sb)
    assert np.array_equal(a, b)
    for method in ("leapfrog", "ruth4"):
        a = oracle.fixed(mw, w0, t, method)
        b = gala_ref_strict.fixed(mw, w0, t, method)
        assert np.array_equal(a, b)
    for pot in _pots().values():
        q = np.random.default_rng(1).normal(0, 6, size=(3, 40))
        assert np.array_equal(oracle.gradient(pot, q), gala_ref_strict.gradient(pot, q))


def test_dop853_failure_codes(oracle):
    """nmax exceeded -> -2 (dop853.cpp:340-347), per batch."""
    mw = W.mw_composite()
    w0 = W.mw_ics(12, seed=6)
    t = g.parse_time_specification(dt=0.5, n_steps=400)
    _, st, _ = oracle.dop853(mw, w0, t, nmax=5, nbatch=5)
    assert list(st) == [-2, -2, -2]


def test_dop853_out_stride_consistent(oracle):
    mw = W.mw_composite()
    w0 = W.mw_ics(9, seed=8)
    t = g.parse_time_specification(dt=0.5, n_steps=300)
    full, _, _ = oracle.dop853(mw, w0, t, nbatch=4)
    strided, _, _ = oracle.dop853(mw, w0, t, nbatch=4, out_stride=7)
    assert np.array_equal(full[:, ::7, :], strided)


def test_dop853_status_for_non_finite_initial_conditions():
    """A NaN or infinite initial condition: gala's dop853() built with IEEE arithmetic
    reports -2 (nmax exceeded) and its -Ofast release build -3 (step too small) -- the
    comparisons that decide it are undefined under fast-math.  The restatement gives
    the same code in either build; the other orbit's batch is unaffected."""
    from oracle import Oracle
    from oracle.oracle import ref_available

    if not ref_available():
        pytest.skip("gala's own objects are not built here")
    pot = g.HernquistPotential(m=1e11, c=1.0)
    t = g.parse_time_specification(dt=1.0, n_steps=50)
    for bad in (np.nan, np.inf):
        w0 = np.array([[8.0, 8.0], [0, 0], [0, 0], [0, 0], [0.2, 0.2], [0, 0]])
        w0[0, 1] = bad
        # IEEE builds: exactly -2.  -Ofast builds: the code depends on how the
        # compiler treats the undefined comparisons, so only agreement with
        # gala's own -Ofast build and failure are required.
        st_mine = Oracle("strict").dop853(pot, w0, t, nbatch=1)[1]
        st_gala = Oracle("ref_strict").dop853(pot, w0, t, nbatch=1)[1]
        assert st_mine.tolist() == st_gala.tolist() == [1, -2]
        st_mine = Oracle("fast").dop853(pot, w0, t, nbatch=1)[1]
        st_gala = Oracle("ref").dop853(pot, w0, t, nbatch=1)[1]
        assert st_mine.tolist() == st_gala.tolist() and st_mine[0] == 1 and st_mine[1] < 0


def test_batch_fixed_matches_per_orbit_calls(oracle):
    """The uneven-batch restatement (per-orbit n_steps, dt, integrator) gives the
    bits of one gala call per orbit, threaded or not."""
    pot = W.mw_composite()
    n = 40
    w0 = W.mw_ics(n, seed=21)
    rng = np.random.default_rng(22)
    nsteps = rng.integers(0, 300, n)
    dt = rng.choice(np.array([0.1, 0.5, 1.0]), n)
    method = rng.integers(0, 2, n).astype(np.int32)
    ref = np.empty_like(w0)
    for i in range(n):
        if nsteps[i] == 0:
            ref[:, i] = w0[:, i]
            continue
        t = g.parse_time_specification(dt=float(dt[i]), n_steps=int(nsteps[i]))
        ref[:, i] = oracle.fixed(pot, w0[:, i:i + 1], t, "ruth4" if method[i] else "leapfrog", save_all=False)[:, 0]
    for nth in (1, 4):
        assert np.array_equal(oracle.batch_fixed(pot, w0, nsteps, dt, method, nthreads=nth), ref)


def test_cpu_baseline_is_as_fast_as_gala(gala_ref):
    """The -Ofast restatement timed as the CPU baseline runs no slower than
    gala's own -Ofast objects on the same problems (one thread, best of 3), so
    the GPU/CPU ratios are not inflated by a slow baseline.  (Best of five; the
    25 % margin absorbs timing noise on a shared host -- measured here the
    restatement runs Leapfrog and Ruth4 at gala's speed and DOP853 ~20 % faster.)"""
    import time

    from oracle import Oracle

    fast = Oracle("fast")
    mw = W.mw_composite()

    def best(fn):
        out = []
        for _ in range(5):
            t0 = time.perf_counter()
            fn()
            out.append(time.perf_counter() - t0)
        return min(out)

    w0 = W.mw_ics(100, seed=5)
    t = g.parse_time_specification(dt=0.5, n_steps=1500)
    for kind in ("leapfrog", "ruth4"):
        ours = best(lambda: fast.fixed(mw, w0, t, kind, save_all=False))
        gala = best(lambda: gala_ref.fixed(mw, w0, t, kind, save_all=False))
        assert ours <= 1.25 * gala, (kind, ours, gala)
    ours = best(lambda: fast.dop853(mw, w0, t, atol=1e-12, rtol=1e-10))
    gala = best(lambda: gala_ref.dop853(mw, w0, t, atol=1e-12, rtol=1e-10))
    assert ours <= 1.25 * gala, ("dop853", ours, gala)
