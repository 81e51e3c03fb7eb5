"""GPU parity: the CUDA library (through its C ABI) against the oracle and the
golden fixtures produced by gala's own code.

Tolerances
  * closed-form potentials with only sqrt / division (Hernquist, Plummer): the
    FP64 kernels reproduce the oracle BIT FOR BIT (same expression order, no
    contraction, IEEE sqrt and division on both sides);
  * potentials using pow / log (Kepler, Miyamoto-Nagai, NFW): CUDA's pow/log and
    glibc's may differ by an ulp, so single evaluations agree to rtol 1e-14 and
    integrated orbits to 1e-12 relative in position and velocity;
  * SCF: same series summed in a different order, rtol 1e-10 per evaluation.
"""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import workloads as W

from .conftest import rel_err

pytestmark = pytest.mark.gpu

PARITY = 1e-12


def _pots():
    from ._cases import potentials

    return potentials()


def _orbit_w(orbit):
    return orbit.w()


# ------------------------------------------------------------------ potentials
@pytest.mark.parametrize("name", ["kepler", "hernquist", "plummer", "miyamotonagai", "sphericalnfw",
                                  "flattenednfw", "triaxialnfw", "mw", "shifted_rotated"])
def test_potential_eval_matches_oracle(oracle, golden, name):
    pot = _pots()[name]
    d = golden("potentials.npz")
    q = d["q"]
    exact = name in ("hernquist", "plummer")
    for kind in ("gradient", "value", "density"):
        if kind == "density" and name in ("flattenednfw", "triaxialnfw"):
            continue
        gpu = getattr(pot, {"value": "energy"}.get(kind, kind))(q)
        cpu = getattr(oracle, {"value": "energy"}.get(kind, kind))(pot, q)
        if exact and kind != "density":
            assert np.array_equal(gpu, cpu), kind
        else:
            np.testing.assert_allclose(gpu, cpu, rtol=1e-14 if kind != "density" else 1e-13, atol=0)
        np.testing.assert_allclose(gpu, d[f"{name}/{'value' if kind == 'value' else kind}"], rtol=1e-13, atol=0)
    H = g.Hamiltonian(pot)
    np.testing.assert_allclose(H.gradient(d[f"{name}/w"]), d[f"{name}/hamiltonian_gradient"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(H.energy(d[f"{name}/w"]), oracle.hamiltonian_value(pot, d[f"{name}/w"]),
                               rtol=1e-14, atol=0)


# ----------------------------------------------------------- fixed-step (FP64)
@pytest.mark.parametrize("tag", ["fwd", "bwd"])
@pytest.mark.parametrize("method", ["leapfrog", "ruth4"])
def test_hernquist_fixed_bit_exact(oracle, golden, method, tag):
    d = golden("hernquist_fixed.npz")
    pot = g.HernquistPotential(m=1e11, c=0.5)
    t = d[f"t_{tag}"]
    orbit = pot.integrate_orbit(d["w0"], t=t, Integrator=method)
    w = orbit.w()
    ref = oracle.fixed(pot, d["w0"], t, method)
    assert np.array_equal(w, ref)
    assert np.max(rel_err(w[:, ::50, :], d[f"{method}_{tag}"])) <= 1e-11  # gala -Ofast build


@pytest.mark.parametrize("method", ["leapfrog", "ruth4"])
def test_mw_fixed_parity(oracle, golden, method):
    d = golden("mw_fixed.npz")
    mw = W.mw_composite()
    w = mw.integrate_orbit(d["w0"], t=d["t"], Integrator=method).w()
    ref = oracle.fixed(mw, d["w0"], d["t"], method)
    assert np.max(rel_err(w[:3], ref[:3])) <= PARITY
    assert np.max(rel_err(w[3:], ref[3:])) <= PARITY
    assert np.max(rel_err(w[:, ::50, :], d[method])) <= 1e-11


def test_config1_leapfrog_parity(oracle):
    """Hernquist m=1e11 c=1, 1,024 orbits, dt=1 Myr, 1,000 steps, all snapshots."""
    pot = W.hernquist_potential()
    w0 = W.hernquist_ics(1024)
    orbit = pot.integrate_orbit(w0, dt=1.0, n_steps=1000, Integrator="leapfrog")
    ref = oracle.fixed(pot, w0, g.parse_time_specification(dt=1.0, n_steps=1000), "leapfrog", nthreads=8)
    assert orbit.w().shape == (6, 1001, 1024)
    assert np.array_equal(orbit.w(), ref)


# --------------------------------------------------------------------- DOP853
def test_mw_dop853_parity(oracle, golden):
    d = golden("mw_dop853.npz")
    mw = W.mw_composite()
    orbit = mw.integrate_orbit(d["w0"], t=d["t"], Integrator="dop853",
                               Integrator_kwargs=dict(atol=1e-12, rtol=1e-10, nbatch=10))
    w = orbit.w()
    ref, st, _ = oracle.dop853(mw, d["w0"], d["t"], atol=1e-12, rtol=1e-10, nbatch=10)
    assert np.max(rel_err(w[:3], ref[:3])) <= PARITY
    assert np.max(rel_err(w[3:], ref[3:])) <= PARITY
    assert np.max(rel_err(w[:, ::50, :], d["w"])) <= 1e-11


def _near_circular_ics(oracle, pot, n, seed):
    """Orbits of R in [4, 20] kpc, |z| < 0.3 kpc with the potential's own circular
    speed (from the oracle's gradient at (R, 0, 0)) times 1 + N(0, 0.05) plus a
    small vertical velocity: bound, non-chaotic over the test horizon."""
    rng = np.random.default_rng(seed)
    R = rng.uniform(4.0, 20.0, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    z = rng.uniform(-0.3, 0.3, n)
    gx = oracle.gradient(pot, np.stack([R, np.zeros(n), np.zeros(n)]))[0]
    vc = np.sqrt(np.abs(R * gx)) * (1 + rng.normal(0, 0.05, n))
    return np.stack([R * np.cos(phi), R * np.sin(phi), z, -vc * np.sin(phi), vc * np.cos(phi),
                     rng.normal(0, 0.005, n)])


@pytest.mark.parametrize("name", ["kepler", "hernquist", "plummer", "miyamotonagai", "sphericalnfw",
                                  "flattenednfw", "triaxialnfw", "shifted_rotated"])
def test_dop853_every_component_type_matches_oracle(oracle, name):
    """DOP853 evaluates every component type in its FP64-pipe-lean forms
    (seeded Newton square roots and reciprocals, the table-driven ln, constants
    derived on the host, the shift/rotate path with fused products).  The orbits
    must stay within 1e-12 of the oracle (gala's expressions, strict build), or
    within 10x the oracle's own spread between its strict and -Ofast builds
    where that ulp-level perturbation alone grows past 1e-12 over the horizon:
    the tilted, shifted composite does so late in this run (strict vs -Ofast
    2.4e-11 at 200 Myr, 6e-15 at 100 Myr); every other type is held to 1e-12."""
    from oracle import Oracle

    pot = _pots()[name]
    w0 = _near_circular_ics(oracle, pot, 24, seed=61)
    t = g.parse_time_specification(dt=0.5, n_steps=400)
    orbit = pot.integrate_orbit(w0, t=t, Integrator="dop853",
                                Integrator_kwargs=dict(atol=1e-12, rtol=1e-10, nbatch=8))
    ref, status, _ = oracle.dop853(pot, w0, t, atol=1e-12, rtol=1e-10, nbatch=8)
    assert np.all(status == 1)
    ofast, _, _ = Oracle("fast").dop853(pot, w0, t, atol=1e-12, rtol=1e-10, nbatch=8)
    spread = max(np.max(rel_err(ofast[:3], ref[:3])), np.max(rel_err(ofast[3:], ref[3:])))
    tol = max(PARITY, 10 * spread)
    w = orbit.w()
    ep, ev = np.max(rel_err(w[:3], ref[:3])), np.max(rel_err(w[3:], ref[3:]))
    if name != "shifted_rotated":
        tol = PARITY
    assert ep <= tol and ev <= tol, (name, ep, ev, spread)


def test_dop853_energy_curve_matches_oracle(oracle):
    """Energy-conservation curves E(t) of the GPU and the oracle agree."""
    mw = W.mw_composite()
    w0 = W.mw_ics(40, seed=21)
    t = g.parse_time_specification(dt=0.5, n_steps=1500)
    orbit = mw.integrate_orbit(w0, t=t, Integrator="dop853", Integrator_kwargs=dict(atol=1e-12, rtol=1e-10))
    E_gpu = orbit.energy()
    ref, _, _ = oracle.dop853(mw, w0, t, atol=1e-12, rtol=1e-10)
    E_ref = oracle.hamiltonian_value(mw, ref.reshape(6, -1)).reshape(ref.shape[1:])
    np.testing.assert_allclose(E_gpu, E_ref, rtol=1e-12)
    dE = np.abs((E_gpu - E_gpu[0]) / E_gpu[0])
    assert np.median(dE[-1]) < 1e-8


def test_rotating_frame_dop853(oracle, golden):
    d = golden("mw_rotating_dop853.npz")
    mw = W.mw_composite()
    H = g.Hamiltonian(mw, frame=g.ConstantRotatingFrame(Omega=d["omega"]))
    orbit = H.integrate_orbit(d["w0"], t=d["t"], Integrator="dop853",
                              Integrator_kwargs=dict(atol=1e-12, rtol=1e-10, nbatch=8))
    ref, _, _ = oracle.dop853(mw, d["w0"], d["t"], atol=1e-12, rtol=1e-10, nbatch=8,
                              frame=g.ConstantRotatingFrame(Omega=d["omega"]))
    assert np.max(rel_err(orbit.w(), ref)) <= PARITY
    assert np.max(rel_err(orbit.w()[:, ::50, :], d["w"])) <= 1e-11


def test_dop853_strided_output_identical():
    mw = W.mw_composite()
    w0 = W.mw_ics(30, seed=31)
    full = mw.integrate_orbit(w0, dt=0.5, n_steps=600, Integrator="dop853").w()
    strided = mw.integrate_orbit(w0, dt=0.5, n_steps=600, Integrator="dop853",
                                 Integrator_kwargs=dict(out_stride=100)).w()
    assert strided.shape == (6, 7, 30)
    assert np.array_equal(full[:, ::100, :], strided)


def test_dop853_nmax_failure_raises():
    mw = W.mw_composite()
    w0 = W.mw_ics(5, seed=32)
    with pytest.raises(RuntimeError, match="Integration failed with code -2"):
        mw.integrate_orbit(w0, dt=0.5, n_steps=200, Integrator="dop853", Integrator_kwargs=dict(nmax=3))
    # err_if_fail=0 returns whatever was integrated, no exception
    mw.integrate_orbit(w0, dt=0.5, n_steps=200, Integrator="dop853", Integrator_kwargs=dict(nmax=3, err_if_fail=0))


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_dop853_non_finite_initial_conditions_match_ieee_gala(oracle, bad):
    """A NaN or infinite initial condition: gala's dop853() with IEEE arithmetic
    rejects every step until nmax and reports -2 (its -Ofast build differs, see
    tests/test_oracle.py); the GPU has IEEE arithmetic and reports -2 too, for
    that orbit's batch only, with the same counters as the oracle."""
    import torch

    from gala_gb300 import _abi
    from gala_gb300._device import ptr, stream_handle

    pot = g.HernquistPotential(m=1e11, c=1.0)
    t = g.parse_time_specification(dt=1.0, n_steps=50)
    w0 = np.array([[8.0, 8.0], [0, 0], [0, 0], [0, 0], [0.2, 0.2], [0, 0]])
    w0[0, 1] = bad
    _, st_ref, stats_ref = oracle.dop853(pot, w0, t, nbatch=1, nmax=500)
    assert st_ref.tolist() == [1, -2]
    wd, td = torch.from_numpy(w0).cuda(), torch.from_numpy(t).cuda()
    out = torch.empty((6, len(t), 2), dtype=torch.float64, device="cuda")
    st = torch.zeros(2, dtype=torch.int32, device="cuda")
    stats = torch.zeros((2, 4), dtype=torch.int64, device="cuda")
    _abi.call("gx_dop853_integrate_hamiltonian", pot.packed().for_device(), g.Hamiltonian(pot)._frame_ref(), ptr(wd),
              2, ptr(td), len(t), 1e-10, 1e-10, 500, 0.0, 0, 1, 1, 1, ptr(out), ptr(st), ptr(stats), stream_handle())
    assert st.cpu().tolist() == [1, -2]
    np.testing.assert_array_equal(stats.cpu().numpy(), stats_ref)


# ----------------------------------------------------------------- edge cases
@pytest.mark.parametrize("method", ["leapfrog", "ruth4", "dop853"])
def test_single_orbit_shapes_and_save_all(oracle, method):
    pot = g.HernquistPotential(m=1e11, c=0.5)
    w0 = np.array([10.0, 0.0, 0.0, 0.0, 0.2, 0.02])
    orbit = pot.integrate_orbit(w0, dt=1.0, n_steps=100, Integrator=method)
    assert orbit.w().shape == (6, 101)
    assert orbit.t.shape == (101,)
    last = pot.integrate_orbit(w0, dt=1.0, n_steps=100, Integrator=method, save_all=False)
    assert last.w().shape == (6, 1)
    assert np.array_equal(last.w()[:, 0], orbit.w()[:, -1])
    assert last.t.shape == (1,) and last.t[0] == orbit.t[-1]


def test_empty_and_ragged_batches(oracle):
    mw = W.mw_composite()
    orbit = mw.integrate_orbit(np.zeros((6, 0)), dt=1.0, n_steps=10, Integrator="dop853")
    assert orbit.w().shape[-1] == 0
    w0 = W.mw_ics(257, seed=33)   # 2 full batches of 100 + one of 57; then nbatch 128 -> 128+128+1
    for nb in (100, 128, 256):
        w = mw.integrate_orbit(w0, dt=0.5, n_steps=200, Integrator="dop853",
                               Integrator_kwargs=dict(nbatch=nb)).w()
        ref, _, _ = oracle.dop853(mw, w0, g.parse_time_specification(dt=0.5, n_steps=200), nbatch=nb)
        assert np.max(rel_err(w, ref)) <= PARITY


def test_shift_rotate_integration(oracle):
    pot = _pots()["shifted_rotated"]
    w0 = W.mw_ics(64, seed=34)
    t = g.parse_time_specification(dt=1.0, n_steps=300)
    for method in ("leapfrog", "ruth4"):
        w = pot.integrate_orbit(w0, t=t, Integrator=method).w()
        ref = oracle.fixed(pot, w0, t, method)
        assert np.max(rel_err(w, ref)) <= PARITY


def test_invalid_arguments_raise():
    pot = g.HernquistPotential(m=1e11, c=0.5)
    with pytest.raises(ValueError):
        pot.integrate_orbit(np.zeros((4, 3)), dt=1.0, n_steps=10)
    with pytest.raises(ValueError):
        pot.integrate_orbit(np.ones((6, 3)), dt=0.0, t1=0.0, t2=1.0)
    with pytest.raises(TypeError):
        g.Hamiltonian(pot, frame=g.ConstantRotatingFrame([0, 0, 1.0])).integrate_orbit(
            np.ones((6, 3)), dt=1.0, n_steps=10, Integrator="leapfrog")
    with pytest.raises(ValueError):
        pot.integrate_orbit(np.ones((6, 3)), dt=1.0, n_steps=10, Integrator="dop853",
                            Integrator_kwargs=dict(nbatch=0))


# ------------------------------------------------------------------------ SCF
def test_scf_gpu_matches_fortran_and_oracle(oracle, golden):
    d = golden("scf_fortran.npz")
    for name in ["simple-hernquist", "multi-hernquist", "simple-nonsph", "random", "wang-zhao"]:
        pot = g.SCFPotential(m=1.0, r_s=1.0, Snlm=d[f"{name}/S"], Tnlm=d[f"{name}/T"])
        pot.G = 1.0
        gr = pot.gradient(d["xyz"])
        ph = pot.energy(d["xyz"])
        np.testing.assert_allclose(gr, d[f"{name}/grad"], rtol=1e-6)
        np.testing.assert_allclose(ph, d[f"{name}/pot"], rtol=1e-6)
        np.testing.assert_allclose(gr, oracle.gradient(pot, d["xyz"]), rtol=1e-10, atol=1e-14)
        np.testing.assert_allclose(ph, oracle.energy(pot, d["xyz"]), rtol=1e-10)
        np.testing.assert_allclose(pot.density(d["xyz"]), oracle.density(pot, d["xyz"]), rtol=1e-10, atol=1e-14)


def test_scf_leapfrog_matches_oracle(oracle):
    rng = np.random.default_rng(41)
    nmax, lmax = 6, 4
    S = rng.normal(size=(nmax + 1, lmax + 1, lmax + 1)) * np.exp(-0.5 * np.arange(nmax + 1))[:, None, None]
    T = rng.normal(size=S.shape) * np.exp(-0.5 * np.arange(nmax + 1))[:, None, None]
    for l in range(lmax + 1):
        S[:, l, l + 1:] = 0.0
        T[:, l, l + 1:] = 0.0
        T[:, l, 0] = 0.0
        S[:, l] *= (l + 1.0) ** -2
        T[:, l] *= (l + 1.0) ** -2
    S[0, 0, 0] = 1.0
    pot = g.SCFPotential(m=1e12, r_s=20.0, Snlm=S, Tnlm=T)
    w0 = W.mw_ics(32, seed=42)
    t = g.parse_time_specification(dt=1.0, n_steps=200)
    w = pot.integrate_orbit(w0, t=t, Integrator="leapfrog").w()
    ref = oracle.fixed(pot, w0, t, "leapfrog")
    assert np.max(rel_err(w, ref)) <= 1e-10


def test_fast64_forms_within_an_ulp():
    """The FP64 forms the DOP853 force uses in place of library calls -- the
    table-driven ln (Tang's method), sqrt and 1/x from FP32 seeds and two Newton
    steps -- against CUDA's log on the same GPU and numpy's log / sqrt / division
    (correctly rounded or within half an ulp): at most 2 ulp apart anywhere, at
    most 1 ulp for sqrt and 1/x.  Subnormal, zero and huge arguments take the
    library path."""
    import torch

    from gala_gb300 import _abi
    from gala_gb300._device import ptr, stream_handle

    rng = np.random.default_rng(3)
    x = np.concatenate([1 + rng.random(20000) * 10.0 ** rng.uniform(-8, 0.5, 20000),
                        10.0 ** rng.uniform(-300, 300, 20000), [1.0, 2.0, 0.5, 1e-310, 0.0, 1e300]])
    xd = torch.from_numpy(x).cuda()
    out = torch.empty((4, len(x)), dtype=torch.float64, device="cuda")
    _abi.call("gx_selfcheck_fast64", ptr(xd), len(x), ptr(out), stream_handle())
    torch.cuda.synchronize()
    ln_f, ln_cuda, sq, rc = out.cpu().numpy()
    with np.errstate(divide="ignore"):
        ln_np, sq_np, rc_np = np.log(x), np.sqrt(x), 1.0 / x
    fin = np.isfinite(ln_np) & (ln_np != 0)
    for ref in (ln_np, ln_cuda):
        assert np.max(np.abs(ln_f[fin] - ref[fin]) / np.spacing(np.abs(ref[fin]))) <= 2.0
    assert np.array_equal(ln_f[~fin], ln_np[~fin])
    assert np.max(np.abs(sq - sq_np) / np.spacing(sq_np + 1e-320)) <= 1.0
    ok = np.isfinite(rc_np)
    assert np.max(np.abs(rc[ok] - rc_np[ok]) / np.spacing(np.abs(rc_np[ok]))) <= 1.0
    assert np.array_equal(rc[~ok], rc_np[~ok])
