"""GPU orbit extrema (Orbit.pericenter / apocenter / zmax / eccentricity) against
the oracle (gala's _max_helper with numpy polyfit).

The GPU refines each extremum with the same 3-point parabola written in
coordinates centred on the middle sample; gala's polyfit works on the raw
times, so the two differ by gala's own cancellation error (relative ~1e-12 for
these grids): values are compared at rtol 1e-9, times at 1e-9 of the time span.
The extremum sets (counts) must agree exactly; approximate=True (the samples
themselves) must agree to an ulp of hypot."""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import workloads as W
from oracle import orbit_oracle as OO

pytestmark = pytest.mark.gpu


def _mw_orbits(n=48, dt=1.0, n_steps=2500):
    mw = W.mw_composite()
    w0 = W.mw_ics(n, seed=77)
    return mw.integrate_orbit(w0, dt=dt, n_steps=n_steps, Integrator="leapfrog")


@pytest.mark.parametrize("dt", [1.0, -1.0])
def test_extrema_match_oracle(dt):
    orbit = _mw_orbits(dt=dt)
    w, t = orbit.w(), orbit.t
    span = abs(t[-1] - t[0])
    for kind, meth in (("peri", orbit.pericenter), ("apo", orbit.apocenter), ("zmax", orbit.zmax)):
        ref = OO.extrema(w, t, kind)
        vals, times = meth(func=None, return_times=True)
        assert len(vals) == len(ref)
        for (rv, rt), v, tt in zip(ref, vals, times):
            assert len(v) == len(rv)
            np.testing.assert_allclose(v, rv, rtol=1e-9, atol=0)
            np.testing.assert_allclose(tt, rt, rtol=0, atol=1e-9 * span)
        np.testing.assert_allclose(meth(), OO.reduce(w, t, kind), rtol=1e-9)
        np.testing.assert_allclose(meth(func=np.min), OO.reduce(w, t, kind, np.min), rtol=1e-9)
        np.testing.assert_allclose(meth(func=np.max), OO.reduce(w, t, kind, np.max), rtol=1e-9)
        np.testing.assert_allclose(meth(approximate=True), OO.reduce(w, t, kind, approximate=True), rtol=1e-14)
    np.testing.assert_allclose(orbit.eccentricity(), OO.eccentricity(w, t), rtol=1e-8)


def test_single_orbit_shapes_and_device_orbit():
    mw = W.mw_composite()
    w0 = W.mw_ics(1, seed=78)[:, 0]
    o_dev = mw.integrate_orbit(w0, dt=0.5, n_steps=3000, Integrator="dop853", return_device=True)
    peri = o_dev.pericenter()
    assert np.ndim(peri) == 0
    o = mw.integrate_orbit(w0, dt=0.5, n_steps=3000, Integrator="dop853")
    np.testing.assert_allclose(peri, OO.reduce(o.w(), o.t, "peri")[0], rtol=1e-9)
    v, tt = o.apocenter(func=None, return_times=True)
    assert v.ndim == 1 and tt.shape == v.shape
    with pytest.raises(ValueError):
        o.apocenter(return_times=True)
    # another callable reduces all extrema on the host
    np.testing.assert_allclose(o.zmax(func=np.median), np.median(OO.extrema(o.w(), o.t, "zmax")[0][0]), rtol=1e-9)


def test_too_short_orbit_gives_nan():
    mw = W.mw_composite()
    o = mw.integrate_orbit(W.mw_ics(3, seed=79), dt=1.0, n_steps=1, Integrator="leapfrog")
    assert np.all(np.isnan(o.pericenter()))


def _check_all(orbit, approx_rtol=1e-14):
    w, t = orbit.w(), orbit.t
    span = abs(t[-1] - t[0])
    for kind, meth in (("peri", orbit.pericenter), ("apo", orbit.apocenter), ("zmax", orbit.zmax)):
        ref = OO.extrema(w, t, kind)
        vals, times = meth(func=None, return_times=True)
        for (rv, rt), v, tt in zip(ref, vals, times):
            assert len(v) == len(rv)
            np.testing.assert_allclose(v, rv, rtol=1e-9, atol=0)
            np.testing.assert_allclose(tt, rt, rtol=0, atol=1e-9 * span)
        cnt = np.array([len(rv) for rv, _ in ref])
        for func in (np.mean, np.min, np.max):
            got = meth(func=func)
            exp = np.array([func(rv) if len(rv) else np.nan for rv, _ in ref])
            np.testing.assert_allclose(got, exp, rtol=1e-9)
            assert np.array_equal(np.isnan(got), cnt == 0)
        np.testing.assert_allclose(meth(approximate=True),
                                   np.array([np.mean(rv) if len(rv) else np.nan
                                             for rv, _ in OO.extrema(w, t, kind, approximate=True)]),
                                   rtol=approx_rtol)


def test_dense_extrema_fill_the_staging_rings():
    """Zig-zag samples: about a third of all samples are strict local maxima of
    |z| and of r, so every warp stages and checks its candidates many times per
    chunk of samples; 300 orbits (two full 128-orbit blocks and a ragged one)
    and 1,003 samples (not a multiple of the 8-sample chunk)."""
    rng = np.random.default_rng(5)
    n, nt = 300, 1003
    t = np.linspace(0.0, 50.0, nt)
    sign = np.where(np.arange(nt) % 2 == 0, 1.0, -1.0)[:, None]
    pos = np.empty((3, nt, n))
    pos[0] = 5.0 + rng.uniform(-1, 1, (nt, n))
    pos[1] = rng.uniform(-2, 2, (nt, n))
    pos[2] = sign * (1.0 + 0.5 * rng.uniform(0, 1, (nt, n)))
    vel = np.zeros_like(pos)
    _check_all(g.Orbit(pos=pos, vel=vel, t=t), approx_rtol=1e-13)


def test_planar_and_smooth_orbits_ragged_sizes():
    """Orbits in the plane z = 0 (no z maxima at all: NaN statistics) beside
    smooth epicyclic orbits, with a descending time grid and 37 orbits."""
    n, nt = 37, 2005
    t = np.linspace(100.0, 0.0, nt)
    ph = np.linspace(0, 2 * np.pi, n, endpoint=False)[None, :]
    tt = t[:, None]
    R = 8.0 + 1.5 * np.cos(0.37 * tt + ph)
    pos = np.stack([R * np.cos(0.11 * tt), R * np.sin(0.11 * tt), 0.7 * np.sin(0.53 * tt + 2 * ph)])
    pos[2, :, ::3] = 0.0
    _check_all(g.Orbit(pos=pos, vel=np.zeros_like(pos), t=t))
    z = g.Orbit(pos=pos, vel=np.zeros_like(pos), t=t).zmax()
    assert np.all(np.isnan(z[::3])) and not np.any(np.isnan(np.delete(z, np.s_[::3])))


def test_guiding_radius_and_periods_match_oracle(oracle):
    """Orbit.guiding_radius evaluates the potential on the GPU (one call per
    solver step for all orbits) and must agree with gala's scipy 'hybr' solve on
    the oracle's potential to 1e-7.  The central difference of step 1e-4 in
    c_d_dr amplifies a relative difference of the two potentials about 1e6-fold
    in R_g (2e-15 of noise gives 2e-9); the potential tests bound that
    difference by 1e-14, so 1e-7 keeps a tenfold margin.  estimate_period runs
    gala's peak-to-peak estimate on the orbit."""
    orbit = _mw_orbits(n=32, dt=1.0, n_steps=3000)
    w, t = orbit.w(), orbit.t
    mw = orbit.potential
    Rg = orbit.guiding_radius()
    ref = OO.guiding_radius(w, lambda q, tt: oracle.energy(mw, q, tt))
    np.testing.assert_allclose(Rg, ref, rtol=1e-7)
    P = orbit.estimate_period()
    for k, name in enumerate("xyz"):
        np.testing.assert_array_equal(P[name], [OO.peak_to_peak_period(t, w[k, :, n]) for n in range(32)])


def test_gala_orbit_settings():
    """gala's test_orbit.py on the CUDA path:
    * test_guiding_radius (:363-380): Hernquist runs quietly, NFW with b = 0.95 warns;
    * test_apocenter_pericenter_period (:383-446), point mass with G m = 4 pi^2 (gala's
      solar-system numbers): apo- and pericentre within 1e-2 of the roots of
      2 (E - Phi(r)) - L^2 / r^2, scatter of the individual extrema below 1e-4,
      and the multi-orbit approximate calls."""
    import warnings

    from scipy import optimize as so

    for pot, warns in ((g.HernquistPotential(m=1e10, c=10.0), False),
                       (g.NFWPotential(m=1e10, r_s=10.0, b=0.95), True)):
        vc = pot.circular_velocity(np.array([[10.0], [0.0], [0.0]]))[0]
        orbit = pot.integrate_orbit(np.array([10.0, 0, 0, 0, 1.3 * vc, 0]), dt=0.5, n_steps=1000,
                                    Integrator="dop853")
        if warns:
            with pytest.warns(RuntimeWarning):
                orbit.guiding_radius()
        else:
            with warnings.catch_warnings():
                warnings.simplefilter("error")
                assert np.isfinite(orbit.guiding_radius())

    pot = g.KeplerPotential(m=4 * np.pi ** 2 / g.units.G)
    w = pot.integrate_orbit(np.array([1.0, 0, 0, 0, 1.5 * np.pi, 0]), dt=0.01, n_steps=10000, Integrator="dop853")
    apo, per, zmax = w.apocenter(), w.pericenter(), w.zmax()
    assert np.shape(apo) == np.shape(per) == np.shape(zmax) == () and apo > per
    E = np.mean(w.energy())
    L = np.mean(np.linalg.norm(w.angular_momentum(), axis=0))

    def func(r):
        return 2 * (E - pot.energy(np.array([[r], [0.0], [0.0]]))[0]) - L ** 2 / r ** 2

    assert np.isclose(apo, so.brentq(func, 0.9, 1.0), rtol=1e-2)
    assert np.isclose(per, so.brentq(func, 0.3, 0.5), rtol=1e-2)
    apos, pers = np.asarray(w.apocenter(func=None)), np.asarray(w.pericenter(func=None))
    assert 0 < np.std(apos) / np.mean(apos) < 1e-4 and 0 < np.std(pers) / np.mean(pers) < 1e-4
    w2 = pot.integrate_orbit(np.array([[1.0, 1.1], [0, 0], [0, 0], [0, 0], [1.5 * np.pi] * 2, [0, 0]]), dt=0.01,
                             n_steps=10000)
    for f in (w2.pericenter, w2.apocenter, w2.zmax, w2.eccentricity):
        assert np.shape(f(approximate=True)) == (2,)
