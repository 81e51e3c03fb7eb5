"""CPU: the orbit-extremum oracle (gala's _max_helper restated with numpy /
scipy) on gala's own known-answer setting (tests/dynamics/test_orbit.py:
test_eccentricity and test_apocenter_pericenter_period), restated in galactic
units: an eccentric Kepler orbit whose apo- and pericentre follow from its
energy and angular momentum."""
import numpy as np
from scipy import optimize as so

import gala_gb300 as g
from oracle import orbit_oracle as OO


def _kepler_orbit(oracle, v_frac, n_steps=10000):
    pot = g.KeplerPotential(m=1e11)
    r0 = 10.0
    vc = np.sqrt(g.units.G * 1e11 / r0)
    period = 2 * np.pi * r0 / vc
    w0 = np.array([[r0], [0.0], [0.0], [0.0], [v_frac * vc], [0.0]])
    t = g.parse_time_specification(dt=period / 100, n_steps=n_steps)
    w, st, _ = oracle.dop853(pot, w0, t, atol=1e-12, rtol=1e-10)
    assert np.all(st == 1)
    return pot, w[:, :, 0], t


def test_circular_kepler_eccentricity(oracle):
    pot, w, t = _kepler_orbit(oracle, 1.0, n_steps=4000)
    assert abs(OO.eccentricity(w, t)[0]) < 1e-3


def test_eccentric_kepler_apo_peri(oracle):
    pot, w, t = _kepler_orbit(oracle, 0.75)
    apo = OO.reduce(w, t, "apo")[0]
    per = OO.reduce(w, t, "peri")[0]
    assert apo > per
    E = np.mean(oracle.hamiltonian_value(pot, w))
    L = np.mean(np.linalg.norm(np.cross(w[:3].T, w[3:].T), axis=1))

    def f(r):
        return 2 * (E - oracle.energy(pot, np.array([[r], [0.0], [0.0]]))[0]) - L ** 2 / r ** 2

    pred_apo = so.brentq(f, 9.0, 10.5)
    pred_per = so.brentq(f, 2.0, 6.0)
    np.testing.assert_allclose(apo, pred_apo, rtol=1e-2)
    np.testing.assert_allclose(per, pred_per, rtol=1e-2)
    apos, _ = OO.extrema(w, t, "apo")[0]
    pers, _ = OO.extrema(w, t, "peri")[0]
    assert 0 < np.std(apos) / np.mean(apos) < 1e-4
    assert 0 < np.std(pers) / np.mean(pers) < 1e-4


def test_parabola_refinement_on_a_sampled_cosine():
    """The parabola vertex recovers the peaks of a sampled smooth signal far
    better than the samples themselves."""
    t = np.linspace(0.0, 1000.0, 2001)
    f = 10.0 + 2.0 * np.cos(2 * np.pi * (t - 3.3) / 97.0)
    v, tt = OO.max_helper(f, t)
    va, _ = OO.max_helper(f, t, approximate=True)
    assert np.all(np.abs(v - 12.0) < 1e-6) and np.all(np.abs(va - 12.0) > np.abs(v - 12.0))
    np.testing.assert_allclose((tt - 3.3) / 97.0, np.round((tt - 3.3) / 97.0), atol=1e-4)


# -------------------------------------------------- guiding radius and periods
class _HostPotential:
    """The oracle's energy behind the potential interface guiding_radius uses."""

    def __init__(self, oracle, pot):
        self.oracle, self.pot = oracle, pot

    def energy(self, q, t=0.0):
        return self.oracle.energy(self.pot, q, t)


def _circular_mw_orbits(oracle, radii):
    from gala_gb300 import dynamics as D
    from gala_gb300 import workloads as W

    mw = W.mw_composite()
    e = _HostPotential(oracle, mw).energy
    dphi = D._d_dr_midplane(e, np.asarray(radii), 0.0)
    vc = np.sqrt(np.asarray(radii) * dphi)
    n = len(radii)
    w0 = np.zeros((6, n))
    w0[0], w0[4] = radii, vc
    t = g.parse_time_specification(dt=1.0, n_steps=1500)
    return mw, oracle.fixed(mw, w0, t, "leapfrog"), t


def test_guiding_radius_known_answer_and_gala_solver(oracle):
    """A circular midplane orbit's guiding radius is its radius; the vectorised
    solve agrees with gala's scipy 'hybr' solve (orbit.py:555-599) to 1e-8
    (measured 1e-10: hybr stops at xtol 1e-5 of its step, near the root that
    is far inside; the finite-difference dPhi/dR carries ~1e-11 noise)."""
    from gala_gb300 import dynamics as D
    from gala_gb300 import workloads as W

    radii = np.array([3.0, 8.0, 15.0, 25.0])
    mw, w, t = _circular_mw_orbits(oracle, radii)
    hp = _HostPotential(oracle, mw)
    orbit = g.Orbit.from_w(w, t=t)
    Rg = orbit.guiding_radius(potential=hp)
    np.testing.assert_allclose(Rg, radii, rtol=1e-6)   # the leapfrog orbit is circular to ~1e-7
    np.testing.assert_allclose(Rg, OO.guiding_radius(w, hp.energy), rtol=1e-8)
    # generic disk orbits
    w0 = W.mw_ics(24, seed=12)
    w2 = oracle.fixed(mw, w0, t, "leapfrog")
    o2 = g.Orbit.from_w(w2, t=t)
    np.testing.assert_allclose(o2.guiding_radius(potential=hp), OO.guiding_radius(w2, hp.energy), rtol=1e-8)
    # one orbit returns a scalar, as gala's does
    one = g.Orbit.from_w(w2[:, :, 3], t=t)
    assert np.ndim(one.guiding_radius(potential=hp)) == 0
    # edge cases of the solve: L_z = 0 -> 0, a bad start -> nan
    out = D._guiding_radius_solve(np.array([5.0, np.nan, 5.0]), np.array([0.0, 1.0, 1.0]),
                                  lambda R: D._d_dr_midplane(hp.energy, R, 0.0))
    assert out[0] == 0.0 and np.isnan(out[1]) and np.isfinite(out[2])


def test_guiding_radius_warns_for_varying_lz(oracle):
    import pytest

    from gala_gb300 import workloads as W

    tri = g.NFWPotential(m=5e11, r_s=15.0, a=1.0, b=0.8, c=0.6)
    t = g.parse_time_specification(dt=1.0, n_steps=800)
    w = oracle.fixed(tri, W.mw_ics(4, seed=3), t, "leapfrog")
    with pytest.warns(RuntimeWarning, match="constant Lz"):
        g.Orbit.from_w(w, t=t).guiding_radius(potential=_HostPotential(oracle, tri))
    with pytest.raises(ValueError, match="potential"):
        g.Orbit.from_w(w, t=t).guiding_radius()


def test_estimate_period_known_answer_and_gala(oracle):
    """Kepler circular orbit: every coordinate's period is 2 pi r / v_c; and the
    product's peak finder agrees with gala's argrelmax form on MW orbits."""
    import pytest

    from gala_gb300 import dynamics as D
    from gala_gb300 import workloads as W

    pot, w, t = _kepler_orbit(oracle, 1.0, n_steps=1000)
    r0, vc = 10.0, np.sqrt(g.units.G * 1e11 / 10.0)
    P = g.Orbit.from_w(w, t=t).estimate_period()
    assert set(P) == {"x", "y", "z"}
    np.testing.assert_allclose([P["x"][0], P["y"][0]], 2 * np.pi * r0 / vc, rtol=2e-3)
    assert np.isnan(P["z"][0])   # z stays 0: below the amplitude threshold
    mw = W.mw_composite()
    t2 = g.parse_time_specification(dt=1.0, n_steps=3000)
    w2 = oracle.fixed(mw, W.mw_ics(12, seed=8), t2, "leapfrog")
    P2 = g.Orbit.from_w(w2, t=t2).estimate_period()
    for k, name in enumerate("xyz"):
        ref = np.array([OO.peak_to_peak_period(t2, w2[k, :, n]) for n in range(12)])
        np.testing.assert_array_equal(P2[name], ref)
    assert np.isnan(D.peak_to_peak_period(np.arange(5.0), np.zeros(5)))
    with pytest.raises(ValueError, match="time array"):
        g.Orbit(pos=w2[:3], vel=w2[3:]).estimate_period()


# -------------------------------------------------- gala's tests/dynamics/test_orbit.py settings
def test_peak_to_peak_period_known_answer():
    """test_estimate_period (test_orbit.py:449-470): R(t) = 0.25 sin(2 pi t / T) + 1
    over t in [0, 10] with 16384 samples gives T to 1e-3; the azimuth 2 pi t mod
    2 pi gives 1."""
    from gala_gb300.dynamics import peak_to_peak_period

    t = np.linspace(0, 10.0, 16384)
    for true_T in (1.0, 2.0, 4.123):
        R = 0.25 * np.sin(2 * np.pi / true_T * t) + 1.0
        assert np.isclose(peak_to_peak_period(t, R), true_T, rtol=1e-3)
        assert np.isclose(OO.peak_to_peak_period(t, R), true_T, rtol=1e-3)
    phi = (2 * np.pi * t) % (2 * np.pi)
    assert np.isclose(peak_to_peak_period(t, phi), 1.0, rtol=1e-3)
    pos = np.zeros((3, len(t)))
    pos[0], pos[1] = np.cos(phi), np.sin(phi)
    P = g.Orbit(pos=pos, vel=np.zeros_like(pos), t=t).estimate_period()
    assert set(P) == {"x", "y", "z"}


def _gala_guiding_cases():
    """test_guiding_radius (test_orbit.py:363-380): from (10, 0, 0) kpc at 1.3 v_c in
    a Hernquist sphere (no warning) and in an NFW halo with b = 0.95 (warning)."""
    cases = []
    for pot, warns in ((g.HernquistPotential(m=1e10, c=10.0), False),
                       (g.NFWPotential(m=1e10, r_s=10.0, b=0.95), True)):
        cases.append((pot, warns))
    return cases


def test_gala_guiding_radius_setting_oracle(oracle):
    import warnings

    import pytest

    t = g.parse_time_specification(dt=0.5, n_steps=1000)
    for pot, warns in _gala_guiding_cases():
        q = np.array([[10.0], [0.0], [0.0]])
        vc = np.sqrt(10.0 * np.abs(oracle.gradient(pot, q)[0, 0]))
        w0 = np.array([[10.0], [0.0], [0.0], [0.0], [1.3 * vc], [0.0]])
        w, st, _ = oracle.dop853(pot, w0, t)
        assert np.all(st == 1)
        orbit = g.Orbit.from_w(w[:, :, 0], t=t)
        hp = _HostPotential(oracle, pot)
        if warns:
            with pytest.warns(RuntimeWarning):
                orbit.guiding_radius(potential=hp)
        else:
            with warnings.catch_warnings():
                warnings.simplefilter("error")
                Rg = orbit.guiding_radius(potential=hp)
            assert 10.0 < Rg < 30.0   # 1.3 v_c: outside the start, the orbit's apocentre side
