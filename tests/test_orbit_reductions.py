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
