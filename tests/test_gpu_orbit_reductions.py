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
