"""Composites larger than the by-value descriptor (gala's test_no_max_n_components,
tests/potential/potential/test_composite.py:182-200: 1,024 shifted Hernquist
spheres).  The FP64 kernels read such a potential from a component table in
device memory; every result is checked against the oracle, which composes any
number of components."""
import numpy as np
import pytest

import gala_gb300 as g
from gala_gb300 import _abi

from .conftest import rel_err

pytestmark = pytest.mark.gpu


def _line_of_spheres(n=1024):
    ms = np.linspace(10, 100, n)                     # Msun
    x0 = np.linspace(-10e-3, 10e-3, n)                # kpc (gala: -10 .. 10 pc)
    return g.CompositePotential(**{f"yo{i}": g.HernquistPotential(m=ms[i], c=1e-4, origin=[x0[i], 0.0, 0.0])
                                   for i in range(n)})


def _points(n, seed):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.02, 0.5, n)
    u = rng.normal(size=(3, n))
    return r * u / np.linalg.norm(u, axis=0)


def test_large_composite_evaluation_matches_oracle(oracle):
    pot = _line_of_spheres()
    assert pot.packed().large
    q = _points(2000, 1)
    np.testing.assert_allclose(pot.gradient(q), oracle.gradient(pot, q), rtol=1e-13, atol=0)
    np.testing.assert_allclose(pot.energy(q), oracle.energy(pot, q), rtol=1e-13, atol=0)
    np.testing.assert_allclose(pot.density(q), oracle.density(pot, q), rtol=1e-12, atol=0)


def _ics(n, seed):
    rng = np.random.default_rng(seed)
    q = _points(n, seed)
    r = np.linalg.norm(q, axis=0)
    vc = np.sqrt(g.units.G * 56320.0 / r)             # total mass of the spheres
    a = rng.normal(size=(3, n))
    a -= np.sum(a * q, axis=0) * q / r ** 2
    return np.vstack([q, vc * a / np.linalg.norm(a, axis=0)])


def test_large_composite_orbits_match_oracle(oracle):
    pot = _line_of_spheres()
    w0 = _ics(64, 2)
    t = g.parse_time_specification(dt=5.0, n_steps=200)
    for method in ("leapfrog", "ruth4"):
        w = pot.integrate_orbit(w0, t=t, Integrator=method).w()
        ref = oracle.fixed(pot, w0, t, method)
        assert np.max(rel_err(w, ref)) <= 1e-13, method
    # DOP853 fuses its stage sums (the oracle, like gala, does not) and sums the
    # batch norm in another order; next to 1,024 sub-parsec spheres these
    # ulp-level differences grow faster than around the smooth MW composite
    # (measured 1.6e-12 at the worst output), hence 5e-12 here against 1e-12 there
    w = pot.integrate_orbit(w0, t=t, Integrator="dop853", Integrator_kwargs=dict(atol=1e-12, rtol=1e-10)).w()
    ref, st, _ = oracle.dop853(pot, w0, t, atol=1e-12, rtol=1e-10)
    assert np.all(st == 1)
    assert np.max(rel_err(w, ref)) <= 5e-12


def test_large_composite_fp32_forms_refuse():
    pot = _line_of_spheres(40)
    w0 = _ics(8, 3)
    with pytest.raises(_abi.GxError, match="GX_MAX_COMPONENTS"):
        pot.integrate_orbit(w0, dt=1.0, n_steps=10, Integrator="leapfrog", Integrator_kwargs=dict(precision="fp32c"))
