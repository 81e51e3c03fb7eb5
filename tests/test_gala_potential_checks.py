"""gala's own potential and integrator checks, run twice: on the oracle (CPU)
and on the CUDA path (marked gpu).

* numerical gradient vs gradient: 16 random points within twice |w0|,
  finite-difference step 1e-3 |w0|, rtol 1e-5 (potential_helpers.py:265-299);
* numerical Laplacian vs 4 pi G rho, rtol 1e-2 (:301-347);
* rotation / shift: a rotated or shifted copy equals the original evaluated at
  R (x - x0), gradients rotated back (:518-546);
* scalar positions are refused with ValueError (test_regression_165, :505-516);
* point-mass closure: a circular orbit returns to its start after one period
  at atol 1e-6 (tests/integrate/test_pyintegrators.py:96-104).

The canonical instances are gala's (canonical_potentials.py:18-70) in galactic
units; gala's Kepler instance is in solar-system units, so here the point mass
is 1e11 Msun at 10 kpc.  gala differentiates with the findiff package on a
9-point stencil; this file uses fourth-order central differences.
"""
import numpy as np
import pytest

import gala_gb300 as g

CANONICAL = {
    # name: (potential, w0, has density)
    "kepler": (g.KeplerPotential(m=1e11), [10.0, 0.0, 0.0, 0.0, 0.2, 0.0], False),
    "hernquist": (g.HernquistPotential(m=1e11, c=0.26), [1.0, 0.0, 0.0, 0.0, 0.1, 0.1], True),
    "plummer": (g.PlummerPotential(m=1e11, b=0.26), [1.0, 0.0, 0.0, 0.0, 0.1, 0.1], True),
    "miyamotonagai": (g.MiyamotoNagaiPotential(m=1e11, a=6.5, b=0.26), [8.0, 0.0, 0.0, 0.0, 0.22, 0.1], True),
    "sphericalnfw": (g.NFWPotential(m=1e11, r_s=12.0), [19.0, 2.7, -6.9, 0.0352238, -0.03579493, 0.075], True),
    "flattenednfw": (g.NFWPotential(m=1e11, r_s=12.0, c=0.7), [19.0, 2.7, -6.9, 0.0352238, -0.03579493, 0.075],
                     False),
    "triaxialnfw": (g.NFWPotential(m=1e11, r_s=12.0, a=1.0, b=0.95, c=0.9),
                    [19.0, 2.7, -6.9, 0.0352238, -0.03579493, 0.075], False),
    "milkyway": (g.MilkyWayPotential(), [8.0, 0.0, 0.0, 0.0, 0.22, 0.1], True),
}
ROTATED = ("miyamotonagai", "flattenednfw", "triaxialnfw")


def _points(name, seed=42):
    w0 = np.asarray(CANONICAL[name][1])
    r = np.linalg.norm(w0[:3])
    rng = np.random.default_rng(seed)
    return rng.uniform(-2 * r, 2 * r, size=(3, 16)), 1e-3 * r


def _stencil(pts, dx):
    """(3, 16, 3, 5) points: for each axis the offsets -2..2 dx around each point."""
    out = np.repeat(pts[:, :, None, None], 3, axis=2).repeat(5, axis=3)
    for k in range(3):
        out[k, :, k, :] += np.arange(-2, 3) * dx
    return out


def check_gradient(name, energy, gradient):
    pts, dx = _points(name)
    phi = energy(_stencil(pts, dx).reshape(3, -1)).reshape(16, 3, 5)
    num = (phi[..., 0] - 8 * phi[..., 1] + 8 * phi[..., 3] - phi[..., 4]) / (12 * dx)
    assert np.allclose(gradient(pts), num.T, rtol=1e-5)


def check_density(name, energy, density):
    pts, dx = _points(name)
    phi = energy(_stencil(pts, dx).reshape(3, -1)).reshape(16, 3, 5)
    d2 = (-phi[..., 0] + 16 * phi[..., 1] - 30 * phi[..., 2] + 16 * phi[..., 3] - phi[..., 4]) / (12 * dx * dx)
    assert np.allclose(4 * np.pi * g.units.G * density(pts), d2.sum(axis=1), rtol=1e-2)


def check_rotation_shift(name, evaluate):
    """evaluate(potential, kind, x) -> values (kind: energy / gradient / density)."""
    pot = CANONICAL[name][0]
    x = np.array([10.0, 5.0, 3.0])[:, None]
    x0 = np.array([1.0, 1.0, 3.0])
    R = np.array([[0.0, 1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    kinds = ("energy", "gradient") + (("density",) if CANONICAL[name][2] else ())
    for kind in kinds:
        base = lambda q: evaluate(pot, kind, q)  # noqa: E731
        back = (lambda v: R.T @ v) if kind == "gradient" else (lambda v: v)
        np.testing.assert_allclose(evaluate(pot.replicate(R=R), kind, x), back(base(R @ x)), rtol=1e-13)
        np.testing.assert_allclose(evaluate(pot.replicate(origin=x0), kind, x), base(x - x0[:, None]), rtol=1e-13)
        np.testing.assert_allclose(evaluate(pot.replicate(R=R, origin=x0), kind, x),
                                   back(base(R @ (x - x0[:, None]))), rtol=1e-13)


def _unit_point_mass():
    """G m = 1: the circular orbit at r = 1 kpc has v = 1 kpc/Myr, period 2 pi Myr."""
    pot = g.KeplerPotential(m=1.0 / g.units.G)
    w0 = np.array([[1.0], [0.0], [0.0], [0.0], [1.0], [0.0]])
    t = g.parse_time_specification(t1=0.0, t2=2 * np.pi, n_steps=10_000)
    return pot, w0, t


# ---------------------------------------------------------------- oracle (CPU)
@pytest.mark.parametrize("name", sorted(CANONICAL))
def test_oracle_gradient_is_the_numerical_gradient(oracle, name):
    pot = CANONICAL[name][0]
    check_gradient(name, lambda q: oracle.energy(pot, q), lambda q: oracle.gradient(pot, q))


@pytest.mark.parametrize("name", sorted(n for n in CANONICAL if CANONICAL[n][2]))
def test_oracle_density_is_the_laplacian(oracle, name):
    pot = CANONICAL[name][0]
    check_density(name, lambda q: oracle.energy(pot, q), lambda q: oracle.density(pot, q))


@pytest.mark.parametrize("name", ROTATED)
def test_oracle_rotation_shift(oracle, name):
    check_rotation_shift(name, lambda p, kind, q: getattr(oracle, kind)(p, q))


def test_scalar_positions_are_refused():
    pot = CANONICAL["miyamotonagai"][0]
    for meth in (pot.energy, pot.gradient, pot.circular_velocity):
        with pytest.raises(ValueError):
            meth(8.0)


@pytest.mark.parametrize("method", ["leapfrog", "ruth4", "dop853"])
def test_oracle_point_mass_orbit_closes(oracle, method):
    pot, w0, t = _unit_point_mass()
    if method == "dop853":
        w, st, _ = oracle.dop853(pot, w0, t, atol=1e-10, rtol=1e-10)
        assert np.all(st == 1)
    else:
        w = oracle.fixed(pot, w0, t, method)
    assert np.allclose(w[:, 0, 0], w[:, -1, 0], atol=1e-6)


# ---------------------------------------------------------------- CUDA path
@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CANONICAL))
def test_gpu_gradient_is_the_numerical_gradient(name):
    pot = CANONICAL[name][0]
    check_gradient(name, pot.energy, pot.gradient)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(n for n in CANONICAL if CANONICAL[n][2]))
def test_gpu_density_is_the_laplacian(name):
    pot = CANONICAL[name][0]
    check_density(name, pot.energy, pot.density)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ROTATED)
def test_gpu_rotation_shift(name):
    check_rotation_shift(name, lambda p, kind, q: getattr(p, kind)(q))


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["leapfrog", "ruth4", "dop853"])
def test_gpu_point_mass_orbit_closes(method):
    pot, w0, t = _unit_point_mass()
    kw = dict(Integrator_kwargs=dict(atol=1e-10, rtol=1e-10)) if method == "dop853" else {}
    w = pot.integrate_orbit(w0, t=t, Integrator=method, **kw).w()
    assert np.allclose(w[:, 0], w[:, -1], atol=1e-6)


# ---------------------------------------------------------------- rotating frames
# tests/potential/hamiltonian/test_with_frame_potential.py:118-177, with G m = 1
# (the same numbers as gala's dimensionless units): a circular orbit co-rotating
# with the frame stays put; with Omega = (1, 1, 1) the Jacobi constant
# H - Omega . L (H = p^2/2 + Phi - Omega . L, builtin_frames.cpp:73-94) holds to 1e-9.
def _rotating_cases():
    pot = g.KeplerPotential(m=1.0 / g.units.G)
    co = (g.ConstantRotatingFrame(Omega=[0.0, 0.0, 1.0]), np.array([[1.0], [0], [0], [0], [1.0], [0]]),
          g.parse_time_specification(dt=1.0, n_steps=1000), dict(atol=1e-10, rtol=1e-10))
    off = (g.ConstantRotatingFrame(Omega=[1.0, 1.0, 1.0]), np.array([[1.0], [0], [0], [0], [1.1], [0]]),
           g.parse_time_specification(dt=0.1, n_steps=10000), dict(atol=1e-12, rtol=1e-12))
    return pot, co, off


def check_rotating(integrate, hamiltonian_value):
    pot, co, off = _rotating_cases()
    frame, w0, t, kw = co
    w = integrate(pot, frame, w0, t, kw)
    assert np.allclose(w[0], 1.0, atol=1e-7) and np.allclose(w[1:3], 0.0, atol=1e-7)
    frame, w0, t, kw = off
    w = integrate(pot, frame, w0, t, kw)
    L = np.cross(w[:3], w[3:], axis=0)
    C = hamiltonian_value(pot, frame, w) - np.sum(frame.Omega[:, None] * L, axis=0)
    assert np.all(np.abs((C[1:] - C[0]) / C[0]) < 1e-9)


def test_oracle_rotating_frame_kepler(oracle):
    def integrate(pot, frame, w0, t, kw):
        w, st, _ = oracle.dop853(pot, w0, t, frame=frame, **kw)
        assert np.all(st == 1)
        return w[:, :, 0]

    check_rotating(integrate, lambda pot, frame, w: oracle.hamiltonian_value(pot, w, frame=frame))


@pytest.mark.gpu
def test_gpu_rotating_frame_kepler():
    def integrate(pot, frame, w0, t, kw):
        return g.Hamiltonian(pot, frame=frame).integrate_orbit(w0, t=t, Integrator="dop853",
                                                               Integrator_kwargs=kw).w()

    check_rotating(integrate, lambda pot, frame, w: g.Hamiltonian(pot, frame=frame).energy(w))


# ---------------------------------------------------------------- composite vs Python integrators
# tests/potential/potential/test_composite.py:58-88: Kepler (1 Msun) + Hernquist
# (0.5 Msun, c = 0.1 au) in solar-system units from (1 au, 2 pi au/yr), dt 0.01,
# 1000 steps; the C integrators (DOP853 at atol = rtol = 1e-14, Leapfrog) agree
# with gala's Python ones -- scipy's dop853 and the Python leapfrog
# (pyintegrators/leapfrog.py:131-138) -- within np.allclose.  gala runs scipy at
# its default rtol 1e-6, whose own error puts one velocity near a zero crossing
# 1.1e-7 off (outside allclose's atol 1e-8); here scipy runs at 1e-14 as well,
# and the two DOP853 codes agree to 5e-10.  G m = 4 pi^2 and 2 pi^2 in galactic
# units give the same numbers as gala's solar-system units.
def _composite_case():
    pot = g.CCompositePotential(one=g.KeplerPotential(m=4 * np.pi ** 2 / g.units.G),
                                two=g.HernquistPotential(m=2 * np.pi ** 2 / g.units.G, c=0.1))
    w0 = np.array([1.0, 0, 0, 0, 2 * np.pi, 0])
    t = g.parse_time_specification(dt=0.01, n_steps=1000)
    return pot, w0, t


def _python_dop853(gradient, w0, t):
    """gala's DOPRI853Integrator: scipy's ode('dop853') stepped to each output time."""
    from scipy.integrate import ode

    def rhs(_, w):
        return np.concatenate([w[3:], -gradient(w[:3, None])[:, 0]])

    solver = ode(rhs).set_integrator("dop853", atol=1e-14, rtol=1e-14)
    solver.set_initial_value(w0, t[0])
    out = [w0]
    for tk in t[1:]:
        solver.integrate(tk)
        assert solver.successful()
        out.append(solver.y)
    return np.array(out).T


def _python_leapfrog(gradient, w0, t):
    """gala's Python LeapfrogIntegrator: half-kick start, drift, kick (leapfrog.py:90-138)."""
    dt = t[1] - t[0]
    x, v = w0[:3].copy(), w0[3:].copy()
    v_half = v - 0.5 * dt * gradient(x[:, None])[:, 0]
    out = [w0]
    for _ in t[1:]:
        x = x + v_half * dt
        a = -gradient(x[:, None])[:, 0]
        v = v_half + 0.5 * dt * a
        v_half = v_half + dt * a
        out.append(np.concatenate([x, v]))
    return np.array(out).T


def check_composite(integrate, gradient):
    pot, w0, t = _composite_case()
    w_c = integrate(pot, w0, t, "dop853")
    w_py = _python_dop853(lambda q: gradient(pot, q), w0, t)
    assert np.allclose(w_c[:3], w_py[:3]) and np.allclose(w_c[3:], w_py[3:])
    w_c = integrate(pot, w0, t, "leapfrog")
    w_py = _python_leapfrog(lambda q: gradient(pot, q), w0, t)
    assert np.allclose(w_c[:3], w_py[:3]) and np.allclose(w_c[3:], w_py[3:])


def test_oracle_composite_matches_python_integrators(oracle):
    def integrate(pot, w0, t, method):
        if method == "dop853":
            w, st, _ = oracle.dop853(pot, w0[:, None], t, atol=1e-14, rtol=1e-14)
            assert np.all(st == 1)
            return w[:, :, 0]
        return oracle.fixed(pot, w0[:, None], t, method)[:, :, 0]

    check_composite(integrate, oracle.gradient)


@pytest.mark.gpu
def test_gpu_composite_matches_python_integrators():
    def integrate(pot, w0, t, method):
        kw = dict(Integrator_kwargs=dict(atol=1e-14, rtol=1e-14)) if method == "dop853" else {}
        return pot.integrate_orbit(w0, t=t, Integrator=method, **kw).w()

    check_composite(integrate, lambda pot, q: pot.gradient(q))


# ---------------------------------------------------------------- enclosed mass
def check_mass_enclosed(with_energy):
    """r^2 |dPhi/dr| / G with gala's step 1e-3 (core.py:649-707): the Hernquist
    M(<r) = m r^2 / (r + c)^2 and the Kepler mass, to the difference's accuracy."""
    hern = with_energy(g.HernquistPotential(m=1e11, c=0.26))
    q = np.array([[1.0, 5.0, 30.0], [0.5, 0.0, -4.0], [0.2, 2.0, 1.0]])
    r = np.linalg.norm(q, axis=0)
    np.testing.assert_allclose(hern.mass_enclosed(q), 1e11 * r ** 2 / (r + 0.26) ** 2, rtol=1e-5)
    kep = with_energy(g.KeplerPotential(m=3e10))
    np.testing.assert_allclose(kep.mass_enclosed(q[:, :, None]), np.full((3, 1), 3e10), rtol=1e-5)
    neg = with_energy(g.KeplerPotential(m=-3e10))
    assert np.all(neg.mass_enclosed(q) < 0)


def test_oracle_mass_enclosed(oracle):
    def with_energy(pot):
        pot.energy = lambda q, t=0.0: oracle.energy(pot, q, t)  # the oracle behind the API
        return pot

    check_mass_enclosed(with_energy)
    with pytest.raises(ValueError):
        g.KeplerPotential(m=1.0).mass_enclosed(3.0)


@pytest.mark.gpu
def test_gpu_mass_enclosed():
    check_mass_enclosed(lambda pot: pot)


# ---------------------------------------------------------------- NFW (test_all_builtin.py:255-342)
def check_nfw(gradient, mass_enclosed):
    """Flattened NFW differs from spherical (regression for gala issue #254);
    from_circular_velocity gives v_c at r_ref; the enclosed mass follows
    m (ln(1 + r/r_s) - (r/r_s) / (1 + r/r_s)) to 1e-6 for r in [1, 400] kpc."""
    w0 = np.array([19.0, 2.7, -6.9])[:, None]
    flat = g.NFWPotential(m=1e11, r_s=12.0, c=0.7)
    sph = g.NFWPotential(m=1e11, r_s=12.0)
    assert not np.allclose(gradient(flat, w0), gradient(sph, w0))
    vc = 220.0 * g.units.KMS_TO_KPC_MYR
    for r_ref in (3.0, 8.0, 21.7234):
        pot = g.NFWPotential.from_circular_velocity(v_c=vc, r_s=20.0, r_ref=r_ref)
        q = np.array([[r_ref], [0.0], [0.0]])
        assert np.allclose(np.sqrt(r_ref * np.abs(gradient(pot, q)[0, 0])), vc)
    pot = g.NFWPotential.from_circular_velocity(v_c=vc, r_s=20.0, r_ref=8.0)
    m, rs = pot.parameters["m"], pot.parameters["r_s"]
    r = np.linspace(1.0, 400.0, 100)
    R = np.zeros((3, len(r)))
    R[0] = r
    true = m * (np.log(1 + r / rs) - (r / rs) / (1 + r / rs))
    assert np.allclose(true, mass_enclosed(pot, R), rtol=1e-6)


def test_oracle_nfw_checks(oracle):
    def menc(pot, R):
        pot.energy = lambda q, t=0.0: oracle.energy(pot, q, t)
        return pot.mass_enclosed(R)

    check_nfw(lambda pot, q: oracle.gradient(pot, q), menc)


@pytest.mark.gpu
def test_gpu_nfw_checks():
    check_nfw(lambda pot, q: pot.gradient(q), lambda pot, R: pot.mass_enclosed(R))
