"""Seeded synthetic workloads with the shapes and distributions of the benchmark
configurations (galactic units: kpc, Myr, Msun; velocities in kpc/Myr).

* ``hernquist_1k``  -- Hernquist(m=1e11, c=1), 1,024 orbits with r ~ U[5, 20],
  isotropic positions, tangential circular velocity times (1 + N(0, 0.1)) per
  component; Leapfrog, dt = 1 Myr, 1,000 steps, every snapshot kept.
* ``mw_composite``  -- nucleus Hernquist(1.7e9, 0.07) + bulge Hernquist(5e9, 1)
  + Miyamoto-Nagai disk (6.8e10, 3, 0.28) + spherical NFW halo (5.4e11, 15.6),
  in that order; orbits with R ~ U[2, 30], phi ~ U[0, 2 pi), |z| < 2,
  v = v_c(R) phi_hat + isotropic N(0, 30 km/s).
"""
from __future__ import annotations

import numpy as np

from .potential import CCompositePotential, HernquistPotential, MiyamotoNagaiPotential, NFWPotential
from .units import G, KMS_TO_KPC_MYR

SEED_BASE = 1000


def hernquist_potential():
    return HernquistPotential(m=1e11, c=1.0)


def hernquist_ics(n=1024, seed=SEED_BASE + 1, m=1e11, c=1.0):
    """Isotropic positions with r ~ U[5, 20] kpc; velocity = v_c(r) times a random
    unit vector perpendicular to r, each component scaled by (1 + N(0, 0.1))."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(5.0, 20.0, n)
    u = rng.normal(size=(3, n))
    rhat = u / np.linalg.norm(u, axis=0)
    a = rng.normal(size=(3, n))
    a -= np.sum(a * rhat, axis=0) * rhat
    that = a / np.linalg.norm(a, axis=0)
    vc = np.sqrt(G * m * r / (r + c) ** 2)
    v = vc * that * (1.0 + rng.normal(0.0, 0.1, size=(3, n)))
    return np.ascontiguousarray(np.vstack([r * rhat, v]))


def mw_composite():
    pot = CCompositePotential()
    pot["nucleus"] = HernquistPotential(m=1.7e9, c=0.07)
    pot["bulge"] = HernquistPotential(m=5e9, c=1.0)
    pot["disk"] = MiyamotoNagaiPotential(m=6.8e10, a=3.0, b=0.28)
    pot["halo"] = NFWPotential(m=5.4e11, r_s=15.6)
    return pot


def _mw_vcirc_numpy(R):
    """Circular speed of the mw_composite in the midplane, closed form (numpy)."""
    Gm = lambda m: G * m  # noqa: E731
    # d Phi / dR at (R, 0, 0)
    dh1 = Gm(1.7e9) / (R + 0.07) ** 2
    dh2 = Gm(5e9) / (R + 1.0) ** 2
    dmn = Gm(6.8e10) * R * (R ** 2 + (3.0 + 0.28) ** 2) ** -1.5
    u = R / 15.6
    dnfw = Gm(5.4e11) / 15.6 / u ** 3 / 15.6 ** 2 * (np.log(1 + u) - u / (1 + u)) * R
    return np.sqrt(R * (dh1 + dh2 + dmn + dnfw))


def mw_ics(n=100_000, seed=SEED_BASE + 2, sigma_kms=30.0):
    rng = np.random.default_rng(seed)
    R = rng.uniform(2.0, 30.0, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    z = rng.uniform(-2.0, 2.0, n)
    vc = _mw_vcirc_numpy(R)
    sig = sigma_kms * KMS_TO_KPC_MYR
    vx = -vc * np.sin(phi) + rng.normal(0, sig, n)
    vy = vc * np.cos(phi) + rng.normal(0, sig, n)
    vz = rng.normal(0, sig, n)
    return np.ascontiguousarray(np.vstack([R * np.cos(phi), R * np.sin(phi), z, vx, vy, vz]))


def uneven_steps(n=262_144, seed=SEED_BASE + 3):
    """Per-orbit n_steps log-uniform in [100, 20000], dt from {0.1, 0.5, 1.0} Myr,
    integrator 0 (Leapfrog) for the first half and 1 (Ruth4) for the second,
    then shuffled."""
    rng = np.random.default_rng(seed)
    nsteps = np.round(np.exp(rng.uniform(np.log(100), np.log(20000), n))).astype(np.int64)
    dt = rng.choice(np.array([0.1, 0.5, 1.0]), n)
    method = (np.arange(n) >= n // 2).astype(np.int32)
    rng.shuffle(method)
    return nsteps, dt, method


def scf_coefficients(nmax=12, lmax=8, seed=SEED_BASE + 4):
    """S, T ~ N(0, 1) exp(-0.5 n) (l + 1)^-2, S000 = 1, zero for m > l, T_nl0 = 0."""
    rng = np.random.default_rng(seed)
    n = np.arange(nmax + 1)[:, None, None]
    l = np.arange(lmax + 1)[None, :, None]
    m = np.arange(lmax + 1)[None, None, :]
    amp = np.exp(-0.5 * n) * (l + 1.0) ** -2
    S = rng.normal(size=(nmax + 1, lmax + 1, lmax + 1)) * amp
    T = rng.normal(size=(nmax + 1, lmax + 1, lmax + 1)) * amp
    mask = m <= l
    S = np.where(mask, S, 0.0)
    T = np.where(mask, T, 0.0)
    T[:, :, 0] = 0.0
    S[0, 0, 0] = 1.0
    return S, T


def scf_potential(nmax=12, lmax=8, seed=SEED_BASE + 4):
    """SCF halo: m = 1e12 Msun, r_s = 20 kpc, coefficients from scf_coefficients."""
    from .potential import SCFPotential

    S, T = scf_coefficients(nmax, lmax, seed)
    return SCFPotential(m=1e12, r_s=20.0, Snlm=S, Tnlm=T)


def scf_ics(n=262_144, seed=SEED_BASE + 5, m=1e12, r_s=20.0):
    """Orbits in the SCF halo: r ~ U[5, 100] kpc isotropic, velocity = the
    Hernquist (m, r_s) circular speed in a random tangential direction times
    (1 + N(0, 0.1)) per component."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(5.0, 100.0, n)
    u = rng.normal(size=(3, n))
    rhat = u / np.linalg.norm(u, axis=0)
    a = rng.normal(size=(3, n))
    a -= np.sum(a * rhat, axis=0) * rhat
    that = a / np.linalg.norm(a, axis=0)
    vc = np.sqrt(G * m * r / (r + r_s) ** 2)
    v = vc * that * (1.0 + rng.normal(0.0, 0.1, size=(3, n)))
    return np.ascontiguousarray(np.vstack([r * rhat, v]))


def stream_progenitors(n=512, seed=SEED_BASE + 6):
    """Mock-stream progenitors: phase-space positions drawn as mw_ics, Plummer
    masses m ~ U[1e4, 1e6] Msun and scale radii b ~ U[5, 20] pc.
    Returns (w0 (6, n), m (n,), b (n,) in kpc)."""
    rng = np.random.default_rng(seed)
    w0 = mw_ics(n, seed=seed + 100)
    m = rng.uniform(1e4, 1e6, n)
    b = rng.uniform(5e-3, 20e-3, n)
    return w0, m, b


def stream_progenitor_potentials(m, b):
    from .potential import PlummerPotential

    return [PlummerPotential(m=float(mi), b=float(bi)) for mi, bi in zip(m, b)]
