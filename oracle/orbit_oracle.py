"""ORACLE (test infrastructure only): gala's orbit extremum estimates restated
with numpy / scipy, used to check the GPU reduction kernel.

Follows src/gala/dynamics/orbit.py: ``_max_helper`` (:391-426) -- interior
strict local maxima from ``scipy.signal.argrelmax(arr, mode="wrap")`` with the
two ends removed, each refined by ``np.polynomial.polynomial.polyfit`` of
degree 2 through the three samples around it, vertex at -c1 / (2 c2) -- and
``pericenter`` (:439-495, maxima of -r), ``apocenter`` (:497-553, maxima of r),
``zmax`` (:600-656, maxima of |z|), ``eccentricity`` (:658-681).  A time grid
running backwards is reversed first, as gala does.  The spherical radius is
astropy's (hypot(hypot(x, y), z), PhysicsSphericalRepresentation.from_cartesian),
the cylindrical z is z.

Also restated: the static <-> constant-rotating frame transformations
(src/gala/potential/frame/builtin/transformations.py:10-56, 96-191) used by the
mock-stream DFs in a rotating frame (df.pyx:172-233); ``guiding_radius`` (orbit.py:555-599 with core.py:943-967 and
c_d_dr, cpotential.cpp:317-343) through scipy.optimize.root as gala calls it,
and ``peak_to_peak_period`` (src/gala/dynamics/util.py:14-69) with argrelmax /
argrelmin, behind ``Orbit.estimate_period`` (orbit.py:683-727).
"""
from __future__ import annotations

import numpy as np
from scipy.signal import argrelmax


def max_helper(arr, t, approximate=False):
    """Values and times of the interior local maxima of arr(t) (orbit.py:391-426)."""
    arr = np.asarray(arr, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    ix = argrelmax(arr, mode="wrap")[0]
    ix = ix[(ix != 0) & (ix != (len(arr) - 1))]
    if approximate:
        return arr[ix], t[ix]
    better_times = np.zeros(ix.shape, dtype=float)
    better_arr = np.zeros(ix.shape, dtype=float)
    for i, j in enumerate(ix):
        tvals = t[j - 1:j + 2]
        rvals = arr[j - 1:j + 2]
        coeffs = np.polynomial.polynomial.polyfit(tvals, rvals, 2)
        better_times[i] = (-coeffs[1]) / (2 * coeffs[2])
        better_arr[i] = (coeffs[2] * better_times[i] ** 2) + (coeffs[1] * better_times[i]) + coeffs[0]
    return better_arr, better_times


def _orbits(w, t):
    """(6, ntimes[, N]) -> list of (6, ntimes) with time increasing."""
    w = np.asarray(w, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    if w.ndim == 2:
        w = w[:, :, None]
    if t[-1] < t[0]:
        w = w[:, ::-1]
        t = t[::-1]
    return [w[:, :, n] for n in range(w.shape[2])], t


def extrema(w, t, kind, approximate=False):
    """Per orbit: (values, times) of pericenters ('peri'), apocenters ('apo') or
    z maxima ('zmax')."""
    orbits, t = _orbits(w, t)
    out = []
    for o in orbits:
        if kind == "peri":
            v, tt = max_helper(-np.hypot(np.hypot(o[0], o[1]), o[2]), t, approximate)
            out.append((-v, tt))
        elif kind == "apo":
            out.append(max_helper(np.hypot(np.hypot(o[0], o[1]), o[2]), t, approximate))
        elif kind == "zmax":
            out.append(max_helper(np.abs(o[2]), t, approximate))
        else:
            raise ValueError(kind)
    return out


def reduce(w, t, kind, func=np.mean, approximate=False):
    return np.array([func(v) for v, _ in extrema(w, t, kind, approximate)])


def eccentricity(w, t, approximate=False):
    ra = reduce(w, t, "apo", approximate=approximate)
    rp = reduce(w, t, "peri", approximate=approximate)
    return (ra - rp) / (ra + rp)


def d_dr(energy, R, t=0.0):
    """c_d_dr (src/gala/potential/potential/src/cpotential.cpp:317-343) at (R, 0, 0):
    (Phi(q + h q/r) - Phi(q - h q/r)) / (2 h) with h = 1e-4."""
    R = np.atleast_1d(np.asarray(R, dtype=np.float64))
    h = 1e-4
    z = np.zeros_like(R)
    plus = energy(np.stack([R + h * (R / R), z, z]), t)
    minus = energy(np.stack([R - h * (R / R), z, z]), t)
    return (plus - minus) / (2.0 * h)


def guiding_radius(w, energy, t=0.0, **root_kwargs):
    """Orbit.guiding_radius (orbit.py:555-599) with _guiding_radius_helper and
    _guiding_radius_rootfunc (src/gala/dynamics/core.py:943-967): for each orbit,
    scipy.optimize.root (method 'hybr', xtol 1e-5 by default) on
    |Lz| - R sqrt(R |dPhi/dR|) from the mean cylindrical radius, nan where root
    reports failure.  Each orbit starts from its own mean radius (gala takes the
    mean over all orbits, which only works for one orbit).  w: (6, ntimes[, N]);
    energy(q (3, n), t) -> (n,)."""
    from scipy.optimize import root

    root_kwargs.setdefault("options", {"xtol": 1e-5})
    root_kwargs.setdefault("method", "hybr")
    w = np.asarray(w, dtype=np.float64)
    w2 = w if w.ndim == 3 else w[..., None]
    out = np.zeros(w2.shape[2])
    for i in range(w2.shape[2]):
        x, y, _, vx, vy, _ = w2[:, :, i]
        R0 = np.mean(np.hypot(x, y))
        Lz = np.mean(x * vy - y * vx)

        def rootfunc(R, Lz):
            dphi = d_dr(energy, R[0], t)
            return Lz - R * np.sqrt(R * np.abs(dphi))

        res = root(rootfunc, R0, args=(np.abs(Lz),), **root_kwargs)
        out[i] = res.x[0] if res.success else np.nan
    return out if w.ndim == 3 else out[0]


def peak_to_peak_period(t, f, amplitude_threshold=1e-2):
    """peak_to_peak_period (src/gala/dynamics/util.py:14-69): mean spacing of the
    interior maxima and of the interior minima (argrelmax / argrelmin with
    mode 'wrap', ends removed), averaged; nan when the mean peak-to-trough
    amplitude is below the threshold."""
    from scipy.signal import argrelmin

    t = np.asarray(t, dtype=np.float64)
    f = np.asarray(f, dtype=np.float64)
    max_ix = argrelmax(f, mode="wrap")[0]
    max_ix = max_ix[(max_ix != 0) & (max_ix != (len(f) - 1))]
    min_ix = argrelmin(f, mode="wrap")[0]
    min_ix = min_ix[(min_ix != 0) & (min_ix != (len(f) - 1))]
    if abs(np.mean(f[max_ix]) - np.mean(f[min_ix])) < amplitude_threshold:
        return np.nan
    T_max = np.mean(t[max_ix[1:]] - t[max_ix[:-1]]) if len(max_ix) > 0 else np.nan
    T_min = np.mean(t[min_ix[1:]] - t[min_ix[:-1]]) if len(min_ix) > 0 else np.nan
    return np.mean([T_max, T_min])


def rodrigues_axis_angle_rotate(x, vec, theta):
    """Rodrigues' rotation of x (3, N) about the unit axis vec by theta (N,)
    (transformations.py:10-56, the same expression)."""
    x = np.array(x).T
    vec = np.array(vec).T
    theta = np.array(theta).T[..., None]
    out = np.cos(theta) * x + np.sin(theta) * np.cross(vec, x) + (1 - np.cos(theta)) * (vec * x).sum(axis=-1)[
        ..., None] * vec
    return out.T


def constantrotating_static(Omega, pos, vel, t, sign):
    """_constantrotating_static_helper (transformations.py:96-153) for a 3D
    Omega: sign +1 static -> rotating, -1 rotating -> static; pos, vel (3, N),
    t (N,).  Returns (pos, vel)."""
    Omega = -np.asarray(Omega, dtype=np.float64)
    vec = Omega / np.linalg.norm(Omega)
    theta = np.linalg.norm(Omega) * np.asarray(t, dtype=np.float64)
    return (rodrigues_axis_angle_rotate(pos, vec, sign * theta),
            rodrigues_axis_angle_rotate(vel, vec, sign * theta))
