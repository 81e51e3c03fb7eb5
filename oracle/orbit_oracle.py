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
