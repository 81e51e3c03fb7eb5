"""Time specification and integrator names (gala.integrate equivalents)."""
from __future__ import annotations

import numpy as np

__all__ = [
    "parse_time_specification",
    "Integrator",
    "LeapfrogIntegrator",
    "Ruth4Integrator",
    "DOPRI853Integrator",
    "get_integrator",
]


def _march(t1, t2, dt):
    """t1, t1 + dt, (t1 + dt) + dt, ... -- each time the previous one plus dt, so
    the rounding is that of a running sum -- for as long as the time lies
    strictly before t2 in the direction of dt."""
    m = int(np.ceil((t2 - t1) / dt)) + 2
    while True:
        seq = np.cumsum(np.concatenate([[t1], np.full(m, dt)]))
        before = (seq < t2) if dt > 0 else (seq > t2)
        if not before[-1]:
            return seq[: int(np.argmin(before))]
        m *= 2


def parse_time_specification(units=None, dt=None, n_steps=None, t1=None, t2=None, t=None):
    """Array of times from a time specification.

    Same combinations, arithmetic and errors as gala's
    ``parse_time_specification`` (src/gala/integrate/timespec.py:10-147):
    ``t``; ``dt, n_steps[, t1]``; ``dt, t1, t2``; array ``dt, t1``;
    ``n_steps, t1, t2``.
    """
    # times given as quantities (anything with to_value) are converted to Myr,
    # as gala decomposes them in the unit system (timespec.py:74-89)
    dt, t1, t2, t = (x.to_value("Myr") if hasattr(x, "to_value") else x for x in (dt, t1, t2, t))
    if n_steps is not None:
        n_steps = int(n_steps)

    if t is not None:
        return np.asarray(t).astype(np.float64)

    if dt is None and (t1 is None or t2 is None or n_steps is None):
        raise ValueError("Invalid specification of integration time. See docstring for more information.")

    if dt is not None and n_steps is not None:
        if t1 is None:
            t1 = 0.0
        times = parse_time_specification(units, dt=np.ones(n_steps + 1) * dt, t1=t1)

    elif dt is not None and t1 is not None and t2 is not None:
        if (t2 < t1 and dt < 0) or (t2 > t1 and dt > 0):
            times = _march(float(t1), float(t2), float(dt))
            # a backward grid ends exactly on t2, a forward one stops short of it
            if dt < 0 and times[-1] != t2:
                times = np.append(times, float(t2))
            return times
        if dt == 0:
            raise ValueError("dt must be non-zero.")
        raise ValueError("If t2 < t1, dt must be negative. If t1 < t2, dt must be positive.")

    elif isinstance(dt, np.ndarray) and t1 is not None:
        times = np.cumsum(np.append([0.0], dt)) + t1
        times = times[:-1]

    elif dt is None and not (t1 is None or t2 is None or n_steps is None):
        times = np.linspace(t1, t2, n_steps, endpoint=True)

    else:
        raise ValueError("Invalid options. See docstring.")

    return times.astype(np.float64)


class Integrator:
    """Marker base class; the integration itself runs in the CUDA library."""

    name = None


class LeapfrogIntegrator(Integrator):
    name = "leapfrog"


class Ruth4Integrator(Integrator):
    name = "ruth4"


class DOPRI853Integrator(Integrator):
    name = "dopri853"


_integrator_name_mapping = {
    "leapfrog": LeapfrogIntegrator,
    "dopri853": DOPRI853Integrator,
    "dop853": DOPRI853Integrator,
    "ruth4": Ruth4Integrator,
}


def get_integrator(name):
    """Integrator class from a name or class (src/gala/integrate/lookup.py:23-84)."""
    if not isinstance(name, str):
        if name not in list(_integrator_name_mapping.values()):
            raise ValueError(
                f"Integrator class '{name}' is not recognized. Valid classes are: "
                f"{list(_integrator_name_mapping.values())}")
        return name
    key = name.lower()
    if key == "rk5":
        raise ValueError("Cython integration not supported for 'rk5': gala has no C RK5 integrator")
    if key not in _integrator_name_mapping:
        raise ValueError(
            f"Integrator '{name}' is not recognized. Valid names are: {list(_integrator_name_mapping.keys())}")
    return _integrator_name_mapping[key]
