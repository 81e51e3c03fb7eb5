"""PhaseSpacePosition and Orbit containers (gala.dynamics equivalents).

Arrays are plain float64 in galactic units.  An Orbit may hold its phase-space
array on the GPU (a torch tensor) and converts to numpy on first host access.
"""
from __future__ import annotations

import numpy as np

from ._trace import traced

__all__ = ["PhaseSpacePosition", "Orbit"]


def _to_numpy(a):
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def _galactic(x, unit):
    """x as float64 in the given galactic unit: quantities (anything with
    ``to_value``) are converted, plain arrays are taken as galactic."""
    if hasattr(x, "to_value"):
        return np.asarray(x.to_value(unit), dtype=np.float64)
    return np.asarray(x, dtype=np.float64)


def phase_space_array(w):
    """(6, ...) float64 array of a phase-space position: this library's
    PhaseSpacePosition, any object with ``xyz`` / ``v_xyz`` (gala's
    PhaseSpacePosition, converted to kpc and kpc/Myr), or an array."""
    if isinstance(w, PhaseSpacePosition):
        return w.w()
    if hasattr(w, "xyz") and hasattr(w, "v_xyz"):
        return np.concatenate([_galactic(w.xyz, "kpc"), _galactic(w.v_xyz, "kpc / Myr")], axis=0)
    return w


# -- HDF5 serialisation helpers (gala's layout: src/gala/io.py:4-47,
#    src/gala/dynamics/core.py:572-640) ----------------------------------------
_FRAME_MODULE = "gala.potential.frame.builtin.frames"
_FRAME_UNITS = [b"kpc", b"Myr", b"solMass", b"rad", b"km / s"]


def _h5_open(f, mode):
    """(file or group, opened here): a file name is opened with this library's
    HDF5 module; an open h5py or gala_gb300.hdf5 file or group is used as is."""
    import os

    if isinstance(f, (str, os.PathLike)):
        from .hdf5 import File

        return File(f, mode), True
    return f, False


def _attr_text(v):
    if isinstance(v, bytes):
        return v.decode("utf-8")
    if isinstance(v, np.ndarray) and v.ndim == 0:
        return _attr_text(v[()])
    return None if v is None else str(v)


def quantity_to_hdf5(f, key, value, unit):
    """A dataset with a 'unit' attribute (quantity_to_hdf5, src/gala/io.py:28-47)."""
    f[key] = np.asarray(value)
    f[key].attrs["unit"] = unit


def quantity_from_hdf5(dset, physical_type=None):
    """The dataset's values in galactic units (quantity_from_hdf5, src/gala/io.py:4-25):
    values stored with another unit of the same physical type are converted."""
    from .potential_io import _unit_factor

    values = np.asarray(dset[()], dtype=np.float64)
    unit = _attr_text(dset.attrs["unit"]) if "unit" in dset.attrs else None
    if unit:
        factor = _unit_factor(unit, physical_type)
        if factor != 1.0:
            values = values * factor
    return values


def _frame_to_hdf5(f, frame):
    from .hamiltonian import ConstantRotatingFrame

    g = f.create_group("frame")
    g.attrs["module"] = _FRAME_MODULE
    g.attrs["class"] = frame.__class__.__name__
    g.create_dataset("units", data=list(_FRAME_UNITS))
    pars = g.create_group("parameters")
    if isinstance(frame, ConstantRotatingFrame):
        quantity_to_hdf5(pars, "Omega", frame.Omega, "1 / Myr")


def _frame_from_hdf5(f):
    from .hamiltonian import ConstantRotatingFrame, StaticFrame

    if "frame" not in f:
        return None
    g = f["frame"]
    cls = _attr_text(g.attrs["class"])
    if cls == "StaticFrame":
        return StaticFrame()
    if cls == "ConstantRotatingFrame":
        return ConstantRotatingFrame(Omega=quantity_from_hdf5(g["parameters/Omega"], "frequency"))
    raise ValueError(f"frame class {cls!r} is not available in gala_gb300")


# -- guiding radius and periods (src/gala/dynamics/orbit.py:555-599, 683-727) --
_D_DR_STEP = 1e-4  # c_d_dr's fixed step (cpotential.cpp:327)


def _d_dr_midplane(energy, R, t):
    """dPhi/dr at (R, 0, 0) as c_d_dr forms it (cpotential.cpp:317-343): the
    central difference (Phi(R + h) - Phi(R - h)) / (2 h), h = 1e-4; every R in
    one call of energy(q (3, 2n), t)."""
    R = np.asarray(R, dtype=np.float64)
    n = R.size
    q = np.zeros((3, 2 * n))
    q[0, :n] = R + _D_DR_STEP
    q[0, n:] = R - _D_DR_STEP
    phi = np.asarray(energy(q, t), dtype=np.float64)
    return (phi[:n] - phi[n:]) / (2.0 * _D_DR_STEP)


def _guiding_radius_solve(R0, Lz, dphi_dr, max_expand=60, max_iter=200):
    """Root R > 0 of |Lz| - R sqrt(R |dPhi/dR(R)|) for every orbit at once
    (the function of _guiding_radius_rootfunc, src/gala/dynamics/core.py:943-948).

    The root is bracketed by doubling / halving from R0, then found by the
    Illinois form of regula falsi until the bracket stops shrinking; each step
    evaluates dphi_dr (one call for all orbits).  |Lz| = 0 gives R = 0; an orbit
    whose root cannot be bracketed gives nan, as gala's failed roots do."""
    R0 = np.atleast_1d(np.asarray(R0, dtype=np.float64))
    L = np.abs(np.atleast_1d(np.asarray(Lz, dtype=np.float64)))
    out = np.full(R0.shape, np.nan)
    live = np.isfinite(R0) & (R0 > 0) & np.isfinite(L)
    zero = live & (L == 0)
    out[zero] = 0.0
    live &= ~zero

    def f(R):
        Rs = np.where(live, R, 1.0)  # placeholders keep the batched call finite
        return L - Rs * np.sqrt(Rs * np.abs(dphi_dr(Rs)))

    fr = f(R0)
    out[live & (fr == 0)] = R0[live & (fr == 0)]
    live &= fr != 0
    a, fa = R0.copy(), fr.copy()   # side with f > 0 (R too small)
    b, fb = R0.copy(), fr.copy()   # side with f < 0 (R too large)
    need_hi = live & (fr > 0)
    need_lo = live & (fr < 0)
    for _ in range(max_expand):
        if not (need_hi.any() or need_lo.any()):
            break
        trial = np.where(need_hi, b * 2.0, np.where(need_lo, a * 0.5, b))
        ft = f(trial)
        hi_done = need_hi & (ft <= 0)
        b = np.where(need_hi, trial, b)
        fb = np.where(need_hi, ft, fb)
        a = np.where(need_hi & ~hi_done, trial, a)
        fa = np.where(need_hi & ~hi_done, ft, fa)
        lo_done = need_lo & (ft >= 0)
        a = np.where(need_lo, trial, a)
        fa = np.where(need_lo, ft, fa)
        b = np.where(need_lo & ~lo_done, trial, b)
        fb = np.where(need_lo & ~lo_done, ft, fb)
        need_hi &= ~hi_done
        need_lo &= ~lo_done
    live &= ~(need_hi | need_lo)       # never bracketed: nan
    exact = live & ((fa == 0) | (fb == 0))
    out[exact] = np.where(fa[exact] == 0, a[exact], b[exact])
    live &= ~exact
    side = np.zeros(R0.shape, dtype=np.int8)  # Illinois: which end was kept last
    for _ in range(max_iter):
        if not live.any():
            break
        with np.errstate(divide="ignore", invalid="ignore"):
            x = b - fb * (b - a) / (fb - fa)
        x = np.where(live & (x > np.minimum(a, b)) & (x < np.maximum(a, b)), x, 0.5 * (a + b))
        fx = f(x)
        done = live & ((fx == 0) | (np.abs(b - a) <= 4.0 * np.finfo(float).eps * np.abs(x)))
        out[done] = x[done]
        live &= ~done
        pos = live & (fx > 0)
        neg = live & (fx < 0)
        a = np.where(pos, x, a)
        b = np.where(neg, x, b)
        fb = np.where(pos & (side == 1), 0.5 * fb, fb)
        fa = np.where(neg & (side == -1), 0.5 * fa, fa)
        fa = np.where(pos, fx, fa)
        fb = np.where(neg, fx, fb)
        side = np.where(pos, 1, np.where(neg, -1, side)).astype(np.int8)
    out[live] = 0.5 * (a[live] + b[live])
    return out


def peak_to_peak_period(t, f, amplitude_threshold=1e-2):
    """Period of a time series from its interior peaks and troughs
    (peak_to_peak_period, src/gala/dynamics/util.py:14-69): the mean spacing
    of the strict local maxima and of the strict local minima (the two ends
    excluded), averaged; nan when the mean peak minus the mean trough is
    below amplitude_threshold."""
    t = np.asarray(t, dtype=np.float64)
    f = np.asarray(f, dtype=np.float64)
    mid = f[1:-1]
    peaks = np.nonzero((mid > f[:-2]) & (mid > f[2:]))[0] + 1
    troughs = np.nonzero((mid < f[:-2]) & (mid < f[2:]))[0] + 1
    # gala's result is nan whenever either set has fewer than two members
    if len(peaks) < 2 or len(troughs) < 2:
        return np.nan
    if abs(np.mean(f[peaks]) - np.mean(f[troughs])) < amplitude_threshold:
        return np.nan
    return np.mean([np.mean(np.diff(t[peaks])), np.mean(np.diff(t[troughs]))])


def _frame_times(t, w):
    """Times for a frame rotation of the rows w (..., 6): an orbit's time axis
    is the first axis after the components (ntimes[, norbits])."""
    if t is None:
        raise ValueError("Time array must be provided if not passing an Orbit subclass.")
    t = np.asarray(t, dtype=np.float64)
    if t.ndim == 1 and w.ndim == 3 and t.shape[0] == w.shape[0]:
        return t[:, None]  # (ntimes, norbits)
    return t


class PhaseSpacePosition:
    """Positions and velocities with gala's axis convention: (ndim, ...)."""

    def __init__(self, pos, vel, frame=None, copy=True):
        pos = np.array(pos, dtype=np.float64, copy=copy)
        vel = np.array(vel, dtype=np.float64, copy=copy)
        if pos.shape != vel.shape:
            raise ValueError(f"pos and vel must have the same shape, got {pos.shape} and {vel.shape}")
        self.pos = pos
        self.vel = vel
        self.frame = frame

    @property
    def ndim(self):
        return self.pos.shape[0]

    @property
    def shape(self):
        return self.pos.shape[1:]

    @property
    def xyz(self):
        return self.pos

    # gala's component attributes
    x = property(lambda self: self.pos[0])
    y = property(lambda self: self.pos[1])
    z = property(lambda self: self.pos[2])
    v_x = property(lambda self: self.vel[0])
    v_y = property(lambda self: self.vel[1])
    v_z = property(lambda self: self.vel[2])

    @property
    def v_xyz(self):
        return self.vel

    def w(self, units=None):
        """(2 ndim, ...) array of positions then velocities (dynamics/core.py:476-525)."""
        return np.vstack((self.pos, self.vel)) if self.pos.ndim > 1 else np.concatenate((self.pos, self.vel))

    @classmethod
    def from_w(cls, w, units=None, copy=True, **kwargs):
        """From a (2 ndim, ...) array (dynamics/core.py:528-567)."""
        w = np.asarray(w)
        ndim = w.shape[0] // 2
        return cls(pos=w[:ndim], vel=w[ndim:], copy=copy, **kwargs)

    def kinetic_energy(self):
        return 0.5 * np.sum(self.vel ** 2, axis=0)

    def to_frame(self, frame, current_frame=None, t=None):
        """The same points in another frame (PhaseSpacePosition.to_frame,
        src/gala/dynamics/core.py:384-428): static <-> ConstantRotatingFrame by
        gala's rotation (transformations.py:96-191; `t` is required unless
        this is an Orbit, whose times are used), static <-> static is the
        identity.  Other pairs raise ValueError as in gala."""
        from .hamiltonian import ConstantRotatingFrame, StaticFrame, rotate_frame

        cur = self.frame if current_frame is None else current_frame
        if cur is None:
            raise ValueError(f"If no frame was specified when this {self.__class__.__name__} was initialized, you "
                             "must pass the current frame in via the current_frame argument to transform to a new "
                             "frame.")
        if t is None:
            t = getattr(self, "t", None)
        w = np.moveaxis(self.w(), 0, -1)  # (..., 6)
        if isinstance(cur, StaticFrame) and isinstance(frame, StaticFrame):
            out = w
        elif isinstance(cur, StaticFrame) and isinstance(frame, ConstantRotatingFrame):
            out = rotate_frame(w, _frame_times(t, w), frame.Omega, to_rotating=True)
        elif isinstance(cur, ConstantRotatingFrame) and isinstance(frame, StaticFrame):
            out = rotate_frame(w, _frame_times(t, w), cur.Omega, to_rotating=False)
        else:
            raise ValueError(f"Unsupported frame transformation: {cur} to {frame}")
        out = np.moveaxis(out, -1, 0)
        if isinstance(self, Orbit):
            return Orbit(pos=out[:3], vel=out[3:], t=self.t, frame=frame)
        return PhaseSpacePosition(pos=out[:3], vel=out[3:], frame=frame)

    def angular_momentum(self):
        """L = x cross v, shape (3, ...) (PhaseSpacePosition.angular_momentum,
        src/gala/dynamics/core.py)."""
        return np.cross(self.pos, self.vel, axis=0)

    def potential_energy(self, potential):
        return potential.energy(self.pos)

    def energy(self, hamiltonian):
        from .hamiltonian import Hamiltonian

        H = hamiltonian if isinstance(hamiltonian, Hamiltonian) else Hamiltonian(hamiltonian)
        return H.energy(self.w())

    # -- HDF5 (PhaseSpacePosition.to_hdf5 / from_hdf5, dynamics/core.py:572-640)
    def _write_hdf5(self, f):
        if self.frame is not None:
            _frame_to_hdf5(f, self.frame)
        quantity_to_hdf5(f, "pos", self.pos, "kpc")
        quantity_to_hdf5(f, "vel", self.vel, "kpc / Myr")

    def to_hdf5(self, f):
        """Write to an HDF5 file name (created, or overwritten) or an open file or
        group, in gala's layout: ``pos`` and ``vel`` datasets with a ``unit``
        attribute and a ``frame`` group.  Returns the file or group."""
        f, close = _h5_open(f, "w")
        self._write_hdf5(f)
        if close:
            f.close()
        return f

    @classmethod
    def from_hdf5(cls, f):
        """Read what ``to_hdf5`` (or gala's) wrote; values in galactic units."""
        f, close = _h5_open(f, "r")
        try:
            return cls(pos=quantity_from_hdf5(f["pos"], "length"), vel=quantity_from_hdf5(f["vel"], "speed"),
                       frame=_frame_from_hdf5(f))
        finally:
            if close:
                f.close()


class Orbit(PhaseSpacePosition):
    """An integrated orbit: w has shape (6, ntimes[, norbits])."""

    def __init__(self, pos=None, vel=None, t=None, hamiltonian=None, potential=None, frame=None, copy=True,
                 w_device=None):
        self._w_dev = w_device
        self._w_host = None
        if w_device is None:
            super().__init__(pos, vel, frame=frame, copy=copy)
            if self.pos.ndim < 1:
                self.pos = self.pos.reshape(1)
                self.vel = self.vel.reshape(1)
        self.t = None if t is None else np.atleast_1d(np.asarray(t, dtype=np.float64))
        if hamiltonian is not None:
            self.potential = hamiltonian.potential
            self.frame = hamiltonian.frame
            self.hamiltonian = hamiltonian
        else:
            self.potential = potential
            self.frame = frame
            self.hamiltonian = None
        if self.t is not None and w_device is None and self.pos.shape[1] != len(self.t):
            raise ValueError(
                "Position and velocity must have the same length along axis=1 as the length of the "
                f"time array {len(self.t)} vs {self.pos.shape[1]}")

    # Lazy host materialisation of a device-resident result.
    def _host(self):
        if self._w_dev is not None and self._w_host is None:
            w = _to_numpy(self._w_dev)
            self._w_host = w
            self.pos = w[:3]
            self.vel = w[3:]
        return self

    def __getattr__(self, name):
        if name in ("pos", "vel"):
            if self.__dict__.get("_w_dev") is not None:
                self._host()
                return self.__dict__[name]
        raise AttributeError(name)

    @property
    def w_device(self):
        """The (6, ntimes[, norbits]) result as a CUDA tensor, if it was kept on the GPU."""
        return self._w_dev

    @classmethod
    def from_w(cls, w, units=None, t=None, hamiltonian=None, copy=True, **kwargs):
        if hasattr(w, "is_cuda") and w.is_cuda:
            return cls(t=t, hamiltonian=hamiltonian, w_device=w, **kwargs)
        w = np.asarray(w)
        ndim = w.shape[0] // 2
        return cls(pos=w[:ndim], vel=w[ndim:], t=t, hamiltonian=hamiltonian, copy=copy, **kwargs)

    @property
    def ntimes(self):
        if self.__dict__.get("_w_dev") is not None and self.__dict__.get("_w_host") is None:
            return int(self._w_dev.shape[1])
        return self.pos.shape[1]

    @property
    def norbits(self):
        if self.__dict__.get("_w_dev") is not None and self.__dict__.get("_w_host") is None:
            return 1 if self._w_dev.ndim < 3 else int(self._w_dev.shape[2])
        return 1 if self.pos.ndim < 3 else self.pos.shape[2]

    def energy(self, hamiltonian=None):
        """Energy along the orbit (Orbit.energy, src/gala/dynamics/orbit.py:361-389)."""
        H = hamiltonian if hamiltonian is not None else self.hamiltonian
        if H is None:
            raise ValueError("To compute the total energy, a hamiltonian object must be provided!")
        from .hamiltonian import Hamiltonian

        if not isinstance(H, Hamiltonian):
            H = Hamiltonian(H)
        return H.energy(self.w())

    def guiding_radius(self, potential=None, t=0.0, **root_kwargs):
        """Guiding-center radius R_g of each orbit: R_g v_c(R_g) = |<L_z>| with
        v_c from dPhi/dR in the midplane (Orbit.guiding_radius, orbit.py:555-599).

        The potential is evaluated on the GPU, all orbits in each call.  Each orbit
        starts from its own time-averaged cylindrical radius (gala averages over
        all orbits, so only single orbits work there) and the root is solved to
        full precision (``root_kwargs``, gala's options for scipy's root, are
        accepted and not needed).  Orbits whose L_z varies by more than 1e-8
        relative get gala's RuntimeWarning about axisymmetry.
        """
        import warnings

        if potential is None:
            potential = self.potential
        if potential is None:
            raise ValueError("You must specify a potential if it is not already defined on the orbit")
        x, y = self.pos[0], self.pos[1]
        R0 = np.atleast_1d(np.mean(np.hypot(x, y), axis=0))
        Lzs = self.angular_momentum()[2]
        mean_Lz = np.atleast_1d(np.mean(Lzs, axis=0))
        with np.errstate(divide="ignore", invalid="ignore"):
            check = np.abs(np.atleast_1d(np.std(Lzs, axis=0)) / mean_Lz) > 1e-8
        if np.any(check):
            warnings.warn(
                f"{check.sum()} orbits do not have constant Lz (see orbits at indices: "
                f"{list(np.where(check)[0][:10])}, ...). Are you sure you are using an axisymmetric potential?",
                RuntimeWarning)
        Rg = _guiding_radius_solve(R0, mean_Lz, lambda R: _d_dr_midplane(potential.energy, R, t))
        return Rg.reshape(self.pos.shape[2:]) if self.pos.ndim > 2 else Rg[0]

    def estimate_period(self):
        """Period of each Cartesian coordinate of each orbit from its peaks and
        troughs (Orbit.estimate_period, orbit.py:683-727): a dict of arrays of
        shape (norbits,) keyed 'x', 'y', 'z' (gala returns a table with these
        columns)."""
        if self.t is None:
            raise ValueError("To compute the period, a time array is needed. Specify a time array when creating "
                             "this object.")
        periods = {}
        for k, name in enumerate("xyz"):
            q = self.pos[k]
            if q.ndim == 1:
                periods[name] = np.atleast_1d(peak_to_peak_period(self.t, q))
            else:
                periods[name] = np.array([peak_to_peak_period(self.t, q[:, n]) for n in range(q.shape[1])])
        return periods

    # -- HDF5 (Orbit.to_hdf5 / from_hdf5, src/gala/dynamics/orbit.py:236-323) --
    def _write_hdf5(self, f):
        super()._write_hdf5(f)
        if self.potential is not None:
            from .potential_io import to_dict, yaml_dump

            f["potential"] = yaml_dump(to_dict(self.potential)).encode("utf-8")
        if self.t is not None:
            quantity_to_hdf5(f, "time", self.t, "Myr")

    @classmethod
    def from_hdf5(cls, f):
        """Read an orbit written by ``to_hdf5`` or by gala.  The potential is
        rebuilt from its YAML when its classes exist here; otherwise a
        warning is issued and the orbit has no potential."""
        import warnings

        from .potential_io import from_dict, yaml_load

        f, close = _h5_open(f, "r")
        try:
            pos = quantity_from_hdf5(f["pos"], "length")
            vel = quantity_from_hdf5(f["vel"], "speed")
            t = quantity_from_hdf5(f["time"], "time") if "time" in f else None
            frame = _frame_from_hdf5(f)
            potential = None
            if "potential" in f:
                text = f["potential"][()]
                text = text.decode("utf-8") if isinstance(text, bytes) else str(text)
                try:
                    potential = from_dict(yaml_load(text))
                except (ValueError, KeyError, TypeError, NotImplementedError) as e:
                    warnings.warn(f"the orbit's potential could not be rebuilt: {e}", RuntimeWarning)
        finally:
            if close:
                f.close()
        return cls(pos=pos, vel=vel, t=t, frame=frame, potential=potential)

    def __getitem__(self, idx):
        w = self.w()
        if not isinstance(idx, tuple):
            idx = (idx,)
        wi = w[(slice(None),) + idx]
        t = self.t[idx[0]] if self.t is not None else None
        if wi.ndim >= 2 and t is not None and np.ndim(t) > 0:
            return Orbit.from_w(wi, t=t, hamiltonian=self.hamiltonian)
        return PhaseSpacePosition.from_w(wi)

    # -- extrema (src/gala/dynamics/orbit.py:391-681), computed on the GPU ------
    _KINDS = {"peri": 0, "apo": 1, "zmax": 2}

    def _device_w_t(self):
        import torch

        from ._device import as_device_f64, require_cuda

        dev = require_cuda()
        if self.t is None:
            raise ValueError("extrema need the orbit's time array")
        w = self._w_dev if self._w_dev is not None else self.w()
        wd = as_device_f64(w, dev)
        if wd.ndim == 2:
            wd = wd[:, :, None]
        return wd.contiguous(), torch.from_numpy(np.ascontiguousarray(self.t, dtype=np.float64)).to(dev)

    @traced("orbit_extrema")
    def _extrema_run(self, approximate, keep):
        import torch

        from . import _abi
        from ._device import ptr, stream_handle

        wd, td = self._device_w_t()
        nt, n = int(wd.shape[1]), int(wd.shape[2])
        dev = wd.device
        count = torch.zeros((3, n), dtype=torch.int32, device=dev)
        sm, mn, mx = (torch.zeros((3, n), dtype=torch.float64, device=dev) for _ in range(3))
        vals = torch.zeros((3, n, keep), dtype=torch.float64, device=dev) if keep else None
        times = torch.zeros((3, n, keep), dtype=torch.float64, device=dev) if keep else None
        _abi.call("gx_orbit_extrema", ptr(wd), ptr(td), nt, n, int(bool(approximate)), int(keep), ptr(count),
                  ptr(sm), ptr(mn), ptr(mx), ptr(vals) if keep else None, ptr(times) if keep else None,
                  stream_handle())
        out = {"count": count.cpu().numpy(), "sum": sm.cpu().numpy(), "min": mn.cpu().numpy(),
               "max": mx.cpu().numpy()}
        if keep:
            out["vals"] = vals.cpu().numpy()
            out["times"] = times.cpu().numpy()
        return out

    def _extrema(self, kind, return_times, func, approximate):
        if return_times and func is not None:
            raise ValueError("Cannot return times if reducing using an input function. Pass `func=None` if you "
                             "want to return all individual values and times.")
        k = self._KINDS[kind]
        cache = self.__dict__.setdefault("_ext_cache", {})
        if approximate not in cache:
            cache[approximate] = self._extrema_run(approximate, 0)
        st = cache[approximate]
        cnt = st["count"][k]
        single = self.norbits == 1
        if func is np.mean or func is np.min or func is np.max:
            with np.errstate(invalid="ignore", divide="ignore"):
                v = {np.mean: st["sum"][k] / cnt, np.min: st["min"][k], np.max: st["max"][k]}[func]
            v = np.where(cnt > 0, v, np.nan)
            return float(v[0]) if single else v
        keep = max(int(cnt.max()), 1)
        full = self._extrema_run(approximate, keep)
        vals = [full["vals"][k, i, :cnt[i]] for i in range(len(cnt))]
        tms = [full["times"][k, i, :cnt[i]] for i in range(len(cnt))]
        if func is not None:
            v = np.array([func(x) for x in vals])
            return float(v[0]) if single else v
        if return_times:
            return (vals[0], tms[0]) if single else (vals, tms)
        return vals[0] if single else vals

    def pericenter(self, return_times=False, func=np.mean, approximate=False):
        """Pericentres from the local minima of r, each refined by a parabola
        (Orbit.pericenter, orbit.py:439-495)."""
        return self._extrema("peri", return_times, func, approximate)

    def apocenter(self, return_times=False, func=np.mean, approximate=False):
        """Apocentres from the local maxima of r (Orbit.apocenter, orbit.py:497-553)."""
        return self._extrema("apo", return_times, func, approximate)

    def zmax(self, return_times=False, func=np.mean, approximate=False):
        """Maximum |z| excursions (Orbit.zmax, orbit.py:600-656)."""
        return self._extrema("zmax", return_times, func, approximate)

    def eccentricity(self, **kw):
        """(r_apo - r_peri) / (r_apo + r_peri) from the mean apo- and pericentre
        (Orbit.eccentricity, orbit.py:658-681)."""
        ra = self.apocenter(**kw)
        rp = self.pericenter(**kw)
        return (ra - rp) / (ra + rp)

