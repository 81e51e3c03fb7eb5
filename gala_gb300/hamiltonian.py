"""Hamiltonian (potential + reference frame) and the orbit-integration entry point.

``Hamiltonian.integrate_orbit`` follows gala's dispatch
(src/gala/potential/hamiltonian/chamiltonian.pyx:224-380): default integrator,
time specification, array shapes, errors and the ``Orbit`` it returns are
gala's, while the integration itself is one call into the CUDA library
(gx_leapfrog_integrate_hamiltonian / gx_ruth4_integrate_hamiltonian /
gx_dop853_integrate_hamiltonian).
"""
from __future__ import annotations

import ctypes as C
import warnings

import numpy as np

from . import _abi
from .dynamics import Orbit, phase_space_array
from .integrate import (DOPRI853Integrator, LeapfrogIntegrator, Ruth4Integrator, get_integrator,
                        parse_time_specification)
from .potential import PotentialBase
from ._trace import traced

__all__ = ["StaticFrame", "ConstantRotatingFrame", "Hamiltonian"]


def cost_order(potential, w0d, stream_handle_):
    """Processing order for per-orbit adaptive integration: orbits by their
    dynamical frequency at the start, max(sqrt(|grad Phi| / r), |v| / r), highest
    first -- the step count of an adaptive integrator over a fixed time span
    grows with it -- so the lanes of a warp get orbits of similar cost.  (N,)
    int32 CUDA tensor."""
    import torch

    from ._device import ptr

    n = w0d.shape[1]
    q = w0d[:3].contiguous()
    g = torch.empty((3, n), dtype=torch.float64, device=w0d.device)
    _abi.call("gx_potential_gradient", potential.packed().for_device(), 0.0, ptr(q), n, ptr(g), stream_handle_)
    r = torch.linalg.vector_norm(q, dim=0).clamp_min(1e-300)
    key = torch.maximum(torch.sqrt(torch.linalg.vector_norm(g, dim=0) / r),
                        torch.linalg.vector_norm(w0d[3:], dim=0) / r)
    key = torch.nan_to_num(key, nan=0.0, posinf=1e300)
    return torch.argsort(key, descending=True, stable=True).to(torch.int32).contiguous()


class FrameBase:
    _type = None

    def __init__(self, *args, units=None):
        self.units = units

    def c_frame(self):
        f = _abi.gx_frame()
        f.type = self._type
        for k, v in enumerate(self._params()):
            f.params[k] = v
        return f

    def _params(self):
        return []


class StaticFrame(FrameBase):
    """Static inertial frame (static_frame_*, builtin_frames.cpp:8-24)."""

    _type = _abi.GX_FRAME_STATIC


class ConstantRotatingFrame(FrameBase):
    """Frame rotating at constant angular velocity Omega (rad/Myr) about the origin
    (constant_rotating_frame_3d_*, builtin_frames.cpp:73-112)."""

    _type = _abi.GX_FRAME_CONSTANT_ROTATING

    def __init__(self, Omega, units=None):
        super().__init__(units=units)
        if hasattr(Omega, "unit") and hasattr(Omega, "to_value"):
            # a quantity: to 1/Myr, angles dimensionless as gala's Omega parameter takes them
            import astropy.units as u

            Omega = Omega.to_value(1 / u.Myr, equivalencies=u.dimensionless_angles())
        self.Omega = np.asarray(Omega, dtype=np.float64).reshape(3)

    def _params(self):
        return list(self.Omega)


def rotate_frame(w, t, Omega, to_rotating):
    """Phase-space rows between a static frame and ConstantRotatingFrame(Omega),
    gala's static_to_constantrotating / constantrotating_to_static
    (src/gala/potential/frame/builtin/transformations.py:96-191): positions and
    velocities (the canonical momenta of the rotating Hamiltonian) are both
    turned about the axis -Omega/|Omega| by +|Omega| t (to the rotating frame)
    or -|Omega| t (to the static one), by Rodrigues' formula.

    w : (..., 6) numpy array or torch tensor; t : times broadcasting against
    w[..., 0].  Returns the same kind as w."""
    Omega = np.asarray(Omega, dtype=np.float64).reshape(3)
    om = float(np.linalg.norm(Omega))
    if om == 0.0:
        return w
    k = -Omega / om
    sign = 1.0 if to_rotating else -1.0
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(w, torch.Tensor):
        kt = torch.as_tensor(k, dtype=w.dtype, device=w.device)
        th = sign * om * torch.as_tensor(t, dtype=w.dtype, device=w.device)[..., None]
        c, sn = torch.cos(th), torch.sin(th)

        def rot(x):
            return c * x + sn * torch.cross(kt.expand_as(x), x, dim=-1) + (1 - c) * (x * kt).sum(-1, keepdim=True) * kt

        return torch.cat([rot(w[..., :3]), rot(w[..., 3:])], dim=-1)
    w = np.asarray(w, dtype=np.float64)
    th = sign * om * np.asarray(t, dtype=np.float64)[..., None]
    c, sn = np.cos(th), np.sin(th)

    def rot(x):
        return c * x + sn * np.cross(k, x) + (1 - c) * (x * k).sum(-1, keepdims=True) * k

    return np.concatenate([rot(w[..., :3]), rot(w[..., 3:])], axis=-1)


class Hamiltonian:
    """A potential in a reference frame (chamiltonian.pyx:40-77)."""

    def __init__(self, potential, frame=None):
        if isinstance(potential, Hamiltonian):
            frame = potential.frame
            potential = potential.potential
        if not isinstance(potential, PotentialBase):
            raise TypeError(f"potential must be a Potential object, not {type(potential)}")
        if frame is None:
            frame = StaticFrame()
        if not isinstance(frame, FrameBase):
            raise TypeError(f"frame must be a Frame object, not {type(frame)}")
        self.potential = potential
        self.frame = frame
        self.units = potential.units
        self.ndim = 6
        self.c_enabled = True

    def _frame_ref(self):
        self._cframe = self.frame.c_frame()
        return C.byref(self._cframe)

    # --- evaluation ----------------------------------------------------------
    def _prepare_w(self, w):
        w = np.asarray(phase_space_array(w), dtype=np.float64)
        if w.shape[0] != 6:
            raise ValueError(f"Invalid phase-space shape {w.shape}: expected (6, ...)")
        return w

    @traced("hamiltonian_energy")
    def energy(self, w, t=0.0):
        """Value of the Hamiltonian (chamiltonian.pyx:107-128) at w of shape (6, ...)."""
        import torch

        from ._device import as_device_f64, ptr, stream_handle

        w = self._prepare_w(w)
        shape = w.shape
        wd = as_device_f64(w.reshape(6, -1))
        n = wd.shape[1]
        out = torch.empty(n, dtype=torch.float64, device=wd.device)
        _abi.call("gx_hamiltonian_value", self.potential.packed().for_device(), self._frame_ref(), float(t),
                  ptr(wd), n, ptr(out), stream_handle())
        return out.cpu().numpy().reshape(shape[1:])

    @traced("hamiltonian_gradient")
    def gradient(self, w, t=0.0):
        """(qdot, pdot) at w (hamiltonian_gradient_T, chamiltonian.cpp:38-57); note gala's
        Hamiltonian.gradient returns dH/dw with the momentum half negated (:88-99)."""
        import torch

        from ._device import as_device_f64, ptr, stream_handle

        w = self._prepare_w(w)
        shape = w.shape
        wd = as_device_f64(w.reshape(6, -1))
        n = wd.shape[1]
        out = torch.empty((6, n), dtype=torch.float64, device=wd.device)
        _abi.call("gx_hamiltonian_gradient", self.potential.packed().for_device(), self._frame_ref(), float(t),
                  ptr(wd), n, ptr(out), stream_handle())
        return out.cpu().numpy().reshape(shape)

    def _integrate_surrogate(self, w0, kw, save_all, return_device, Integrator, **time_spec):
        """Leapfrog with a learned surrogate force (Integrator_kwargs surrogate=)."""
        import torch

        from .surrogate import SurrogatePotential

        if Integrator is not LeapfrogIntegrator:
            raise ValueError("the surrogate integrates with the LeapfrogIntegrator only")
        if not isinstance(self.frame, StaticFrame):
            raise TypeError("the surrogate integrates in a StaticFrame only")
        sp = kw["surrogate"]
        if not isinstance(sp, SurrogatePotential):
            sp = SurrogatePotential.load(sp, self.potential)
        elif sp.scf is not self.potential and not np.array_equal(sp.scf.packed().params,
                                                                 self.potential.packed().params):
            raise ValueError("the surrogate was trained for a different potential")
        stride = int(kw.get("out_stride", 1))
        if stride < 1:
            raise ValueError(f"out_stride must be >= 1 (got {stride})")
        arr = w0 if isinstance(w0, torch.Tensor) else np.asarray(w0, dtype=np.float64)
        if arr.ndim == 0 or arr.shape[0] != 6:
            raise ValueError(f"Invalid initial conditions shape {tuple(arr.shape)}. Expected shape (6, ...)")
        t = np.ascontiguousarray(parse_time_specification(self.units, **time_spec), dtype=np.float64)
        if len(t) < 2:
            raise ValueError("ntimes must be greater than 1")
        dt = float(t[1] - t[0])
        n_steps = len(t) - 1
        if isinstance(arr, torch.Tensor):
            w = arr.reshape(6, -1).to(device=sp.dev, dtype=torch.float64).contiguous()
        else:
            w = torch.from_numpy(np.ascontiguousarray(arr.reshape(6, -1))).to(sp.dev)
        if not save_all:
            w, _ = sp.integrate_leapfrog(w, dt, n_steps)
            out, t_out = w[:, None], t[-1:]
        else:
            snaps, t_out = [w], [t[0]]
            for j in range(stride, n_steps + 1, stride):
                w, _ = sp.integrate_leapfrog(w, dt, stride)
                snaps.append(w)
                t_out.append(t[j])
            out, t_out = torch.stack(snaps, dim=1), np.array(t_out)
        wr = out if return_device else out.cpu().numpy()
        if wr.shape[-1] == 1:
            wr = wr[..., 0]
        if return_device:
            return Orbit.from_w(wr, t=t_out, hamiltonian=self)
        return Orbit.from_w(w=wr, t=t_out, hamiltonian=self, copy=False)

    # --- integration ---------------------------------------------------------    # --- integration ---------------------------------------------------------
    @traced("integrate_orbit")
    def integrate_orbit(self, w0, Integrator=None, Integrator_kwargs=dict(), cython_if_possible=True,
                        save_all=True, return_device=False, stream=None, **time_spec):
        """Integrate orbits from w0 (shape (6,) or (6, N)) and return an Orbit.

        Extra keyword (not in gala): ``return_device=True`` keeps the result on
        the GPU (``Orbit.w_device``); the host copy is made on first access.
        DOP853 accepts gala's Integrator_kwargs (atol, rtol, nmax, err_if_fail,
        log_output, nbatch) plus ``dt_max`` and ``nstiff``.  Every integrator
        accepts two more Integrator_kwargs:

        * ``out_stride`` -- keep every k-th output time (t[0], t[k], ...);
        * ``precision`` -- ``"fp64"`` (default: gala's arithmetic, the parity
          form) or ``"fp32c"``: FP32 forces with compensated FP32 state (Leapfrog,
          Ruth4), or FP32 DOP853 stages with FP64 time / error norm /
          accept-reject and per-orbit step control (DOP853; ``nbatch`` does not
          apply).  Closed-form potentials only; results are not bit-compatible
          with gala (FP32 force accuracy, ~1e-7 relative per evaluation).
        * ``surrogate`` -- a trained ``SurrogatePotential`` of this (SCF)
          potential, or the path of one saved with ``SurrogatePotential.save``:
          Leapfrog in FP32 with the learned force on the tensor cores (the
          analytic force outside its trained radii).  Snapshots are taken every
          ``out_stride`` steps (the run is continued from each snapshot).
        """
        import torch

        from ._device import ptr, require_cuda, stream_handle

        if Integrator is None and isinstance(self.frame, StaticFrame):
            Integrator = LeapfrogIntegrator
        elif Integrator is None:
            Integrator = DOPRI853Integrator
        Integrator = get_integrator(Integrator)

        if Integrator in (LeapfrogIntegrator, Ruth4Integrator) and not isinstance(self.frame, StaticFrame):
            warnings.warn(
                "Using a symplectic integrator with a non-static frame can lead to wildly incorrect orbits. "
                "It is recommended that you use DOPRI853Integrator instead.", RuntimeWarning)

        # Every argument is checked before the device is touched, in gala's order:
        # initial-condition shape (chamiltonian.pyx:309-310), time specification
        # (timespec.py:91-145), then the integrator's own checks (leapfrog.pyx:61-68).
        w0 = phase_space_array(w0)
        if isinstance(w0, torch.Tensor):
            arr_w0 = w0
        else:
            arr_w0 = np.asarray(w0, dtype=np.float64)
        if arr_w0.ndim == 0 or arr_w0.shape[0] != 6:
            raise ValueError(
                f"Invalid initial conditions shape {tuple(arr_w0.shape)}. Expected shape (6, ...) but got shape "
                f"{tuple(arr_w0.shape)}.")
        t = np.ascontiguousarray(parse_time_specification(self.units, **time_spec), dtype=np.float64)
        ntimes = len(t)
        if ntimes < 2:
            raise ValueError("ntimes must be greater than 1")
        symplectic = Integrator in (LeapfrogIntegrator, Ruth4Integrator)
        if symplectic and not isinstance(self.frame, StaticFrame):
            raise TypeError(
                f"{'Leapfrog' if Integrator is LeapfrogIntegrator else 'Ruth4'} integration is currently only "
                f"supported for StaticFrame, not {self.frame.__class__.__name__}")
        kw = dict(Integrator_kwargs)
        if kw.get("surrogate") is not None:
            return self._integrate_surrogate(w0, kw, save_all, return_device, Integrator, **time_spec)
        precision = str(kw.get("precision", "fp64")).lower()
        if precision not in ("fp64", "fp32c"):
            raise ValueError(f"precision must be 'fp64' or 'fp32c' (got {precision!r})")
        stride = int(kw.get("out_stride", 1))
        if stride < 1:
            raise ValueError(f"out_stride must be >= 1 (got {stride})")
        if not symplectic:
            atol = float(kw.get("atol", 1e-10))
            rtol = float(kw.get("rtol", 1e-10))
            nmax = int(kw.get("nmax", 0))
            err_if_fail = int(kw.get("err_if_fail", 1))
            nbatch = int(kw.get("nbatch", 100))
            dt_max = float(kw.get("dt_max", 0.0))
            nstiff = int(kw.get("nstiff", 0))
            if not 1 <= nbatch <= 1024:
                raise ValueError(f"nbatch must be in [1, 1024] (got {nbatch})")

        dev = require_cuda()
        if isinstance(arr_w0, torch.Tensor):
            w0d = arr_w0.reshape(6, -1).to(device=dev, dtype=torch.float64).contiguous()
        else:
            host = torch.from_numpy(np.ascontiguousarray(arr_w0.reshape(6, -1)))
            if torch.cuda.is_available():
                host = host.pin_memory()
            w0d = host.to(dev, non_blocking=True)
        n = w0d.shape[1]

        td = torch.from_numpy(t).to(dev)
        st = stream_handle(stream)
        pot = self.potential.packed().for_device()
        frame = self._frame_ref()

        if symplectic and precision == "fp32c":
            n_out = (ntimes - 1) // stride + 1
            out = torch.empty((6, n_out, n) if save_all else (6, n), dtype=torch.float64, device=dev)
            _abi.call("gx_fixed_fp32", pot, 0 if Integrator is LeapfrogIntegrator else 1, ptr(w0d), n, ptr(td),
                      ntimes, int(bool(save_all)), stride, ptr(out), st)
            t_out = t[::stride]
        elif symplectic:
            out = torch.empty((6, ntimes, n) if save_all else (6, n), dtype=torch.float64, device=dev)
            name = ("gx_leapfrog_integrate_hamiltonian" if Integrator is LeapfrogIntegrator
                    else "gx_ruth4_integrate_hamiltonian")
            _abi.call(name, pot, frame, ptr(w0d), n, ptr(td), ntimes, int(bool(save_all)), ptr(out), st)
            t_out = t
            if save_all and stride > 1:
                out = out[:, ::stride].contiguous()
                t_out = t[::stride]
        elif precision == "fp32c":
            n_out = (ntimes - 1) // stride + 1
            out = torch.empty((6, n_out, n) if save_all else (6, n), dtype=torch.float64, device=dev)
            status = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
            counter = torch.zeros(1, dtype=torch.int32, device=dev)
            order = cost_order(self.potential, w0d, st)
            _abi.call("gx_dop853_fp32", pot, frame, ptr(w0d), n, ptr(td), ntimes, atol, rtol, nmax, dt_max, nstiff,
                      int(bool(save_all)), stride, ptr(order), ptr(out), ptr(status), None, ptr(counter), st)
            if err_if_fail == 1 and n > 0:
                res = status.cpu().numpy()
                bad = res[res < 0]
                if bad.size:
                    raise RuntimeError(f"Integration failed with code {int(bad[0])}")
            t_out = t[::stride]
        else:
            n_out = (ntimes - 1) // stride + 1
            nb = (n + nbatch - 1) // nbatch
            out = torch.empty((6, n_out, n) if save_all else (6, n), dtype=torch.float64, device=dev)
            status = torch.zeros(max(nb, 1), dtype=torch.int32, device=dev)
            _abi.call("gx_dop853_integrate_hamiltonian", pot, frame, ptr(w0d), n, ptr(td), ntimes, atol, rtol,
                      nmax, dt_max, nstiff, int(bool(save_all)), nbatch, stride, ptr(out), ptr(status), None, st)
            if err_if_fail == 1 and n > 0:
                res = status.cpu().numpy()
                bad = res[res < 0]
                if bad.size:
                    raise RuntimeError(f"Integration failed with code {int(bad[0])}")
            t_out = t[::stride]

        if not save_all:
            t_out = t[-1:]
        # chamiltonian.pyx:359-360 and 370-371: a single orbit loses its last axis,
        # and save_all=False keeps a length-1 time axis.
        w = out if return_device else out.cpu().numpy()
        if w.shape[-1] == 1:
            w = w[..., 0]
        if not save_all:
            w = w[:, None]
        if return_device:
            return Orbit.from_w(w, t=t_out, hamiltonian=self)
        return Orbit.from_w(w=w, t=t_out, hamiltonian=self, copy=False)
