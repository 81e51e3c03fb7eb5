"""Direct n-body integration: gala.dynamics.nbody.DirectNBody on the GPU.

``DirectNBody`` keeps gala's constructor and ``integrate_orbit``
(src/gala/dynamics/nbody/core.py:20-280): massive bodies are moved to the
front, the system is integrated with DOPRI853 exactly as direct_nbody_dop853
does (nbody.pyx:30-115: dop853_helper with Fwrapper_direct_nbody, nstiff = -1)
or with Leapfrog as leapfrog_integrate_nbody does (leapfrog.pyx:161-255), and
the result is put back in the input order.  ``integrate_systems`` /
``integrate_systems_leapfrog`` run many independent systems of the same shape in
one launch (gx_nbody_dop853 / gx_nbody_leapfrog).

Particle potentials must be single, unrotated components of the types the GPU
body kernel evaluates (Null, Kepler, Hernquist, Plummer, Miyamoto-Nagai,
spherical NFW); ``None`` means a test particle (gala's NullPotential).
"""
from __future__ import annotations

import numpy as np

from . import _abi
from .dynamics import Orbit, PhaseSpacePosition
from .hamiltonian import Hamiltonian, StaticFrame
from .integrate import DOPRI853Integrator, LeapfrogIntegrator, get_integrator, parse_time_specification
from .potential import NullPotential, PotentialBase
from ._trace import traced

__all__ = ["DirectNBody", "BODY_DTYPE", "body_record", "pack_bodies", "integrate_systems",
           "integrate_systems_leapfrog"]

# numpy mirror of gx_body (include/gala_gb300.h)
BODY_DTYPE = np.dtype([("type", "<i4"), ("n_params", "<i4"), ("params", "<f8", (7,))])
assert BODY_DTYPE.itemsize == 64

GPU_BODY_TYPES = (_abi.GX_POT_NULL, _abi.GX_POT_KEPLER, _abi.GX_POT_HERNQUIST, _abi.GX_POT_PLUMMER,
                  _abi.GX_POT_MIYAMOTONAGAI, _abi.GX_POT_SPHERICALNFW)


def is_null(pot) -> bool:
    return pot is None or isinstance(pot, NullPotential)


def body_record(pot) -> np.ndarray:
    """The gx_body of one particle potential (a 0-d BODY_DTYPE record)."""
    rec = np.zeros((), dtype=BODY_DTYPE)
    if is_null(pot):
        rec["type"] = _abi.GX_POT_NULL
        rec["n_params"] = 1
        rec["params"][0] = pot.G if pot is not None else 0.0
        return rec
    if not isinstance(pot, PotentialBase):
        raise TypeError(f"particle potentials must be potential objects or None, not {type(pot)}")
    comps = pot._components()
    if len(comps) != 1:
        raise NotImplementedError("a particle potential must be a single component on the GPU")
    typ, p, q0, R = comps[0]
    if typ not in GPU_BODY_TYPES:
        raise NotImplementedError(f"{type(pot).__name__} is not available as a particle potential on the GPU")
    if np.any(np.asarray(q0) != 0) or not np.array_equal(np.asarray(R), np.eye(3)):
        raise NotImplementedError("particle potentials with an origin or a rotation are not supported")
    p = np.asarray(p, dtype=np.float64).ravel()
    if p.size > 7:
        raise ValueError(f"too many parameters for a particle potential ({p.size})")
    rec["type"] = typ
    rec["n_params"] = p.size
    rec["params"][: p.size] = p
    return rec


def pack_bodies(potentials) -> np.ndarray:
    """BODY_DTYPE array of the given particle potentials (any nesting of lists)."""
    arr = np.asarray(potentials, dtype=object)
    out = np.zeros(arr.shape, dtype=BODY_DTYPE)
    for idx in np.ndindex(arr.shape):
        out[idx] = body_record(arr[idx])
    return out


def bodies_to_device(bodies: np.ndarray, device):
    import torch

    raw = np.ascontiguousarray(bodies).view(np.uint8).reshape(-1)
    return torch.from_numpy(raw.copy()).to(device)


def integrate_systems(hamiltonian, bodies, w0, t, atol=1e-10, rtol=1e-10, nmax=0, dt_max=0.0, nstiff=-1,
                      save_all=True, out_stride=1, return_stats=False, stream=None):
    """Integrate n_systems independent direct n-body systems of the same shape.

    bodies : BODY_DTYPE (n_systems, nbody) potentials of the massive bodies,
             which are the first ``nbody`` of each system's particles
    w0     : (n_systems, nparticles, 6) float64 (numpy or CUDA tensor)
    t      : (ntimes,) output times; h0 = t[1] - t[0] as in dop853_helper
    Returns (w, status[, stats]) as CUDA tensors: w (n_systems, n_out,
    nparticles, 6) if save_all else (n_systems, nparticles, 6).
    """
    import torch

    from ._device import as_device_f64, ptr, require_cuda, stream_handle

    H = hamiltonian if isinstance(hamiltonian, Hamiltonian) else Hamiltonian(hamiltonian)
    dev = require_cuda()
    w0d = as_device_f64(w0, dev)
    if w0d.ndim != 3 or w0d.shape[2] != 6:
        raise ValueError(f"w0 must have shape (n_systems, nparticles, 6), got {tuple(w0d.shape)}")
    ns, npart = int(w0d.shape[0]), int(w0d.shape[1])
    bodies = np.asarray(bodies, dtype=BODY_DTYPE)
    if bodies.ndim != 2 or bodies.shape[0] != ns:
        raise ValueError(f"bodies must have shape (n_systems, nbody), got {bodies.shape}")
    nbody = int(bodies.shape[1])
    if npart < 1:
        raise ValueError("a system needs at least one particle")
    if nbody > npart:
        raise ValueError("more massive bodies than particles")
    t = np.ascontiguousarray(np.asarray(t, dtype=np.float64))
    ntimes = len(t)
    if ntimes < 2:
        raise ValueError("ntimes must be greater than 1")
    if out_stride < 1:
        raise ValueError("out_stride must be >= 1")
    td = torch.from_numpy(t).to(dev)
    bd = bodies_to_device(bodies if nbody else np.zeros((ns, 1), dtype=BODY_DTYPE), dev)
    n_out = (ntimes - 1) // out_stride + 1
    out = torch.empty((ns, n_out, npart, 6) if save_all else (ns, npart, 6), dtype=torch.float64, device=dev)
    status = torch.zeros(max(ns, 1), dtype=torch.int32, device=dev)
    stats = torch.zeros((max(ns, 1), 4), dtype=torch.int64, device=dev) if return_stats else None
    counter = torch.zeros(1, dtype=torch.int64, device=dev)
    if npart <= 32:  # a system is a group of lanes of one warp
        _abi.call("gx_nbody_dop853", H.potential.packed().for_device(), H._frame_ref(), ns, npart, nbody, ptr(bd),
                  ptr(w0d), ptr(td), ntimes, float(atol), float(rtol), int(nmax), float(dt_max), int(nstiff),
                  int(bool(save_all)), int(out_stride), ptr(out), ptr(status),
                  ptr(stats) if stats is not None else None, ptr(counter), stream_handle(stream))
    else:  # wider systems: one CTA each, the state in device scratch
        nbytes = int(_abi.load().gx_nbody_wide_scratch_bytes(ns, npart))
        scratch = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=dev)
        _abi.call("gx_nbody_dop853_wide", H.potential.packed().for_device(), H._frame_ref(), ns, npart, nbody,
                  ptr(bd), ptr(w0d), ptr(td), ntimes, float(atol), float(rtol), int(nmax), float(dt_max),
                  int(nstiff), int(bool(save_all)), int(out_stride), ptr(scratch), nbytes, ptr(out), ptr(status),
                  ptr(stats) if stats is not None else None, stream_handle(stream))
    if return_stats:
        return out, status[:ns], stats[:ns]
    return out, status[:ns]


def integrate_systems_leapfrog(hamiltonian, bodies, w0, t, save_all=True, stream=None):
    """leapfrog_integrate_nbody (leapfrog.pyx:161-255) for n_systems independent
    systems of at most 8 bodies, the first ``bodies.shape[1]`` massive; static
    frame.  Returns w (n_systems, ntimes, nparticles, 6) if save_all, else
    (n_systems, nparticles, 6), as a CUDA tensor."""
    import torch

    from ._device import as_device_f64, ptr, require_cuda, stream_handle

    H = hamiltonian if isinstance(hamiltonian, Hamiltonian) else Hamiltonian(hamiltonian)
    if not isinstance(H.frame, StaticFrame):
        raise TypeError(f"Leapfrog integration is currently only supported for StaticFrame, "
                        f"not {H.frame.__class__.__name__}")
    dev = require_cuda()
    w0d = as_device_f64(w0, dev)
    if w0d.ndim != 3 or w0d.shape[2] != 6:
        raise ValueError(f"w0 must have shape (n_systems, nparticles, 6), got {tuple(w0d.shape)}")
    ns, npart = int(w0d.shape[0]), int(w0d.shape[1])
    bodies = np.asarray(bodies, dtype=BODY_DTYPE)
    nbody = int(bodies.shape[1])
    if not 1 <= npart <= 8:
        raise NotImplementedError(f"Leapfrog systems of {npart} bodies: the GPU kernel takes 1 to 8")
    t = np.ascontiguousarray(np.asarray(t, dtype=np.float64))
    if len(t) < 2:
        raise ValueError("ntimes must be greater than 1")
    td = torch.from_numpy(t).to(dev)
    bd = bodies_to_device(bodies if nbody else np.zeros((ns, 1), dtype=BODY_DTYPE), dev)
    out = torch.empty((ns, len(t), npart, 6) if save_all else (ns, npart, 6), dtype=torch.float64, device=dev)
    _abi.call("gx_nbody_leapfrog", H.potential.packed().for_device(), ns, npart, nbody, ptr(bd), ptr(w0d), ptr(td),
              len(t), int(bool(save_all)), ptr(out), stream_handle(stream))
    return out

class DirectNBody:
    """Direct n-body integration of bodies with their own potentials in an
    optional external potential (gala.dynamics.nbody.DirectNBody)."""

    def __init__(self, w0, particle_potentials, external_potential=None, frame=None, units=None, save_all=True):
        if not isinstance(w0, PhaseSpacePosition):
            raise TypeError("Initial conditions `w0` must be a gala_gb300.PhaseSpacePosition object, "
                            f"not '{w0.__class__.__name__}'")
        if len(w0.shape) > 0 and w0.shape[0] != len(particle_potentials):
            raise ValueError("The number of initial conditions in `w0` must match the number of particle "
                             "potentials passed in with `particle_potentials`.")
        self.particle_potentials = [NullPotential() if p is None else p for p in particle_potentials]
        self.external_potential = NullPotential() if external_potential is None else external_potential
        self.frame = StaticFrame() if frame is None else frame
        self.units = self.external_potential.units
        self.save_all = save_all
        self.H = Hamiltonian(self.external_potential, frame=self.frame)
        self.w0 = w0

    @property
    def w0(self):
        return self._w0

    @w0.setter
    def w0(self, value):
        self._w0 = value
        pos = np.asarray(value.xyz, dtype=np.float64)
        vel = np.asarray(value.v_xyz, dtype=np.float64)
        if pos.ndim == 1:
            pos = pos[:, None]
            vel = vel[:, None]
        self._c_w0 = np.ascontiguousarray(np.vstack((pos, vel)).T)

    def __repr__(self):
        return f"<{self.__class__.__name__} bodies={self._c_w0.shape[0]}>"

    def _order(self):
        """Massive bodies first, each group in input order (core.py:211-224)."""
        front = [i for i, p in enumerate(self.particle_potentials) if not is_null(p)]
        end = [i for i, p in enumerate(self.particle_potentials) if is_null(p)]
        return np.array(front + end, dtype=np.int64), len(front)

    @traced("nbody_integrate_orbit")
    def integrate_orbit(self, Integrator=None, Integrator_kwargs=None, return_device=False, **time_spec):
        """Integrate the bodies; returns an Orbit of shape (3, ntimes, nbodies) if
        save_all, else a PhaseSpacePosition (3, nbodies) (core.py:166-280)."""
        if Integrator_kwargs is None:
            Integrator_kwargs = {}
        Integrator = get_integrator(DOPRI853Integrator if Integrator is None else Integrator)
        if Integrator not in (DOPRI853Integrator, LeapfrogIntegrator):
            raise NotImplementedError(
                f"N-body integration on the GPU is implemented for DOPRI853Integrator and LeapfrogIntegrator, "
                f"not {Integrator.__name__}")
        t = np.ascontiguousarray(parse_time_specification(self.units, **time_spec), dtype=np.float64)
        idx, nbody = self._order()
        reorg = self._c_w0[idx]
        pps = [self.particle_potentials[i] for i in idx]
        bodies = pack_bodies([pps[:nbody]]) if nbody else np.zeros((1, 0), dtype=BODY_DTYPE)
        if Integrator is LeapfrogIntegrator:
            out = integrate_systems_leapfrog(self.H, bodies, reorg[None], t, save_all=self.save_all)
        else:
            kw = dict(Integrator_kwargs)
            err_if_fail = int(kw.pop("err_if_fail", 1))
            kw.pop("log_output", None)
            allowed = {"atol", "rtol", "nmax", "dt_max"}
            extra = set(kw) - allowed
            if extra:
                raise TypeError(f"unexpected Integrator_kwargs {sorted(extra)}")
            out, status = integrate_systems(self.H, bodies, reorg[None], t, save_all=self.save_all, nstiff=-1,
                                            **kw)
            res = int(status.cpu().numpy()[0])
            if res < 0 and err_if_fail == 1:
                raise RuntimeError(f"Integration failed with code {res}")
        undo = np.argsort(idx)
        if self.save_all:
            w = out[0][:, undo]  # (ntimes, nbodies, 6)
            w = w.permute(2, 0, 1).contiguous()  # (6, ntimes, nbodies)
            if return_device:
                return Orbit.from_w(w, t=t, hamiltonian=self.H)
            return Orbit.from_w(w.cpu().numpy(), t=t, hamiltonian=self.H, copy=False)
        w = out[0][undo].T.contiguous()  # (6, nbodies)
        return PhaseSpacePosition.from_w(w.cpu().numpy(), frame=self.frame)
