"""PhaseSpacePosition and Orbit containers (gala.dynamics equivalents).

Arrays are plain float64 in galactic units.  An Orbit may hold its phase-space
array on the GPU (a torch tensor) and converts to numpy on first host access.
"""
from __future__ import annotations

import numpy as np

__all__ = ["PhaseSpacePosition", "Orbit"]


def _to_numpy(a):
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


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

    def potential_energy(self, potential):
        return potential.energy(self.pos)

    def energy(self, hamiltonian):
        from .hamiltonian import Hamiltonian

        H = hamiltonian if isinstance(hamiltonian, Hamiltonian) else Hamiltonian(hamiltonian)
        return H.energy(self.w())


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
        return self.pos.shape[1]

    @property
    def norbits(self):
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

    def __getitem__(self, idx):
        w = self.w()
        if not isinstance(idx, tuple):
            idx = (idx,)
        wi = w[(slice(None),) + idx]
        t = self.t[idx[0]] if self.t is not None else None
        if wi.ndim >= 2 and t is not None and np.ndim(t) > 0:
            return Orbit.from_w(wi, t=t, hamiltonian=self.hamiltonian)
        return PhaseSpacePosition.from_w(wi)
