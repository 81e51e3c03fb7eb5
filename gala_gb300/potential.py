"""Potential classes with gala's constructor signatures and C parameter packing.

Each class packs its parameters exactly as gala's Cython wrapper does,
``[G, *params]`` (``CPotentialWrapper.init``,
src/gala/potential/potential/cpotential.pyx:57-102; builtin wrappers,
src/gala/potential/potential/builtin/cybuiltin.pyx:141-372), and a composite
keeps its components in insertion order (``CCompositePotentialWrapper``,
src/gala/potential/potential/ccompositepotential.pyx:27-67).  The packed form is
the ``gx_potential`` descriptor of include/gala_gb300.h; every evaluation and
integration runs on the GPU through that descriptor.
"""
from __future__ import annotations

import ctypes as C
from collections import OrderedDict

import numpy as np

from . import _abi
from .units import G as G_GALACTIC
from .units import galactic
from ._trace import traced

__all__ = [
    "PotentialBase",
    "NullPotential",
    "KeplerPotential",
    "HernquistPotential",
    "PlummerPotential",
    "MiyamotoNagaiPotential",
    "NFWPotential",
    "SCFPotential",
    "CompositePotential",
    "CCompositePotential",
    "MilkyWayPotential",
]


def _rotation_matrix(R):
    if R is None:
        return np.eye(3)
    if hasattr(R, "as_matrix"):  # scipy.spatial.transform.Rotation
        R = R.as_matrix()
    R = np.asarray(R, dtype=np.float64)
    if R.shape != (3, 3):
        raise ValueError(f"Rotation matrix must have shape (3, 3), got {R.shape}")
    return R


class PackedPotential:
    """A ``gx_potential`` descriptor plus the arrays it points to (kept alive here)."""

    def __init__(self, comps):
        n = len(comps)
        params = [np.asarray(p, dtype=np.float64).ravel() for (_, p, _, _) in comps]
        offsets = np.cumsum([0] + [len(p) for p in params])[:-1]
        self.params = np.ascontiguousarray(np.concatenate(params) if params else np.zeros(1))
        self.components = (_abi.gx_component * max(n, 1))()
        self.has_scf = False
        for i, ((typ, p, q0, R), off) in enumerate(zip(comps, offsets)):
            c = self.components[i]
            c.type = typ
            c.n_params = len(params[i])
            c.param_offset = int(off)
            q0 = np.zeros(3) if q0 is None else np.asarray(q0, dtype=np.float64)
            R = np.eye(3) if R is None else np.asarray(R, dtype=np.float64)
            # cpotential.pyx:99-102: skip the transform iff q0 == 0 and R == I
            c.do_shift_rotate = 0 if (np.all(q0 == 0.0) and np.all(R == np.eye(3))) else 1
            for k in range(3):
                c.q0[k] = q0[k]
            for k in range(9):
                c.R[k] = R.ravel()[k]
            if typ == _abi.GX_POT_SCF:
                self.has_scf = True
        self.desc = _abi.gx_potential()
        self.desc.n_components = n
        self.desc.n_dim = 3
        self.desc.components = C.cast(self.components, C.POINTER(_abi.gx_component))
        self.desc.params = self.params.ctypes.data_as(C.POINTER(C.c_double))
        self.desc.params_device = None
        self.desc.n_params_total = len(self.params)
        self.desc.table_device = None
        self._dev = None
        self._table = None
        # more components than the by-value descriptor holds: the kernels read
        # them from a component table in device memory
        self.large = n > _abi.GX_MAX_COMPONENTS

    def for_device(self):
        """Descriptor with ``params_device`` filled (uploads the parameters once)
        and, for a large composite, the component table in device memory."""
        if (self.has_scf or self.large) and self._dev is None:
            import torch

            from ._device import require_cuda

            self._dev = torch.from_numpy(self.params).to(require_cuda())
            self.desc.params_device = int(self._dev.data_ptr())
        if self.large and self._table is None:
            import torch

            lib = _abi.load()
            nbytes = int(lib.gx_component_table_bytes(self.desc.n_components))
            host = np.zeros(nbytes, dtype=np.uint8)
            _abi.call("gx_pack_component_table", C.byref(self.desc), host.ctypes.data, nbytes)
            self._table = torch.from_numpy(host).to(self._dev.device)
            self.desc.table_device = int(self._table.data_ptr())
        return C.byref(self.desc)

    def for_host(self):
        return C.byref(self.desc)


class PotentialBase:
    """Base class: parameter handling, GPU evaluation and orbit integration.

    Parameters are given positionally in gala's declared order or by keyword;
    values are plain floats in the galactic unit system.
    """

    _param_names: tuple = ()
    _param_defaults: dict = {}
    ndim = 3

    def __init__(self, *args, units=None, origin=None, R=None, **kwargs):
        if units not in (None, galactic, "galactic"):
            raise ValueError("gala_gb300 works in the galactic unit system (kpc, Myr, Msun)")
        self.units = galactic
        self.G = G_GALACTIC
        names = self._param_names
        if len(args) > len(names):
            raise TypeError(f"{type(self).__name__} takes {len(names)} parameters, got {len(args)}")
        params = OrderedDict()
        for name, val in zip(names, args):
            params[name] = val
        for name in names[len(args):]:
            if name in kwargs:
                params[name] = kwargs.pop(name)
            elif name in self._param_defaults:
                params[name] = self._param_defaults[name]
            else:
                raise TypeError(f"{type(self).__name__}: missing required parameter '{name}'")
        if kwargs:
            raise TypeError(f"{type(self).__name__}: unexpected parameters {sorted(kwargs)}")
        self.parameters = OrderedDict((k, self._coerce(k, v)) for k, v in params.items())
        self.origin = np.zeros(3) if origin is None else np.asarray(origin, dtype=np.float64)
        if self.origin.shape != (3,):
            raise ValueError("origin must have shape (3,)")
        self.R = None if R is None else _rotation_matrix(R)
        self._packed = None

    _GALACTIC_UNIT = {"mass": "Msun", "length": "kpc", "dimensionless": ""}

    def _coerce(self, name, v):
        """A parameter value in galactic units.  A quantity (an object with
        ``unit`` and ``to_value``, e.g. astropy's) is converted to the unit of the
        parameter's physical type; a plain number is taken as galactic."""
        if hasattr(v, "unit") and hasattr(v, "to_value"):
            from .potential_io import _PARAM_TYPES

            ptype = _PARAM_TYPES.get(type(self).__name__, {}).get(name)
            if ptype is None:
                raise TypeError(f"{type(self).__name__}: no unit is known for parameter {name!r}")
            v = v.to_value(self._GALACTIC_UNIT[ptype])
        a = np.asarray(v, dtype=np.float64)
        return float(a) if a.ndim == 0 else a

    # --- C packing -----------------------------------------------------------
    def _c_type(self) -> int:
        raise NotImplementedError

    def _c_parameters(self) -> list:
        return [self.parameters[k] for k in self._param_names]

    def _components(self):
        """List of (type, [G, *params], q0, R) in evaluation order."""
        p = np.concatenate([[self.G], np.concatenate([np.atleast_1d(x).ravel() for x in self._c_parameters()])
                            if self._c_parameters() else []])
        return [(self._c_type(), p, self.origin, self.R if self.R is not None else np.eye(3))]

    def packed(self) -> PackedPotential:
        if self._packed is None:
            self._packed = PackedPotential(self._components())
        return self._packed

    @property
    def c_enabled(self):
        return True

    # --- evaluation (GPU) ----------------------------------------------------
    @traced("potential_eval")
    def _eval(self, kind, q, t=0.0):
        import torch

        from ._device import as_device_f64, ptr, stream_handle

        q = np.asarray(q, dtype=np.float64) if not isinstance(q, torch.Tensor) else q
        shape = tuple(q.shape)
        if not shape or shape[0] != 3:  # a scalar is refused, as in gala (regression 165)
            raise ValueError(f"positions must have shape (3, ...), got {shape}")
        qd = as_device_f64(q).reshape(3, -1).contiguous()
        n = qd.shape[1]
        out = torch.empty((3, n) if kind == "gradient" else (n,), dtype=torch.float64, device=qd.device)
        name = {"value": "gx_potential_value", "gradient": "gx_potential_gradient",
                "density": "gx_potential_density"}[kind]
        _abi.call(name, self.packed().for_device(), float(t), ptr(qd), n, ptr(out), stream_handle())
        res = out.cpu().numpy()
        if kind == "gradient":
            return res.reshape(shape)
        return res.reshape(shape[1:])

    def energy(self, q, t=0.0):
        """Potential energy Phi(q) (CPotentialWrapper.energy, cpotential.pyx:104-122)."""
        return self._eval("value", q, t)

    def gradient(self, q, t=0.0):
        """grad Phi(q) (c_gradient, cpotential.cpp:214-287)."""
        return self._eval("gradient", q, t)

    def density(self, q, t=0.0):
        """Density (c_density, cpotential.cpp:192-211)."""
        return self._eval("density", q, t)

    def acceleration(self, q, t=0.0):
        return -self.gradient(q, t)

    def circular_velocity(self, q, t=0.0):
        """sqrt(r |dPhi/dr|) from the gradient (PotentialBase.circular_velocity)."""
        q = np.asarray(q, dtype=np.float64)
        if q.ndim == 0 or q.shape[0] != 3:
            raise ValueError(f"positions must have shape (3, ...), got {q.shape}")
        r = np.sqrt(np.sum(q ** 2, axis=0))
        dPhi_dr = np.sum(self.gradient(q, t) * q, axis=0) / r
        return np.sqrt(r * np.abs(dPhi_dr))

    def mass_enclosed(self, q, t=0.0):
        """Mass within the spherical radius of each position, r^2 |dPhi/dr| / G
        with dPhi/dr the central difference of step 1e-3 along the radial
        direction (PotentialBase.mass_enclosed, src/gala/potential/potential/core.py:649-707);
        negated when the potential's mass parameter is negative, as gala does.
        Both sides of every difference are evaluated in one GPU call."""
        q = np.asarray(q, dtype=np.float64)
        if q.ndim == 0 or q.shape[0] != 3:
            raise ValueError(f"positions must have shape (3, ...), got {q.shape}")
        shape = q.shape[1:]
        q2 = q.reshape(3, -1)
        n = q2.shape[1]
        h = 1e-3
        r = np.sqrt(np.sum(q2 ** 2, axis=0))
        eps = h * q2 / r
        phi = np.asarray(self.energy(np.concatenate([q2 + eps, q2 - eps], axis=1), t))
        menc = np.abs(r * r * (phi[:n] - phi[n:]) / self.G / (2.0 * h))
        sgn = -1.0 if float(np.sum(self.parameters.get("m", 1.0))) < 0 else 1.0
        return (sgn * menc).reshape(shape)

    def replicate(self, **kwargs):
        """A copy with some parameters, the origin or the rotation R replaced
        (PotentialBase.replicate, src/gala/potential/potential/core.py)."""
        params = dict(self.parameters)
        origin = kwargs.pop("origin", self.origin)
        R = kwargs.pop("R", self.R)
        kwargs.pop("units", None)
        unknown = set(kwargs) - set(params)
        if unknown:
            raise TypeError(f"{type(self).__name__} has no parameters {sorted(unknown)}")
        params.update(kwargs)
        return type(self)(**params, origin=origin, R=R)

    # --- integration ---------------------------------------------------------
    def integrate_orbit(self, *args, **kwargs):
        """Integrate an orbit in this potential (PotentialBase.integrate_orbit,
        src/gala/potential/potential/core.py:1150-1184): delegates to
        Hamiltonian(self).integrate_orbit."""
        from .hamiltonian import Hamiltonian

        return Hamiltonian(self).integrate_orbit(*args, **kwargs)

    # --- composition ---------------------------------------------------------
    def __add__(self, other):
        if not isinstance(other, PotentialBase):
            raise TypeError(f"Cannot add a {type(self).__name__} to a {type(other).__name__}")
        new = CCompositePotential()
        for i, pot in enumerate([self, other]):
            if isinstance(pot, CompositePotential):
                for k, v in pot.items():
                    new[f"{i}_{k}" if k in new else k] = v
            else:
                new[str(len(new))] = pot
        return new

    def __repr__(self):
        pars = ", ".join(f"{k}={v if np.ndim(v) == 0 else np.shape(v)}" for k, v in self.parameters.items())
        return f"<{type(self).__name__}: {pars} (kpc,Myr,Msun)>"


class NullPotential(PotentialBase):
    """Zero potential (null_* in builtin_potentials.cpp:18-21)."""

    def _c_type(self):
        return _abi.GX_POT_NULL


class KeplerPotential(PotentialBase):
    """Point mass, params [G, m] (kepler_*, builtin_potentials.cpp:58-88)."""

    _param_names = ("m",)

    def _c_type(self):
        return _abi.GX_POT_KEPLER


class HernquistPotential(PotentialBase):
    """Hernquist sphere, params [G, m, c] (hernquist_*, builtin_potentials.cpp:211-244)."""

    _param_names = ("m", "c")

    def _c_type(self):
        return _abi.GX_POT_HERNQUIST


class PlummerPotential(PotentialBase):
    """Plummer sphere, params [G, m, b] (plummer_*, builtin_potentials.cpp:292-324)."""

    _param_names = ("m", "b")

    def _c_type(self):
        return _abi.GX_POT_PLUMMER


class MiyamotoNagaiPotential(PotentialBase):
    """Miyamoto-Nagai disk, params [G, m, a, b] (builtin_potentials.cpp:1287-1332)."""

    _param_names = ("m", "a", "b")

    def _c_type(self):
        return _abi.GX_POT_MIYAMOTONAGAI


class NFWPotential(PotentialBase):
    """NFW halo, params [G, m, r_s, a, b, c].

    Like gala (src/gala/potential/potential/builtin/core.py:719-734) the C
    implementation is chosen from the axis ratios: spherical when a = b = c = 1,
    flattened when a = b = 1, triaxial otherwise.
    """

    _param_names = ("m", "r_s", "a", "b", "c")
    _param_defaults = {"a": 1.0, "b": 1.0, "c": 1.0}

    def _c_type(self):
        a, b, c = (self.parameters[k] for k in "abc")
        if np.allclose([a, b, c], 1.0):
            return _abi.GX_POT_SPHERICALNFW
        if np.allclose([a, b], 1.0):
            return _abi.GX_POT_FLATTENEDNFW
        return _abi.GX_POT_TRIAXIALNFW

    @classmethod
    def from_circular_velocity(cls, v_c, r_s, a=1.0, b=1.0, c=1.0, r_ref=None, units=None, origin=None, R=None):
        """NFW from the circular velocity v_c (kpc/Myr) at r_ref (default r_s),
        as gala computes it (NFWPotential._vc_rs_rref_to_m,
        src/gala/potential/potential/builtin/core.py:866-870): with u = r_ref / r_s,
        G m / r_s = v_c^2 / u / (ln(1 + u) / u^2 - 1 / (u (1 + u))), i.e. the circular
        speed at r_ref is v_c.  (The formula in gala's docstring differs from its code.)"""
        def galactic(x, unit):  # quantities (anything with to_value) to galactic units
            return x.to_value(unit) if hasattr(x, "to_value") else x

        v_c, r_s = galactic(v_c, "kpc / Myr"), galactic(r_s, "kpc")
        if r_ref is None:
            r_ref = r_s
        r_ref = galactic(r_ref, "kpc")
        u = r_ref / r_s
        m = r_s * (v_c ** 2 / u / (np.log(1 + u) / u ** 2 - 1 / (u * (1 + u)))) / G_GALACTIC
        return cls(m=m, r_s=r_s, a=a, b=b, c=c, units=units, origin=origin, R=R)


class SCFPotential(PotentialBase):
    """SCF basis-function expansion (src/gala/potential/scf/bfe_class.pyx:38-106).

    Packing is gala's: [G, nmax, lmax, m, r_s, Snlm.ravel(), Tnlm.ravel()] with
    Snlm, Tnlm of shape (nmax+1, lmax+1, lmax+1).
    """

    _param_names = ("m", "r_s", "Snlm", "Tnlm")

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        S, T = np.atleast_3d(self.parameters["Snlm"]), np.atleast_3d(self.parameters["Tnlm"])
        if S.shape != T.shape:
            raise ValueError(
                "The input coefficient arrays Snlm and Tnlm must have the same shape! "
                f"Received: {S.shape} and {T.shape}")
        if S.ndim != 3 or S.shape[1] != S.shape[2]:
            raise ValueError(f"Snlm must have shape (nmax+1, lmax+1, lmax+1), got {S.shape}")
        self.nmax = S.shape[0] - 1
        self.lmax = S.shape[1] - 1

    def _c_type(self):
        return _abi.GX_POT_SCF

    def _c_parameters(self):
        p = self.parameters
        return [float(self.nmax), float(self.lmax), p["m"], p["r_s"], p["Snlm"], p["Tnlm"]]


class CompositePotential(PotentialBase, OrderedDict):
    """Ordered collection of potentials, summed in insertion order."""

    def __init__(self, *args, **kwargs):
        OrderedDict.__init__(self)
        self.units = galactic
        self.G = G_GALACTIC
        self.parameters = OrderedDict()
        self.origin = np.zeros(3)
        self.R = None
        self._packed = None
        self.lock = False
        if len(args) == 1 and isinstance(args[0], dict):
            kwargs = dict(args[0], **kwargs)
        elif args:
            raise TypeError("CompositePotential takes potentials as keyword arguments")
        for k, v in kwargs.items():
            self[k] = v

    def __setitem__(self, key, value):
        if getattr(self, "lock", False):
            raise ValueError("Potential object is locked - new components can only be added to unlocked potentials.")
        if not isinstance(value, PotentialBase):
            raise TypeError(f"Potential components may only be Potential objects, not {type(value)}.")
        OrderedDict.__setitem__(self, key, value)
        self._packed = None

    def __hash__(self):
        return id(self)

    def replicate(self, **kwargs):
        raise NotImplementedError("replicate the components and compose them again")

    def __eq__(self, other):
        return self is other

    def _components(self):
        out = []
        for pot in self.values():
            out.extend(pot._components())
        return out

    def __repr__(self):
        return f"<{type(self).__name__}: {', '.join(self.keys())}>"


class CCompositePotential(CompositePotential):
    """Composite of C-implemented components (same as CompositePotential here)."""


class MilkyWayPotential(CCompositePotential):
    """gala's MilkyWayPotential (version v1, src/gala/potential/potential/builtin/special.py:98-124):
    Miyamoto-Nagai disk + Hernquist bulge + Hernquist nucleus + spherical NFW halo.

    ``version`` is gala's selector (special.py:186-216); only "v1" is
    implemented here (v2 needs the MN3 exponential disk)."""

    def __init__(self, disk=None, halo=None, bulge=None, nucleus=None, units=None, version="v1"):
        self.version = str(version).lower()
        if self.version != "v1":
            raise NotImplementedError(f"MilkyWayPotential version {version!r}: only 'v1' is implemented")
        super().__init__()
        disk = dict({"m": 6.8e10, "a": 3.0, "b": 0.28}, **(disk or {}))
        bulge = dict({"m": 5e9, "c": 1.0}, **(bulge or {}))
        nucleus = dict({"m": 1.71e9, "c": 0.07}, **(nucleus or {}))
        halo = dict({"m": 5.4e11, "r_s": 15.62}, **(halo or {}))
        self["disk"] = MiyamotoNagaiPotential(**disk)
        self["bulge"] = HernquistPotential(**bulge)
        self["nucleus"] = HernquistPotential(**nucleus)
        self["halo"] = NFWPotential(**halo)
        self.lock = True
