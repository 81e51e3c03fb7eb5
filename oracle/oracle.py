"""ORACLE (test infrastructure only): ctypes front end of the CPU checkers."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBS = {
    "strict": HERE / "_build" / "liboracle.so",
    "fast": HERE / "_build" / "liboracle_fast.so",
    "ref": HERE / "_ref" / "libgalaref.so",
    "ref_strict": HERE / "_ref" / "libgalaref_strict.so",
}
_P = C.c_void_p


def build(ref: bool = True) -> None:
    """Build the restatement (always) and gala's own objects (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)


def ref_available() -> bool:
    return LIBS["ref"].exists()


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _p(a):
    return a.ctypes.data_as(_P)


class Oracle:
    """One of the CPU checkers; `kind` is 'strict', 'fast', 'ref' or 'ref_strict'."""

    def __init__(self, kind: str = "strict"):
        path = LIBS[kind]
        if not path.exists():
            if kind.startswith("ref"):
                raise FileNotFoundError(f"{path} not built (gala sources unavailable here)")
            build(ref=False)
        self.kind = kind
        self.lib = C.CDLL(str(path))
        self.is_ref = kind.startswith("ref")

    @staticmethod
    def _frame(frame):
        if frame is None:
            return None
        return C.byref(frame.c_frame())

    # ------------------------------------------------------------------ eval
    def gradient(self, pot, q, t=0.0):
        q = _f64(q)
        shape = q.shape
        q2 = _f64(q.reshape(3, -1))
        n = q2.shape[1]
        out = np.zeros((3, n))
        if self.is_ref:
            rc = self.lib.ref_gradient(pot.packed().for_host(), C.c_int64(n), C.c_double(t), _p(q2), _p(out))
            if rc != 0:
                raise NotImplementedError("component not available in the gala build")
        else:
            self.lib.orc_gradient(pot.packed().for_host(), C.c_size_t(n), C.c_double(t), _p(q2), _p(out))
        return out.reshape(shape)

    def _scalar(self, fn_ref, fn_orc, pot, q, t):
        q = _f64(q)
        shape = q.shape
        q2 = _f64(q.reshape(3, -1))
        n = q2.shape[1]
        out = np.zeros(n)
        if self.is_ref:
            rc = getattr(self.lib, fn_ref)(pot.packed().for_host(), C.c_double(t), _p(q2), C.c_int64(n), _p(out))
            if rc != 0:
                raise NotImplementedError("component not available in the gala build")
        else:
            getattr(self.lib, fn_orc)(pot.packed().for_host(), C.c_double(t), _p(q2), C.c_int64(n), _p(out))
        return out.reshape(shape[1:])

    def energy(self, pot, q, t=0.0):
        return self._scalar("ref_potential_value_n", "orc_potential_value_n", pot, q, t)

    def density(self, pot, q, t=0.0):
        return self._scalar("ref_potential_density_n", "orc_potential_density_n", pot, q, t)

    def hamiltonian_value(self, pot, w, frame=None, t=0.0):
        w = _f64(w)
        shape = w.shape
        w2 = _f64(w.reshape(6, -1))
        n = w2.shape[1]
        out = np.zeros(n)
        self.lib.orc_hamiltonian_value_n(pot.packed().for_host(), self._frame(frame), C.c_double(t), _p(w2),
                                         C.c_int64(n), _p(out))
        return out.reshape(shape[1:])

    def hamiltonian_gradient(self, pot, w, frame=None, t=0.0):
        w = _f64(w)
        shape = w.shape
        w2 = _f64(w.reshape(6, -1))
        n = w2.shape[1]
        out = np.zeros((6, n))
        if self.is_ref:
            self.lib.ref_hamiltonian_gradient(pot.packed().for_host(), self._frame(frame), C.c_int64(n),
                                              C.c_double(t), _p(w2), _p(out))
        else:
            self.lib.orc_hamiltonian_gradient(pot.packed().for_host(), self._frame(frame), C.c_size_t(n),
                                              C.c_double(t), _p(w2), _p(out))
        return out.reshape(shape)

    # ------------------------------------------------------------ integrate
    def fixed(self, pot, w0, t, method="leapfrog", save_all=True, nthreads=1):
        """leapfrog / ruth4 integrate_hamiltonian; w0 (6, N) -> (6, ntimes, N) or (6, N)."""
        w0 = _f64(w0)
        t = _f64(t)
        n = w0.shape[1]
        m = 0 if method == "leapfrog" else 1
        out = np.zeros((6, len(t), n) if save_all else (6, n))
        fn = self.lib.ref_fixed_integrate if self.is_ref else self.lib.orc_fixed_integrate
        rc = fn(pot.packed().for_host(), C.c_int(m), _p(w0), C.c_int64(n), _p(t), C.c_int64(len(t)),
                C.c_int(int(save_all)), _p(out), C.c_int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle fixed-step integration failed ({rc})")
        return out

    def dop853(self, pot, w0, t, atol=1e-10, rtol=1e-10, nmax=0, dt_max=0.0, nstiff=0, save_all=True,
               nbatch=100, out_stride=1, frame=None, nthreads=1):
        """dop853_integrate_hamiltonian. Returns (w, status[, stats])."""
        w0 = _f64(w0)
        t = _f64(t)
        n = w0.shape[1]
        nb = (n + nbatch - 1) // nbatch
        status = np.zeros(max(nb, 1), dtype=np.int32)
        if self.is_ref:
            if out_stride != 1:
                raise ValueError("gala's own dop853 driver has no output stride")
            out = np.zeros((6, len(t), n) if save_all else (6, n))
            self.lib.ref_dop853_integrate(
                pot.packed().for_host(), self._frame(frame), _p(w0), C.c_int64(n), _p(t), C.c_int64(len(t)),
                C.c_double(atol), C.c_double(rtol), C.c_int64(nmax), C.c_double(dt_max), C.c_int64(nstiff),
                C.c_int(int(save_all)), C.c_int(nbatch), _p(out), status.ctypes.data_as(_P), C.c_int(nthreads))
            return out, status, None
        n_out = (len(t) - 1) // out_stride + 1
        out = np.zeros((6, n_out, n) if save_all else (6, n))
        stats = np.zeros((max(nb, 1), 4), dtype=np.int64)
        rc = self.lib.orc_dop853_integrate(
            pot.packed().for_host(), self._frame(frame), _p(w0), C.c_int64(n), _p(t), C.c_int64(len(t)),
            C.c_double(atol), C.c_double(rtol), C.c_int64(nmax), C.c_double(dt_max), C.c_int64(nstiff),
            C.c_int(int(save_all)), C.c_int(nbatch), C.c_int64(out_stride), _p(out), status.ctypes.data_as(_P),
            stats.ctypes.data_as(_P), C.c_int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle dop853 failed ({rc})")
        return out, status, stats


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1
