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
    """Build the restatement (always) and gala's own objects (when its sources
    exist); processes building at once take turns on a lock file."""
    import fcntl

    (HERE / "_build").mkdir(exist_ok=True)
    with open(HERE / "_build" / ".build.lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
            if ref:
                subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


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

    def batch_fixed(self, pot, w0, nsteps, dt, method, nthreads=1):
        """Per-orbit Leapfrog (method 0) / Ruth4 (1) with per-orbit n_steps and dt,
        each orbit on its own gala time grid; final states (6, N)."""
        if self.is_ref:
            raise ValueError("batch_fixed is a restatement-only entry point")
        w0 = _f64(w0)
        n = w0.shape[1]
        ns = np.ascontiguousarray(np.asarray(nsteps, dtype=np.int64))
        dt = _f64(dt)
        m = np.ascontiguousarray(np.asarray(method, dtype=np.int32))
        if ns.shape != (n,) or dt.shape != (n,) or m.shape != (n,):
            raise ValueError("nsteps, dt and method must each have one entry per orbit")
        out = np.zeros((6, n))
        rc = self.lib.orc_batch_fixed(pot.packed().for_host(), _p(w0), C.c_int64(n), _p(ns), _p(dt), _p(m),
                                      _p(out), C.c_int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle batch integration failed ({rc})")
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

    # --------------------------------------------------- n-body and streams
    @staticmethod
    def _bodies(b):
        b = np.ascontiguousarray(b)
        if b.dtype.itemsize != 64 or b.dtype.names != ("type", "n_params", "params"):
            raise TypeError("bodies must be a gx_body-layout structured array")
        return b

    def nbody_dop853(self, pot, bodies, nbody, w0, t, atol=1e-10, rtol=1e-10, nmax=0, dt_max=0.0, nstiff=-1,
                     save_all=True, frame=None):
        """direct_nbody_dop853 on one system: bodies (nparticles,) gx_body records
        (massive ones first, nbody of them), w0 (nparticles, 6).  Returns
        (w (ntimes, nparticles, 6) or (nparticles, 6), idid)."""
        b = self._bodies(bodies)
        w0 = _f64(w0)
        t = _f64(t)
        npart = w0.shape[0]
        out = np.zeros((len(t), npart, 6) if save_all else (npart, 6))
        if self.is_ref:
            res = self.lib.ref_nbody_dop853(
                pot.packed().for_host(), self._frame(frame), C.c_int(npart), C.c_int(nbody), _p(b), _p(w0), _p(t),
                C.c_int64(len(t)), C.c_double(atol), C.c_double(rtol), C.c_int64(nmax), C.c_double(dt_max),
                C.c_int64(nstiff), C.c_int(int(save_all)), _p(out))
        else:
            res = self.lib.orc_nbody_dop853(
                pot.packed().for_host(), self._frame(frame), C.c_int(npart), C.c_int(nbody), _p(b), _p(w0), _p(t),
                C.c_int64(len(t)), C.c_double(atol), C.c_double(rtol), C.c_int64(nmax), C.c_double(dt_max),
                C.c_int64(nstiff), C.c_int(int(save_all)), _p(out), None)
        return out, int(res)

    def mockstream_dop853(self, pot, bodies, nbody_w0, time, stream_w0, stream_t1, tfinal, nstream, atol=1e-10,
                          rtol=1e-10, nmax=0, dt_max=0.0, nstiff=-1, frame=None):
        """mockstream_dop853 for one progenitor system.  Returns
        (nbody_w_final (nbodies, 6), stream_w_final (ntot, 6), status (ntimes,))."""
        b = self._bodies(bodies)
        nbody_w0 = _f64(nbody_w0)
        time = _f64(time)
        stream_w0 = _f64(stream_w0).reshape(-1, 6)
        stream_t1 = _f64(stream_t1)
        nstream = np.ascontiguousarray(np.asarray(nstream, dtype=np.int32))
        nb = nbody_w0.shape[0]
        nb_out = np.zeros((nb, 6))
        st_out = np.zeros_like(stream_w0)
        status = np.zeros(len(time), dtype=np.int32)
        fn = self.lib.ref_mockstream_dop853 if self.is_ref else self.lib.orc_mockstream_dop853
        res = fn(pot.packed().for_host(), self._frame(frame), C.c_int(nb), _p(b), _p(nbody_w0), _p(time),
                 C.c_int64(len(time)), _p(stream_w0), _p(stream_t1), C.c_double(tfinal), _p(nstream),
                 C.c_double(atol), C.c_double(rtol), C.c_int64(nmax), C.c_double(dt_max), C.c_int64(nstiff),
                 _p(nb_out), _p(st_out), _p(status))
        if res < 0:
            raise RuntimeError(f"mockstream oracle failed ({res})")
        return nb_out, st_out, status

    def mockstream_animate(self, pot, bodies, nbody_w0, t, stream_w0, nstream, output_every=1, atol=1e-10,
                           rtol=1e-10, nmax=0, frame=None):
        """mockstream_dop853_animate for one progenitor system on the whole grid t.
        Returns (snap (noutput, nbodies + ntot, 6) NaN-filled, snap_t (noutput,),
        w_final (nbodies + ntot, 6), status (ntimes,), stats (4,) or None for gala's code)."""
        b = self._bodies(bodies)
        nbody_w0 = _f64(nbody_w0)
        t = _f64(t)
        stream_w0 = _f64(stream_w0).reshape(-1, 6)
        nstream = np.ascontiguousarray(np.asarray(nstream, dtype=np.int32))
        nb, ntimes = nbody_w0.shape[0], len(t)
        nout = (ntimes - 1) // output_every + 1 + int((ntimes - 1) % output_every != 0)
        allm = nb + int(nstream.sum())
        snap = np.zeros((nout, allm, 6))
        snap_t = np.zeros(nout)
        w_final = np.zeros((allm, 6))
        status = np.zeros(ntimes, dtype=np.int32)
        args = [pot.packed().for_host(), self._frame(frame), C.c_int(nb), _p(b), _p(nbody_w0), _p(t),
                C.c_int64(ntimes), _p(stream_w0), _p(nstream), C.c_int64(output_every), C.c_double(atol),
                C.c_double(rtol), C.c_int64(nmax), _p(snap), _p(snap_t), _p(w_final), _p(status)]
        stats = None
        if self.is_ref:
            res = self.lib.ref_mockstream_dop853_animate(*args)
        else:
            stats = np.zeros(4, dtype=np.int64)
            res = self.lib.orc_mockstream_dop853_animate(*args, _p(stats))
        if res != nout:
            raise RuntimeError(f"mockstream animate oracle failed ({res})")
        return snap, snap_t, w_final, status, stats

    def mockstream_systems(self, pot, bodies, nbody_w, release_t, nstream, stream_w0, t_final, dt0, atol=1e-10,
                           rtol=1e-10, nmax=0, sys_lo=0, sys_hi=None, nthreads=1, frame=None):
        """The release systems of many streams (the GPU entry point's layout):
        bodies (S, nb), nbody_w (S, n_release, nb, 6), stream_w0 (S, ntot, 6).
        Returns (stream_w (S, ntot, 6), nbody_w_final (S, nb, 6), status
        (S, n_release), stats (S, n_release, 4))."""
        if self.is_ref:
            raise NotImplementedError("use mockstream_dop853 for gala's own code")
        b = self._bodies(bodies)
        nbody_w = _f64(nbody_w)
        S, nrel, nb = nbody_w.shape[:3]
        release_t = _f64(release_t)
        nstream = np.ascontiguousarray(np.asarray(nstream, dtype=np.int32))
        stream_w0 = _f64(stream_w0)
        out = np.zeros_like(stream_w0)
        nb_out = np.zeros((S, nb, 6))
        status = np.zeros((S, nrel), dtype=np.int32)
        stats = np.zeros((S, nrel, 4), dtype=np.int64)
        hi = S * nrel if sys_hi is None else sys_hi
        rc = self.lib.orc_mockstream_systems(
            pot.packed().for_host(), self._frame(frame), C.c_int64(S), C.c_int(nb), _p(b), _p(nbody_w),
            C.c_int64(nrel), _p(release_t), _p(nstream), _p(stream_w0), C.c_double(t_final), C.c_double(dt0),
            C.c_double(atol), C.c_double(rtol), C.c_int64(nmax), _p(out), _p(nb_out), _p(status), _p(stats),
            C.c_int64(sys_lo), C.c_int64(hi), C.c_int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle mockstream systems failed ({rc})")
        return out, nb_out, status, stats

    def d2_dr2(self, pot, q, t=0.0):
        """c_d2_dr2 at points q (N, 3)."""
        q = _f64(q).reshape(-1, 3)
        out = np.zeros(q.shape[0])
        if self.is_ref:
            rc = self.lib.ref_d2_dr2_n(pot.packed().for_host(), C.c_double(t), _p(q), C.c_int64(q.shape[0]), _p(out))
            if rc != 0:
                raise NotImplementedError("component not available in the gala build")
        else:
            self.lib.orc_d2_dr2_n(pot.packed().for_host(), C.c_double(t), _p(q), C.c_int64(q.shape[0]), _p(out))
        return out

    def fardal_sample(self, pot, prog_w, prog_m, t, offset, draws, G, lead=True, trail=True, gala_modified=True):
        """FardalStreamDF._sample for one orbit: prog_w (ntimes, k >= 6)."""
        prog_w = _f64(prog_w)
        prog_m = _f64(prog_m)
        t = _f64(t)
        offset = np.ascontiguousarray(np.asarray(offset, dtype=np.int64))
        draws = _f64(draws).reshape(-1, 4)
        out = np.zeros((draws.shape[0], 6))
        self.lib.orc_fardal_sample(pot.packed().for_host(), C.c_int64(len(t)), _p(prog_w),
                                   C.c_int64(prog_w.shape[1]), _p(prog_m), _p(t), _p(offset), _p(draws),
                                   C.c_double(G), C.c_int(int(lead)), C.c_int(int(trail)),
                                   C.c_int(int(gala_modified)), _p(out))
        return out

    def stream_sample(self, pot, prog_w, prog_m, t, offset, kind, draws, G, lead=True, trail=True,
                      gala_modified=True):
        """The release placement of a stream DF for one orbit (kind 0 Fardal,
        1 Lagrange cloud, 2 Chen; df.pyx:410-450, 515-552, 614-700)."""
        ndraw = {0: 4, 1: 3, 2: 6}[kind]
        prog_w = _f64(prog_w)
        prog_m = _f64(prog_m)
        t = _f64(t)
        offset = np.ascontiguousarray(np.asarray(offset, dtype=np.int64))
        draws = _f64(draws).reshape(-1, ndraw)
        out = np.zeros((draws.shape[0], 6))
        self.lib.orc_stream_sample(pot.packed().for_host(), C.c_int64(len(t)), _p(prog_w),
                                   C.c_int64(prog_w.shape[1]), _p(prog_m), _p(t), _p(offset), C.c_int(kind),
                                   C.c_int(ndraw), _p(draws), C.c_double(G), C.c_int(int(lead)),
                                   C.c_int(int(trail)), C.c_int(int(gala_modified)), _p(out))
        return out

    def leapfrog_nbody(self, pot, bodies, nbody, w0, t, save_all=True):
        """leapfrog_integrate_nbody on one system: bodies (n,), w0 (n, 6).
        Returns (ntimes, n, 6) or (n, 6)."""
        b = self._bodies(bodies)
        w0 = _f64(w0)
        t = _f64(t)
        n = w0.shape[0]
        out = np.zeros((len(t), n, 6) if save_all else (n, 6))
        fn = self.lib.ref_leapfrog_nbody if self.is_ref else self.lib.orc_leapfrog_nbody
        rc = fn(pot.packed().for_host(), C.c_int(n), C.c_int(nbody), _p(b), _p(w0), _p(t), C.c_int64(len(t)),
                C.c_int(int(save_all)), _p(out))
        if rc != 0:
            raise RuntimeError(f"leapfrog n-body oracle failed ({rc})")
        return out

    def mockstream_leapfrog(self, pot, bodies, nbody_w0, full_time, stream_w0, stream_t1, tfinal, nstream):
        """mockstream_leapfrog for one progenitor system.  Returns
        (nbody_w_final (nbodies, 6), stream_w_final (ntot, 6))."""
        b = self._bodies(bodies)
        nbody_w0 = _f64(nbody_w0)
        full_time = _f64(full_time)
        stream_w0 = _f64(stream_w0).reshape(-1, 6)
        stream_t1 = _f64(stream_t1)
        nstream = np.ascontiguousarray(np.asarray(nstream, dtype=np.int32))
        nb = nbody_w0.shape[0]
        nb_out = np.zeros((nb, 6))
        st_out = np.zeros_like(stream_w0)
        fn = self.lib.ref_mockstream_leapfrog if self.is_ref else self.lib.orc_mockstream_leapfrog
        rc = fn(pot.packed().for_host(), C.c_int(nb), _p(b), _p(nbody_w0), _p(full_time), C.c_int64(len(full_time)),
                _p(stream_w0), _p(stream_t1), C.c_int64(len(stream_t1)), C.c_double(tfinal), _p(nstream), _p(nb_out),
                _p(st_out))
        if rc != 0:
            raise RuntimeError(f"leapfrog mockstream oracle failed ({rc})")
        return nb_out, st_out

    def mockstream_leapfrog_systems(self, pot, bodies, nbody_w, release_t, nstream, stream_w0, t_final, dt,
                                    sys_lo=0, sys_hi=None, nthreads=1):
        """The Leapfrog release systems of many streams (GPU layout).
        Returns (stream_w (S, ntot, 6), nbody_w_final (S, nb, 6))."""
        b = self._bodies(bodies)
        nbody_w = _f64(nbody_w)
        S, nrel, nb = nbody_w.shape[:3]
        release_t = _f64(release_t)
        nstream = np.ascontiguousarray(np.asarray(nstream, dtype=np.int32))
        stream_w0 = _f64(stream_w0)
        out = np.zeros_like(stream_w0)
        nb_out = np.zeros((S, nb, 6))
        hi = S * nrel if sys_hi is None else sys_hi
        rc = self.lib.orc_mockstream_leapfrog_systems(
            pot.packed().for_host(), C.c_int64(S), C.c_int(nb), _p(b), _p(nbody_w), C.c_int64(nrel), _p(release_t),
            _p(nstream), _p(stream_w0), C.c_double(t_final), C.c_double(dt), _p(out), _p(nb_out), C.c_int64(sys_lo),
            C.c_int64(hi), C.c_int(nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle leapfrog mockstream systems failed ({rc})")
        return out, nb_out

def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1
