"""Mock stellar streams: gala's MockStreamGenerator and FardalStreamDF on the GPU.

The generator follows gala's MockStreamGenerator.run
(src/gala/dynamics/mockstream/mockstream_generator.py:119-372):

1. the progenitor (plus optional massive bodies) is integrated over the time
   grid as a DirectNBody system with DOPRI853 (gx_nbody_dop853);
2. a stream distribution function samples release positions and velocities
   around the progenitor at each release time (FardalStreamDF._sample,
   df.pyx:363-457 -> gx_fardal_sample; the normal draws come from the DF's
   numpy random state in gala's order);
3. mockstream_dop853 (mockstream.pyx:176-303): the bodies are integrated again
   on the release grid, then every release time's system [bodies, particles
   released then] is integrated to the final time (gx_mockstream_dop853); or
   mockstream_leapfrog (mockstream.pyx:442-610): the bodies' Leapfrog trajectory
   on the full grid gives their state at each release time, and every release
   system takes round((t_final - t_release) / dt) Leapfrog steps
   (gx_mockstream_leapfrog, or its FP32-compensated form with
   ``precision="fp32c"``).  With DOP853, ``precision="fp32c"`` runs the release
   systems with FP32 stages and forces and FP64 step control
   (gx_mockstream_dop853_fp32; tolerances of ~1e-8 relative and looser); the
   bodies' own integration stays FP64.

With ``output_every`` (DOP853 only, as in gala) the stream is made by
mockstream_dop853_animate (mockstream.pyx:306-440) instead of step 3: one
system per stream that holds the bodies and every particle released so far,
stepped interval by interval over the whole grid (gx_mockstream_dop853_animate),
with snapshots written to an HDF5 file in gala's layout.

``run`` makes one stream with gala's signature and return values.
``run_batch`` makes many independent streams (one progenitor each, all on one
time grid) in the same three launches; stream s consumes the DF's random draws
after streams 0..s-1, as consecutive ``run`` calls with one DF would.
"""
from __future__ import annotations

import warnings

import numpy as np

from . import _abi, units
from .dynamics import PhaseSpacePosition, _galactic, _h5_open, quantity_from_hdf5, quantity_to_hdf5
from .hamiltonian import Hamiltonian, StaticFrame, rotate_frame
from .integrate import DOPRI853Integrator, LeapfrogIntegrator, get_integrator, parse_time_specification
from .nbody import DirectNBody, bodies_to_device, integrate_systems, integrate_systems_leapfrog, pack_bodies
from .potential import PotentialBase
from ._trace import traced

__all__ = ["MockStream", "BaseStreamDF", "FardalStreamDF", "StreaklineStreamDF", "LagrangeCloudStreamDF",
           "ChenStreamDF", "MockStreamGenerator", "MockStreamBatch"]


class MockStream(PhaseSpacePosition):
    """Stream particles with their release times and tails ('t' trailing, 'l'
    leading) (src/gala/dynamics/mockstream/core.py:12-47)."""

    def __init__(self, pos, vel=None, frame=None, release_time=None, lead_trail=None, copy=True):
        super().__init__(pos=pos, vel=vel, frame=frame, copy=copy)
        n = self.pos.shape[1] if self.pos.ndim > 1 else 1
        if release_time is not None:
            release_time = np.asarray(release_time, dtype=np.float64)
            if len(release_time) != n:
                raise ValueError("shape mismatch: input release time array must have the same shape as the input "
                                 f"phase-space data, minus the component dimension. expected {n}, got "
                                 f"{len(release_time)}")
        self.release_time = release_time
        if lead_trail is not None:
            lead_trail = np.array(lead_trail)
            if len(lead_trail) != n:
                raise ValueError("shape mismatch: input leading/trailing array must have the same shape as the "
                                 f"input phase-space data, minus the component dimension. expected {n}, got "
                                 f"{len(lead_trail)}")
        self.lead_trail = lead_trail

    # -- HDF5 (MockStream.to_hdf5 / from_hdf5, mockstream/core.py:106-150) -----
    def _write_hdf5(self, f):
        super()._write_hdf5(f)
        if self.release_time is not None and len(self.release_time):
            quantity_to_hdf5(f, "release_time", self.release_time, "Myr")
        if self.lead_trail is not None:
            f["lead_trail"] = np.asarray(self.lead_trail).astype("S1")

    @classmethod
    def from_hdf5(cls, f):
        f, close = _h5_open(f, "r")
        try:
            obj = PhaseSpacePosition.from_hdf5(f)
            t = quantity_from_hdf5(f["release_time"], "time") if "release_time" in f else None
            lt = f["lead_trail"][()] if "lead_trail" in f else None
        finally:
            if close:
                f.close()
        if lt is not None:
            lt = np.array([x.decode() if isinstance(x, bytes) else str(x) for x in np.ravel(lt)], dtype="U1")
        return cls(pos=obj.pos, vel=obj.vel, frame=obj.frame, release_time=t, lead_trail=lt)


def split_releases(nstream, cap):
    """Release systems of at most ``cap`` particles: a release with more is cut
    into consecutive groups at the same time, each integrated with its own copy
    of the bodies.  Returns (src, sizes): the release each group belongs to and
    its particle count, in row order.  With Leapfrog this is exact -- the
    particles are test particles on fixed steps, so the bodies' trajectory and
    each particle's are the same in any grouping."""
    src, sizes = [], []
    for i, n in enumerate(np.asarray(nstream, dtype=np.int64)):
        n = int(n)
        if n <= cap:
            src.append(i)
            sizes.append(n)
            continue
        for k in range(0, n, cap):
            src.append(i)
            sizes.append(min(cap, n - k))
    return np.array(src, dtype=np.int64), np.array(sizes, dtype=np.int64)


class BaseStreamDF:
    """Release distribution of stream particles (df.pyx:34-121)."""

    def __init__(self, lead=True, trail=True, random_state=None):
        self._lead = int(lead)
        self._trail = int(trail)
        if random_state is None:
            random_state = np.random.RandomState()
        self.random_state = random_state
        if not self.lead and not self.trail:
            raise ValueError("You must generate either leading or trailing tails (or both!)")

    @property
    def lead(self):
        return self._lead

    @property
    def trail(self):
        return self._trail

    # -- layout of the released particles (df.pyx:194-231) ----------------------
    def release_counts(self, ntimes, release_every=1, n_particles=1):
        """Particles per tail at each time: ``n_particles`` every ``release_every``
        steps, or a per-time array (BaseStreamDF.sample, df.pyx:197-207)."""
        if np.iterable(n_particles):
            n = np.array(n_particles).astype("i4")
            if len(n) != ntimes:
                raise ValueError("If passing in an array n_particles, its shape must match the number of timesteps "
                                 "in the progenitor orbit.")
            return n
        n = np.zeros(ntimes, dtype="i4")
        n[::release_every] = int(n_particles)
        return n

    # kind of release placement of the GPU sampler, and draws per particle
    _KIND, _NDRAW = 0, 4

    def _draws(self, n_rows):
        raise NotImplementedError

    # -- sampling ---------------------------------------------------------------
    def sample_device(self, potential, prog_w, prog_t, prog_m, counts, stream=None, frame=None):
        """Release states for n_streams progenitor orbits on one time grid.

        prog_w : CUDA tensor (n_streams, ntimes, k >= 6): progenitor x, v first
        prog_t : (ntimes,) float64; prog_m : (n_streams, ntimes)
        counts : (ntimes,) particles per tail
        frame  : the frame of prog_w and of the result; a rotating frame is
                 sampled in the static frame, the orbit turned there at its times
                 and every particle back at its release time (df.pyx:172-233)
        Returns (w (n_streams, n_rows, 6) CUDA tensor, release_time (n_rows,),
        lead_trail (n_rows,), offset (ntimes + 1,) int64).
        """
        import torch

        from ._device import as_device_f64, ptr, stream_handle

        rotating = frame is not None and not isinstance(frame, StaticFrame)
        if rotating:
            td = torch.as_tensor(np.asarray(prog_t, dtype=np.float64), device=prog_w.device)
            prog_w = rotate_frame(prog_w[..., :6], td[None, :], frame.Omega, to_rotating=False)
        ns, ntimes = int(prog_w.shape[0]), int(prog_w.shape[1])
        ntail = self._lead + self._trail
        counts = np.asarray(counts, dtype=np.int64)
        offset = np.concatenate([[0], np.cumsum(ntail * counts)]).astype(np.int64)
        n_rows = int(offset[-1])
        prog_m = np.broadcast_to(np.asarray(prog_m, dtype=np.float64), (ns, ntimes))
        if np.any((counts > 0)[None, :] & (prog_m == 0)):
            raise NotImplementedError("a zero progenitor mass at a release time is not supported")
        draws = (np.stack([self._draws(n_rows) for _ in range(ns)]) if ns
                 else np.zeros((0, n_rows, self._NDRAW)))
        dev = prog_w.device
        out = torch.empty((ns, n_rows, 6), dtype=torch.float64, device=dev)
        pw = prog_w.contiguous()
        dd = as_device_f64(draws, dev)
        md = as_device_f64(np.ascontiguousarray(prog_m), dev)
        td = as_device_f64(prog_t, dev)
        od = torch.from_numpy(offset).to(dev)
        _abi.call("gx_stream_sample", potential.packed().for_device(), ns, ntimes, ptr(pw), int(pw.shape[2]),
                  ptr(md), ptr(td), ptr(od), n_rows, self._KIND, ptr(dd), float(potential.G), self._lead,
                  self._trail, getattr(self, "_gala_modified", 0), ptr(out), stream_handle(stream))
        release_time = np.repeat(np.asarray(prog_t, dtype=np.float64), ntail * counts)
        if rotating:
            out = rotate_frame(out, torch.from_numpy(release_time).to(dev)[None, :], frame.Omega, to_rotating=True)
        lt = []
        for n in counts:
            if self._trail:
                lt += ["t"] * int(n)
            if self._lead:
                lt += ["l"] * int(n)
        return out, release_time, np.array(lt, dtype="U1"), offset

    def sample(self, prog_orbit, prog_mass, hamiltonian=None, release_every=1, n_particles=1):
        """Stream initial conditions around a progenitor orbit (df.pyx:125-242)."""
        from ._device import as_device_f64, require_cuda

        if getattr(prog_orbit, "hamiltonian", None) is not None:
            H = prog_orbit.hamiltonian
        elif hamiltonian is not None:
            H = hamiltonian if isinstance(hamiltonian, Hamiltonian) else Hamiltonian(hamiltonian)
        else:
            raise ValueError("a Hamiltonian is needed to sample stream particles")
        x = np.asarray(prog_orbit.xyz, dtype=np.float64)
        v = np.asarray(prog_orbit.v_xyz, dtype=np.float64)
        t = np.asarray(prog_orbit.t, dtype=np.float64)
        ntimes = len(t)
        prog_w = np.ascontiguousarray(np.vstack([x, v]).T.reshape(1, ntimes, 6))
        m = np.squeeze(_galactic(prog_mass, "Msun"))
        m = np.full(ntimes, float(m)) if m.shape == () else m
        counts = self.release_counts(ntimes, release_every, n_particles)
        dev = require_cuda()
        w, rt, lt, _ = self.sample_device(H.potential, as_device_f64(prog_w, dev), t, m[None, :], counts,
                                          frame=H.frame)
        w = w[0].cpu().numpy()
        return MockStream(pos=w[:, :3].T, vel=w[:, 3:].T, frame=H.frame, release_time=rt, lead_trail=lt)


class FardalStreamDF(BaseStreamDF):
    """Fardal et al. (2015) release distribution with gala's parameters
    (FardalStreamDF, df.pyx:300-457)."""

    def __init__(self, gala_modified=None, lead=True, trail=True, random_state=None):
        super().__init__(lead=lead, trail=trail, random_state=random_state)
        if gala_modified is None:
            warnings.warn(
                "The parameter values of the FardalStreamDF have been updated (fixed) to match the parameter "
                "values in the final published version of Fardal+2015. For now, this class uses the Gala modified "
                "parameter values. To use the Fardal+2015 parameters now, set gala_modified=False. To continue to "
                "use the Gala modified parameter values, set gala_modified=True.", FutureWarning)
            gala_modified = True
        self._gala_modified = int(gala_modified)

    def _k(self):
        """(k_mean, k_disp) of the four sampled quantities: R, z, v_t, v_z (df.pyx:390-405)."""
        kvt_fardal = 0.4
        mean = np.array([2.0, 0.0, 0.3, 0.0])
        disp = np.array([0.5 if self._gala_modified else 0.4, 0.5,
                         0.5 if self._gala_modified else kvt_fardal, 0.5])
        return mean, disp

    def _draws(self, n_rows):
        """The four normal draws of n_rows particles, in gala's call order: per
        particle kx, z, v_t, v_z (df.pyx:416-423).  One vectorised call with
        per-element loc/scale consumes the random state exactly as the scalar
        calls do."""
        mean, disp = self._k()
        if n_rows == 0:
            return np.zeros((0, 4))
        loc = np.tile(mean, n_rows)
        scale = np.tile(disp, n_rows)
        return np.asarray(self.random_state.normal(loc, scale), dtype=np.float64).reshape(n_rows, 4)

class StreaklineStreamDF(FardalStreamDF):
    """Kuepper et al. (2012) streakline release (StreaklineStreamDF,
    df.pyx:242-319): every particle at -/+ r_J along the satellite-frame x axis
    (trailing / leading) with -/+ v_J along its y axis, nothing drawn.  That is
    the Fardal placement with k_R = 1, k_z = 0, k_vt = 1, k_vz = 0, so the same
    GPU sampler runs it with those constants in place of the normal draws; the
    random state is not consumed, as in gala."""

    def __init__(self, lead=True, trail=True, random_state=None):
        BaseStreamDF.__init__(self, lead=lead, trail=trail, random_state=random_state)
        self._gala_modified = 1  # multiplies v_t by k_R = 1: no effect

    def _k(self):
        return np.array([1.0, 0.0, 1.0, 0.0]), np.zeros(4)

    def _draws(self, n_rows):
        return np.tile(np.array([1.0, 0.0, 1.0, 0.0]), (n_rows, 1))


class LagrangeCloudStreamDF(BaseStreamDF):
    """Lagrange-cloud stripping (Gibbons et al. 2014, as modified by Erkal et al.
    2019; LagrangeCloudStreamDF, df.pyx:460-555): every particle at -/+ r_J
    along the satellite-frame x axis, its satellite-frame velocity three normal
    draws of dispersion v_disp (km/s), drawn per particle in gala's order."""

    _KIND, _NDRAW = 1, 3

    def __init__(self, v_disp, lead=True, trail=True, random_state=None):
        super().__init__(lead=lead, trail=trail, random_state=random_state)
        self.v_disp = float(_galactic(v_disp, "km / s"))  # km/s, as gala's parameter is given
        self._v_disp = self.v_disp * units.KMS_TO_KPC_MYR

    def _draws(self, n_rows):
        if n_rows == 0:
            return np.zeros((0, 3))
        return np.asarray(self.random_state.normal(0, self._v_disp, size=(n_rows, 3)), dtype=np.float64)


class ChenStreamDF(BaseStreamDF):
    """Chen et al. (2024) release (ChenStreamDF, df.pyx:557-703): per particle one
    multivariate-normal sample of (r/r_J, phi, theta, v/v_esc, alpha, beta) with
    gala's mean and covariance; position Dr = r r_J at angles (phi, theta),
    velocity Dv = v sqrt(2 G m / Dr) at angles (alpha, beta); the leading tail
    turns phi and alpha by pi.  The samples are drawn one particle at a time, as
    gala does, so the random state is consumed identically."""

    _KIND, _NDRAW = 2, 6

    _MEAN = np.array([1.6, -30.0, 0.0, 1.0, 20.0, 0.0])

    @staticmethod
    def _cov():
        cov = np.zeros((6, 6))
        cov[0, 0], cov[1, 1], cov[2, 2], cov[3, 3], cov[4, 4], cov[5, 5] = 0.1225, 529.0, 144.0, 0.0, 400.0, 484.0
        cov[0, 4] = cov[4, 0] = -4.9
        return cov

    def _draws(self, n_rows):
        cov = self._cov()
        out = np.zeros((n_rows, 6))
        for r in range(n_rows):
            out[r] = self.random_state.multivariate_normal(self._MEAN, cov)
        return out


class MockStreamBatch:
    """Result of MockStreamGenerator.run_batch: device tensors for many streams.

    stream_w     (n_streams, n_particles, 6) particles at the final time
    nbody_w      (n_streams, nbodies, 6) bodies at the final time
    release_time (n_particles,), lead_trail (n_particles,)
    status       (n_streams, n_release) dop853() code of each release system
    stats        (n_streams, n_release, 4) or None: nfcn, nstep, naccpt, nrejct
    With output_every (the animate mode) status is (n_streams, ntimes), one code
    per interval of the grid, stats (n_streams, 4) summed over the intervals, and
    snapshots     (n_streams, 6, n_output, nbodies + n_particles) the bodies and
                  particles at snapshot_t, NaN for particles not yet released
    snapshot_t    (n_output,)
    """

    def __init__(self, stream_w, nbody_w, release_time, lead_trail, status, stats, frame, t, snapshots=None,
                 snapshot_t=None):
        self.stream_w = stream_w
        self.nbody_w = nbody_w
        self.release_time = release_time
        self.lead_trail = lead_trail
        self.status = status
        self.stats = stats
        self.frame = frame
        self.t = t
        self.snapshots = snapshots
        self.snapshot_t = snapshot_t

    @property
    def n_streams(self):
        return int(self.stream_w.shape[0])

    def stream(self, s):
        w = self.stream_w[s].cpu().numpy()
        return MockStream(pos=w[:, :3].T, vel=w[:, 3:].T, frame=self.frame, release_time=self.release_time,
                          lead_trail=self.lead_trail)

    def nbody(self, s):
        w = self.nbody_w[s].cpu().numpy()
        return PhaseSpacePosition(pos=w[:, :3].T, vel=w[:, 3:].T, frame=self.frame)

    def write_snapshots(self, s, filename):
        """Stream s's snapshots as mockstream_dop853_animate writes them
        (mockstream.pyx:107-175, 393-430): groups ``stream`` and ``nbody``, each
        with ``pos`` (3, n_output, N) and ``vel`` datasets (NaN where a particle
        is not yet released) and a ``time`` dataset, all with a ``unit``
        attribute.  ``filename`` may be a name or an open file."""
        if self.snapshots is None:
            raise ValueError("this batch holds no snapshots (run with output_every)")
        nb = int(self.nbody_w.shape[1])
        snap = self.snapshots[s].cpu().numpy()
        f, close = _h5_open(filename, "w")
        try:
            for name, part in (("stream", snap[:, :, nb:]), ("nbody", snap[:, :, :nb])):
                g = f.create_group(name)
                quantity_to_hdf5(g, "pos", part[:3], "kpc")
                quantity_to_hdf5(g, "vel", part[3:], "kpc / Myr")
                quantity_to_hdf5(g, "time", np.asarray(self.snapshot_t, dtype=np.float64), "Myr")
        finally:
            if close:
                f.close()


class MockStreamGenerator:
    """Generate mock streams with a release DF in a Hamiltonian
    (src/gala/dynamics/mockstream/mockstream_generator.py:20-118)."""

    def __init__(self, df, hamiltonian, progenitor_potential=None):
        if not isinstance(df, BaseStreamDF):
            raise TypeError("The input distribution function (DF) instance must be a BaseStreamDF subclass "
                            f"instance, not {type(df)}")
        self.df = df
        self.hamiltonian = hamiltonian if isinstance(hamiltonian, Hamiltonian) else Hamiltonian(hamiltonian)
        if progenitor_potential is not None and not isinstance(progenitor_potential, PotentialBase):
            raise TypeError("If specified, the progenitor_potential must be a potential class instance.")
        self.self_gravity = progenitor_potential is not None
        self.progenitor_potential = progenitor_potential

    def _get_nbody(self, prog_w0, nbody):
        """The progenitor plus optional extra bodies as one DirectNBody (:76-117)."""
        if nbody is not None:
            if nbody.external_potential is not self.hamiltonian.potential:
                raise ValueError("The external potential of the input nbody instance must match the potential of "
                                 "the mock stream input hamiltonian!")
            w0 = PhaseSpacePosition(
                pos=np.column_stack([np.reshape(prog_w0.xyz, (3, 1)), np.reshape(nbody.w0.xyz, (3, -1))]),
                vel=np.column_stack([np.reshape(prog_w0.v_xyz, (3, 1)), np.reshape(nbody.w0.v_xyz, (3, -1))]))
            pps = [self.progenitor_potential, *nbody.particle_potentials]
        else:
            w0 = prog_w0
            pps = [self.progenitor_potential]
        return DirectNBody(w0=w0, particle_potentials=pps, external_potential=self.hamiltonian.potential,
                           frame=self.hamiltonian.frame)

    @staticmethod
    def _dop_kwargs(Integrator_kwargs):
        kw = dict(Integrator_kwargs or {})
        err_if_fail = int(kw.pop("err_if_fail", 1))
        kw.pop("log_output", None)
        kw.pop("progress", None)
        extra = set(kw) - {"atol", "rtol", "nmax", "dt_max"}
        if extra:
            raise TypeError(f"unexpected Integrator_kwargs {sorted(extra)}")
        return dict(atol=float(kw.get("atol", 1e-10)), rtol=float(kw.get("rtol", 1e-10)),
                    nmax=int(kw.get("nmax", 0)), dt_max=float(kw.get("dt_max", 0.0))), err_if_fail

    def _generate(self, bodies, body_w0, prog_m, t, counts, dop, err_if_fail, return_stats=False, stream=None,
                  integrator="dop853", precision="fp64", output_every=None):
        """The three stages for n_streams systems.

        bodies  : BODY_DTYPE (S, nb), progenitor first, massive bodies before null ones
        body_w0 : (S, nb, 6) bodies at t[0]
        prog_m  : (S, ntimes) progenitor mass along the orbit grid (increasing time)
        counts  : (ntimes,) particles per tail on the orbit grid
        """
        import torch

        from ._device import ptr, require_cuda, stream_handle

        H = self.hamiltonian
        rotating = not isinstance(H.frame, StaticFrame)
        if rotating and integrator == "leapfrog":
            raise TypeError(f"Leapfrog integration is currently only supported for StaticFrame, not "
                            f"{H.frame.__class__.__name__}")
        if rotating and precision == "fp32c":
            raise NotImplementedError("the FP32 DOP853 forms of mock streams run in a static frame")
        dev = require_cuda()
        S, nb = bodies.shape

        def check(status, what):
            res = status.cpu().numpy().ravel()
            bad = res[res < 0]
            if bad.size and err_if_fail == 1:
                raise RuntimeError(f"Integration failed with code {int(bad[0])}")

        leapfrog = integrator == "leapfrog"
        if precision not in ("fp64", "fp32c"):
            raise ValueError("precision must be 'fp64' or 'fp32c'")

        # 1. the bodies over the requested grid (DirectNBody.integrate_orbit)
        if leapfrog:
            orbit = integrate_systems_leapfrog(H, bodies, body_w0, t, save_all=True, stream=stream)
        else:
            orbit, st = integrate_systems(H, bodies, body_w0, t, save_all=True, nstiff=-1, stream=stream, **dop)
            check(st, "nbody")
        forward = not (t[1] < t[0])
        if forward:
            orbit_t = t
            nbody0 = torch.as_tensor(body_w0, dtype=torch.float64, device=dev)
        else:  # the grid runs backwards: the stream is made forwards from the past (:237-250)
            orbit = torch.flip(orbit, dims=[1])
            orbit_t = t[::-1].copy()
            nbody0 = orbit[:, 0].contiguous()

        # 2. release states from the progenitor orbit (body 0)
        prog_w = orbit.reshape(S, len(orbit_t), nb * 6)
        stream_w0, release_time, lead_trail, _ = self.df.sample_device(H.potential, prog_w, orbit_t, prog_m, counts,
                                                                     stream=stream, frame=H.frame)
        ntail = self.df.lead + self.df.trail
        if output_every is not None:
            return self._animate(bodies, nbody0, orbit_t, ntail * counts, stream_w0, release_time, lead_trail, dop,
                                 output_every, check, return_stats, stream, precision)

        # 3. release grid: times that release particles, plus the first (:271-283)
        rel_idx = np.nonzero(counts > 0)[0]
        if 0 not in rel_idx:
            rel_idx = np.insert(rel_idx, 0, 0)
        time = np.ascontiguousarray(orbit_t[rel_idx])
        nstream = (ntail * counts[rel_idx]).astype(np.int64)
        rel_off = np.concatenate([[0], np.cumsum(nstream)]).astype(np.int64)
        n_rows = int(rel_off[-1])
        max_per = int(nstream.max()) if nstream.size else 0
        if leapfrog:
            return self._release_leapfrog(bodies, orbit, nbody0, orbit_t, forward, time, nstream, rel_off, n_rows,
                                          max_per, stream_w0, release_time, lead_trail, precision, stream)
        if forward and len(rel_idx) == len(orbit_t):
            nbody_w = orbit  # the same dop853_helper call on the same grid (mockstream.pyx:245-255)
        else:
            nbody_w, st = integrate_systems(H, bodies, nbody0, time, save_all=True, nstiff=-1, stream=stream,
                                            **dop)
            check(st, "nbody")
        # releases of more than 32 - nb particles are systems wider than a warp:
        # the 32-lane kernel marks them (-1) and the CTA-per-system kernel then
        # integrates each as the one system gala makes of it (every release, when
        # the bodies alone fill a warp); releases of no particle are skipped, as
        # gala skips them
        wide_rel = np.nonzero((nb + nstream > 32) & (nstream > 0))[0]
        max_group = max(0, min(max_per, 32 - nb))
        n_rel = len(time)
        stream_out = torch.empty((S, n_rows, 6), dtype=torch.float64, device=dev)
        nbody_out = torch.empty((S, nb, 6), dtype=torch.float64, device=dev)
        status = torch.zeros((S, n_rel), dtype=torch.int32, device=dev)
        stats = torch.zeros((S, n_rel, 4), dtype=torch.int64, device=dev) if return_stats else None
        counter = torch.zeros(1, dtype=torch.int64, device=dev)
        bd = bodies_to_device(bodies, dev)
        td = torch.from_numpy(time).to(dev)
        od = torch.from_numpy(rel_off).to(dev)
        dt0 = float(time[1] - time[0])
        if precision == "fp32c":
            # FP32 stages and forces with FP64 step control (gx_mockstream_dop853_fp32)
            if wide_rel.size:
                raise NotImplementedError("the FP32 DOP853 release systems fill at most 32 lanes; release fewer "
                                          "particles per time or use precision='fp64'")
            if not isinstance(H.frame, StaticFrame):
                raise NotImplementedError("the FP32 DOP853 release systems run in a static frame")
            _abi.call("gx_mockstream_dop853_fp32", H.potential.packed().for_device(), S, nb, ptr(bd), ptr(nbody_w),
                      n_rel, ptr(td), ptr(od), max_group, ptr(stream_w0), n_rows, float(orbit_t[-1]), dt0,
                      dop["atol"], dop["rtol"], dop["nmax"], ptr(stream_out), ptr(nbody_out), ptr(status),
                      ptr(stats) if stats is not None else None, ptr(counter), stream_handle(stream))
            check(status, "stream")
            return MockStreamBatch(stream_out, nbody_out, release_time, lead_trail, status, stats, H.frame, orbit_t)
        if nb < 32:
            _abi.call("gx_mockstream_dop853", H.potential.packed().for_device(), H._frame_ref(), S, nb, ptr(bd),
                      ptr(nbody_w), n_rel, ptr(td), ptr(od), max_group, ptr(stream_w0), n_rows, float(orbit_t[-1]),
                      dt0, dop["atol"], dop["rtol"], dop["nmax"], ptr(stream_out), ptr(nbody_out),
                      ptr(status), ptr(stats) if stats is not None else None, ptr(counter), stream_handle(stream))
        if wide_rel.size:
            sys_ids = (wide_rel[:, None] * S + np.arange(S)[None, :]).ravel().astype(np.int64)
            members = nb + int(nstream[wide_rel].max())
            nbytes = int(_abi.load().gx_mockstream_wide_scratch_bytes(len(sys_ids), members))
            scratch = torch.empty(nbytes // 8, dtype=torch.float64, device=dev)
            sd = torch.from_numpy(sys_ids).to(dev)
            _abi.call("gx_mockstream_dop853_wide", H.potential.packed().for_device(), H._frame_ref(), S, nb,
                      ptr(bd), ptr(nbody_w), n_rel, ptr(td), ptr(od), ptr(stream_w0), n_rows, float(orbit_t[-1]),
                      dt0, dop["atol"], dop["rtol"], dop["nmax"], ptr(sd), len(sys_ids), members, ptr(scratch),
                      nbytes, ptr(stream_out), ptr(nbody_out), ptr(status),
                      ptr(stats) if stats is not None else None, stream_handle(stream))
        check(status, "stream")
        return MockStreamBatch(stream_out, nbody_out, release_time, lead_trail, status, stats, H.frame, orbit_t)

    def _animate(self, bodies, nbody0, orbit_t, nstream, stream_w0, release_time, lead_trail, dop, output_every,
                 check, return_stats, stream, precision="fp64"):
        """mockstream_dop853_animate's stage (mockstream.pyx:306-440) for every
        stream: nstream (ntimes,) particles released at each grid time.  With
        precision="fp32c" the systems run with FP32 stages and forces and FP64
        step control (gx_mockstream_dop853_animate_fp32)."""
        import torch

        from ._device import ptr, stream_handle

        H = self.hamiltonian
        S, nb = bodies.shape
        dev = nbody0.device
        ntimes = len(orbit_t)
        nstream = np.ascontiguousarray(nstream, dtype=np.int32)
        n_rows = int(nstream.sum())
        M = nb + n_rows
        lib = _abi.load()
        n_out = int(lib.gx_mockstream_animate_snapshots(ntimes, output_every))
        nbytes = int(lib.gx_mockstream_wide_scratch_bytes(S, M))
        scratch = torch.empty(nbytes // 8, dtype=torch.float64, device=dev)
        snap = torch.empty((S, 6, n_out, M), dtype=torch.float64, device=dev)
        w_out = torch.empty((S, M, 6), dtype=torch.float64, device=dev)
        status = torch.zeros((S, ntimes), dtype=torch.int32, device=dev)
        stats = torch.zeros((S, 4), dtype=torch.int64, device=dev) if return_stats else None
        bd = bodies_to_device(bodies, dev)
        td = torch.from_numpy(np.ascontiguousarray(orbit_t, dtype=np.float64)).to(dev)
        nd = torch.from_numpy(nstream).to(dev)
        nbody0 = nbody0.reshape(S, nb, 6).contiguous()
        common = (S, nb, ptr(bd), ptr(nbody0), ntimes, ptr(td), float(orbit_t[1] - orbit_t[0]), ptr(nd),
                  ptr(stream_w0), n_rows, int(output_every), dop["atol"], dop["rtol"], dop["nmax"], ptr(scratch),
                  nbytes, ptr(snap), ptr(w_out), ptr(status), ptr(stats) if stats is not None else None,
                  stream_handle(stream))
        if precision == "fp32c":
            _abi.call("gx_mockstream_dop853_animate_fp32", H.potential.packed().for_device(), *common)
        else:
            _abi.call("gx_mockstream_dop853_animate", H.potential.packed().for_device(), H._frame_ref(), *common)
        check(status, "stream")
        idx = [0] + [i for i in range(1, ntimes) if i % output_every == 0 or i == ntimes - 1]
        return MockStreamBatch(w_out[:, nb:], w_out[:, :nb], release_time, lead_trail, status, stats, H.frame,
                               orbit_t, snapshots=snap, snapshot_t=np.asarray(orbit_t)[idx])

    def _release_leapfrog(self, bodies, orbit, nbody0, orbit_t, forward, time, nstream, rel_off, n_rows, max_per,
                          stream_w0, release_time, lead_trail, precision, stream):
        """mockstream_leapfrog's release stage (mockstream.pyx:524-593)."""
        import torch

        from ._device import ptr, stream_handle

        H = self.hamiltonian
        S, nb = bodies.shape
        dev = orbit.device
        cap = 8 - nb  # the kernel's systems hold 8 bodies and particles
        if cap < 1:
            raise NotImplementedError(f"{nb} bodies exceed the 8-body Leapfrog system")
        n_rel0, src = len(time), None
        if max_per > cap:  # larger releases in groups at the same time (exact, see split_releases)
            src, sizes = split_releases(nstream, cap)
            time, nstream = time[src], sizes
            rel_off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
            max_per = int(sizes.max())
        # the bodies' trajectory on the full grid; the same call as stage 1 when the grid runs forwards
        traj = orbit if forward else integrate_systems_leapfrog(H, bodies, nbody0, orbit_t, save_all=True,
                                                                stream=stream)
        dt = float(orbit_t[1] - orbit_t[0])
        idx = np.trunc((time - orbit_t[0]) / dt + 0.5).astype(np.int64)  # mockstream.pyx:537
        nbody_w = traj[:, torch.from_numpy(idx).to(dev)].contiguous()
        n_rel = len(time)
        stream_out = torch.empty((S, n_rows, 6), dtype=torch.float64, device=dev)
        nbody_out = torch.empty((S, nb, 6), dtype=torch.float64, device=dev)
        status = torch.zeros((S, n_rel), dtype=torch.int32, device=dev)
        bd = bodies_to_device(bodies, dev)
        td = torch.from_numpy(np.ascontiguousarray(time)).to(dev)
        od = torch.from_numpy(rel_off).to(dev)
        name = "gx_mockstream_leapfrog" if precision == "fp64" else "gx_mockstream_leapfrog_fp32"
        _abi.call(name, H.potential.packed().for_device(), S, nb, ptr(bd), ptr(nbody_w), n_rel, ptr(td), ptr(od),
                  max_per, ptr(stream_w0), n_rows, float(orbit_t[-1]), dt, ptr(stream_out), ptr(nbody_out),
                  ptr(status), stream_handle(stream))
        if src is not None:
            # one status per release, as documented: the worst code over its groups
            idx = torch.from_numpy(src).to(dev).expand(S, -1)
            status = torch.ones((S, n_rel0), dtype=torch.int32, device=dev).scatter_reduce(
                1, idx, status, reduce="amin", include_self=False)
        res = status.cpu().numpy()
        if np.any(res < 0):
            raise RuntimeError(f"release systems rejected: {int(np.sum(res < 0))}")
        return MockStreamBatch(stream_out, nbody_out, release_time, lead_trail, status, None, H.frame, orbit_t)

    @traced("mockstream_run")
    def run(self, prog_w0, prog_mass, nbody=None, release_every=1, n_particles=1, output_every=None,
            output_filename=None, check_filesize=True, overwrite=False, progress=False, Integrator=None,
            Integrator_kwargs=None, **time_spec):
        """One mock stream; returns (stream MockStream, nbody PhaseSpacePosition) (:119-372)."""
        Integrator = get_integrator(DOPRI853Integrator if Integrator is None else Integrator)
        if Integrator not in (DOPRI853Integrator, LeapfrogIntegrator):
            raise ValueError("Currently, only the DOPRI853Integrator and LeapfrogIntegrator are supported for mock "
                             "stream generation.")
        kw_in = dict(Integrator_kwargs or {})
        precision = kw_in.pop("precision", "fp64")
        t = np.ascontiguousarray(parse_time_specification(self.hamiltonian.units, **time_spec), dtype=np.float64)
        if output_every is not None:
            if output_filename is None:
                raise ValueError("If output_every is specified, you must also pass in a filename to store the "
                                 "snapshots in")
            output_every = self._check_animate(output_every, Integrator, precision)
            self._check_output_file(output_filename, overwrite, check_filesize, output_every, t, release_every,
                                    n_particles)
        prog_nbody = self._get_nbody(prog_w0, nbody)
        idx, n_massive = prog_nbody._order()
        if not np.array_equal(idx, np.arange(len(idx))):
            raise NotImplementedError("null-potential bodies must come after the massive ones")
        nb = len(prog_nbody.particle_potentials)
        bodies = pack_bodies([prog_nbody.particle_potentials])
        m = np.squeeze(_galactic(prog_mass, "Msun"))
        m = np.full(len(t), float(m)) if m.shape == () else m
        counts = self.df.release_counts(len(t), release_every, n_particles)
        dop, err_if_fail = self._dop_kwargs(kw_in if Integrator is DOPRI853Integrator else {})
        res = self._generate(bodies, prog_nbody._c_w0.reshape(1, nb, 6), m[None, :], t, counts, dop, err_if_fail,
                             integrator="leapfrog" if Integrator is LeapfrogIntegrator else "dop853",
                             precision=precision, output_every=output_every)
        if output_every is not None:
            res.write_snapshots(0, output_filename)
        return res.stream(0), res.nbody(0)

    @staticmethod
    def _check_animate(output_every, Integrator, precision):
        """The animate mode's integrator checks (mockstream_generator.py:318-336)."""
        if Integrator is LeapfrogIntegrator:
            raise NotImplementedError("Animation output for LeapfrogIntegrator is not implemented")
        if precision not in ("fp64", "fp32c"):
            raise ValueError("precision must be 'fp64' or 'fp32c'")
        output_every = int(output_every)
        if output_every < 1:
            raise ValueError("output_every must be a positive integer")
        return output_every

    def _check_output_file(self, output_filename, overwrite, check_filesize, output_every, t, release_every,
                           n_particles):
        """The snapshot file's checks, before any integration (_init_hdf5_file,
        mockstream.pyx:116-134)."""
        import os

        if not isinstance(output_filename, (str, os.PathLike)):
            return  # an open file or group
        n_out = (len(t) - 1) // output_every + 1 + int((len(t) - 1) % output_every != 0)
        total = (self.df.lead + self.df.trail) * int(self.df.release_counts(len(t), release_every,
                                                                            n_particles).sum())
        if total * n_out * 8 >= 8e9 and check_filesize:
            warnings.warn("Estimated mockstream output file is expected to be >8 GB in size! If you're sure, turn "
                          "this warning off with `check_filesize=False`")
        if os.path.exists(output_filename) and not overwrite:
            raise OSError(f"Mockstream output file {output_filename} already exists! Use overwrite=True to "
                          "overwrite the file.")

    @traced("mockstream_run_batch")
    def run_batch(self, prog_w0, prog_mass, progenitor_potentials=None, release_every=1, n_particles=1,
                  Integrator=None, Integrator_kwargs=None, return_stats=False, stream=None, output_every=None,
                  **time_spec):
        """Many independent streams on one time grid (no extra bodies).

        prog_w0  : (6, S) progenitor phase-space positions (numpy)
        prog_mass: (S,) or (S, ntimes) masses passed to the DF
        progenitor_potentials : list of S potentials (or None: the generator's
                   progenitor_potential for every stream)
        output_every : snapshots every output_every grid steps (the animate
                   mode, DOP853): kept on the device in the returned batch
                   (``snapshots``, ``snapshot_t``; ``write_snapshots`` writes
                   one stream's file)
        Returns a MockStreamBatch of device tensors.
        """
        t = np.ascontiguousarray(parse_time_specification(self.hamiltonian.units, **time_spec), dtype=np.float64)
        w0 = np.asarray(prog_w0, dtype=np.float64)
        if w0.ndim != 2 or w0.shape[0] != 6:
            raise ValueError(f"prog_w0 must have shape (6, n_streams), got {w0.shape}")
        S = w0.shape[1]
        if progenitor_potentials is None:
            progenitor_potentials = [self.progenitor_potential] * S
        if len(progenitor_potentials) != S:
            raise ValueError("one progenitor potential per stream is needed")
        bodies = pack_bodies([[p] for p in progenitor_potentials]).reshape(S, 1)
        m = _galactic(prog_mass, "Msun")
        if m.ndim == 0:
            m = np.full((S, len(t)), float(m))
        elif m.ndim == 1:
            if m.shape[0] != S:
                raise ValueError("prog_mass must have one entry per stream")
            m = np.repeat(m[:, None], len(t), axis=1)
        counts = self.df.release_counts(len(t), release_every, n_particles)
        Integrator = get_integrator(DOPRI853Integrator if Integrator is None else Integrator)
        if Integrator not in (DOPRI853Integrator, LeapfrogIntegrator):
            raise ValueError("only DOPRI853Integrator and LeapfrogIntegrator are supported for mock streams")
        kw_in = dict(Integrator_kwargs or {})
        precision = kw_in.pop("precision", "fp64")
        dop, err_if_fail = self._dop_kwargs(kw_in if Integrator is DOPRI853Integrator else {})
        if output_every is not None:
            output_every = self._check_animate(output_every, Integrator, precision)
        body_w0 = np.ascontiguousarray(w0.T.reshape(S, 1, 6))
        return self._generate(bodies, body_w0, m, t, counts, dop, err_if_fail, return_stats=return_stats,
                              stream=stream, integrator="leapfrog" if Integrator is LeapfrogIntegrator else "dop853",
                              precision=precision, output_every=output_every)
