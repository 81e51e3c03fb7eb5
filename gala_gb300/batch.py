"""Batched integration of many orbits with uneven lengths, steps and integrators.

``BatchIntegrator`` runs Leapfrog and Ruth4 orbits of different ``n_steps`` and
``dt`` in one persistent-kernel launch (gx_batch_integrate_fp32): FP32 forces,
Kahan-compensated FP32 state, FP64 initial/final states and an FP64 energy
diagnostic.  The work schedule is computed on the GPU (longest first, one
integrator per chunk); the whole sequence -- schedule, queue reset, persistent
kernel, energy diagnostic -- can be captured once in a CUDA graph and replayed.
Launch shape (block size, CTAs per SM, chunk size) comes from an autotuner whose
choices are cached per GPU, kernel and potential.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import numpy as np

from . import _abi
from ._abi import GX_BATCH_QUEUE_WORDS
from ._trace import traced

LEAPFROG, RUTH4 = 0, 1
COST = {LEAPFROG: 1.0, RUTH4: 3.0}   # gradient evaluations per step
CACHE = Path(os.environ.get("GALA_GB300_AUTOTUNE", Path(__file__).resolve().parent / "_build" / "autotune.json"))
# launch shapes without an autotune record: the autotuner's choice on a GB300 for
# uneven MW-composite batches (few warps per scheduler keep the longest orbits,
# which set the run time, from sharing issue slots)
DEFAULT_CONFIG = {"fp32c": {"block": 128, "ctas_per_sm": 2, "chunk": 32},
                  "fp64": {"block": 32, "ctas_per_sm": 4, "chunk": 32}}
SEARCH = {
    "fp32c": [{"block": b, "ctas_per_sm": c, "chunk": k} for b in (64, 128, 256) for c in (1, 2, 3, 4, 6, 8, 12, 16)
              for k in (32, 64) if 256 <= b * c <= 1536],
    "fp64": [{"block": b, "ctas_per_sm": c, "chunk": k} for b in (32, 64, 128) for c in (1, 2, 4, 8)
             for k in (32, 64) if 64 <= b * c <= 512],
}
ENTRY = {"fp32c": "gx_batch_integrate_fp32", "fp64": "gx_batch_integrate_fp64"}


def schedule(n_steps, method, chunk):
    """The processing order with an exact sort, in torch: per integrator, orbits
    sorted by cost (longest first) and cut into chunks; chunks of both
    integrators merged by cost, longest first; the tail of each integrator's
    list padded with -1.  BatchIntegrator.capture uses it; one-shot runs build
    the same order on the device with costs binned at 0.54 %
    (gx_batch_schedule)."""
    import torch

    dev = n_steps.device
    cost = n_steps.to(torch.float64) * torch.where(method == RUTH4, COST[RUTH4], COST[LEAPFROG])
    pieces, heads = [], []
    for m in (RUTH4, LEAPFROG):
        idx = torch.nonzero(method == m).flatten()
        if idx.numel() == 0:
            continue
        srt = idx[torch.argsort(cost[idx], descending=True, stable=True)].to(torch.int32)
        pad = (-srt.numel()) % chunk
        if pad:
            srt = torch.cat([srt, torch.full((pad,), -1, dtype=torch.int32, device=dev)])
        chunks = srt.view(-1, chunk)
        pieces.append(chunks)
        heads.append(cost[chunks[:, 0].long()])
    chunks = torch.cat(pieces)
    order = torch.argsort(torch.cat(heads), descending=True, stable=True)
    return chunks[order].reshape(-1).contiguous()


def _to_device(a, tdtype, ndtype, dev):
    """Contiguous CUDA tensor of `a` (numpy, list, or tensor); a pinned host
    tensor is copied asynchronously on the current stream."""
    import torch

    if isinstance(a, torch.Tensor):
        nb = a.device.type == "cpu" and a.is_pinned()
        return a.to(device=dev, dtype=tdtype, non_blocking=nb).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=ndtype))).to(dev)


def _host_view(a):
    """A numpy view of a host array (numpy, list or CPU tensor), else None."""
    import torch

    if isinstance(a, torch.Tensor):
        return a.numpy() if a.device.type == "cpu" else None
    return np.asarray(a)


def _potential_key(potential):
    pk = potential.packed()
    h = hashlib.sha1(pk.params.tobytes())
    for i in range(pk.desc.n_components):
        h.update(bytes([pk.components[i].type, pk.components[i].do_shift_rotate]))
    return h.hexdigest()[:16]


class BatchIntegrator:
    """Integrate N orbits, each with its own n_steps, dt and integrator.

    Parameters
    ----------
    potential : closed-form gala_gb300 potential (SCF is not supported here)
    w0 : (6, N) array-like or CUDA tensor, float64
    n_steps : (N,) integers; dt : (N,) floats; method : (N,) 0 = leapfrog, 1 = ruth4
    precision : "fp32c" (FP32 forces, compensated FP32 state; closed-form
        potentials) or "fp64" (gala's arithmetic in FP64, the plain form)
    config : dict with block, ctas_per_sm, chunk; None = autotuned/cached choice
    checkpoint : keep the integrator state after every run in ``self.state``
        ((12, N) float32 on the device; fp32c only)
    state : a ``state`` of an earlier run to resume from (fp32c only): a run of
        k steps with checkpoint=True, then one of n - k steps with
        state=<its state> (and the same w0, dt, method), gives the bits of one
        run of n steps
    """

    def __init__(self, potential, w0, n_steps, dt, method, config=None, precision="fp32c", checkpoint=False,
                 state=None):
        import torch

        from ._device import as_device_f64, require_cuda

        if precision not in ENTRY:
            raise ValueError(f"precision must be one of {sorted(ENTRY)}")
        self.precision = precision
        self.dev = require_cuda()
        self.potential = potential
        self.w0 = as_device_f64(w0)
        if self.w0.dim() != 2 or self.w0.shape[0] != 6:
            raise ValueError(f"w0 must have shape (6, N), got {tuple(self.w0.shape)}")
        self.n = self.w0.shape[1]
        self.n_steps = _to_device(n_steps, torch.int64, np.int64, self.dev)
        self.dt = as_device_f64(dt)
        self.method = _to_device(method, torch.int32, np.int32, self.dev)
        for name, a in (("n_steps", self.n_steps), ("dt", self.dt), ("method", self.method)):
            if a.shape != (self.n,):
                raise ValueError(f"{name} must have shape ({self.n},), got {tuple(a.shape)}")
        if self.n:
            # host inputs are checked on the host; device inputs in one reduction (one sync)
            ms, ns = _host_view(method), _host_view(n_steps)
            if ms is not None and ns is not None:
                mlo, mhi, nlo = int(ms.min()), int(ms.max()), int(ns.min())
            else:
                mlo, mhi, nlo = torch.stack([self.method.min().to(torch.int64), self.method.max().to(torch.int64),
                                             self.n_steps.min()]).tolist()
            if mlo < 0 or mhi > 1:
                raise ValueError("method must be 0 (leapfrog) or 1 (ruth4)")
            if nlo < 0:
                raise ValueError("n_steps must be non-negative")
        self.sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        self.config = dict(config) if config is not None else self._cached_config()
        self.w_out = torch.empty((6, self.n), dtype=torch.float64, device=self.dev)
        self.E0 = torch.empty(self.n, dtype=torch.float64, device=self.dev)
        self.E1 = torch.empty(self.n, dtype=torch.float64, device=self.dev)
        # work-queue scratch: [0] main-region claims, [1] lead-region claims, flags
        self.counter = torch.zeros(GX_BATCH_QUEUE_WORDS, dtype=torch.int32, device=self.dev)
        self.graph = None
        if (checkpoint or state is not None) and precision != "fp32c":
            raise NotImplementedError("integrator checkpoints are kept by the fp32c form")
        self.state_in = None
        if state is not None:
            self.state_in = torch.as_tensor(state, dtype=torch.float32, device=self.dev).contiguous()
            if self.state_in.shape != (12, self.n):
                raise ValueError(f"state must have shape (12, {self.n}), got {tuple(self.state_in.shape)}")
        self.state = torch.empty((12, self.n), dtype=torch.float32, device=self.dev) if checkpoint else None

    # ------------------------------------------------------------------ run
    def _prepare(self, stream_handle=None, exact=False):
        """The processing order for the current launch shape: built on the
        device on the launching stream (gx_batch_schedule, no host sync, costs
        binned at 0.54 %), or with exact=True by an exact sort in torch (two
        host syncs, about 0.7 ms for 262,144 orbits; the binned order measured
        1.5-2.5 % slower on the uneven MW workload, so a captured graph, which
        replays one order many times, takes the exact one)."""
        import torch

        from ._device import ptr

        chunk = self.config["chunk"]
        if exact:
            self.order = schedule(self.n_steps, self.method, chunk)
            self._order_chunk = chunk
            return
        lib = _abi.load()
        slots = int(lib.gx_batch_schedule_slots(self.n, chunk))
        words = int(lib.gx_batch_schedule_work_words(self.n, chunk))
        if getattr(self, "order", None) is None or self.order.numel() != slots:
            self.order = torch.empty(slots, dtype=torch.int32, device=self.dev)
        if getattr(self, "_sched_work", None) is None or self._sched_work.numel() < words:
            self._sched_work = torch.empty(words, dtype=torch.int32, device=self.dev)
        _abi.call("gx_batch_schedule", ptr(self.n_steps), ptr(self.method), self.n, chunk, ptr(self.order), slots,
                  ptr(self._sched_work), words, stream_handle)
        self._order_chunk = chunk

    def _launch_integrator(self, stream_handle):
        from ._device import ptr

        cfg = self.config
        if getattr(self, "_order_chunk", None) != cfg["chunk"]:
            self._prepare(stream_handle)
        desc = self.potential.packed().for_device()
        common = (desc, ptr(self.w0), self.n, ptr(self.n_steps), ptr(self.dt), ptr(self.method), ptr(self.order),
                  self.order.numel(), cfg["chunk"], cfg["block"], cfg["ctas_per_sm"] * self.sms, ptr(self.counter))
        if self.state_in is not None or self.state is not None:
            _abi.call("gx_batch_integrate_fp32_state", *common,
                      ptr(self.state_in) if self.state_in is not None else None,
                      ptr(self.state) if self.state is not None else None, ptr(self.w_out), stream_handle)
        else:
            _abi.call(ENTRY[self.precision], *common, ptr(self.w_out), stream_handle)
        return desc

    def _launch(self, stream_handle):
        import ctypes as C

        from ._device import ptr

        desc = self._launch_integrator(stream_handle)
        frame = _abi.gx_frame()
        _abi.call("gx_hamiltonian_value", desc, C.byref(frame), 0.0, ptr(self.w0), self.n, ptr(self.E0),
                  stream_handle)
        _abi.call("gx_hamiltonian_value", desc, C.byref(frame), 0.0, ptr(self.w_out), self.n, ptr(self.E1),
                  stream_handle)

    @traced("batch_run")
    def run(self):
        """Integrate every orbit once (eager launch sequence)."""
        from ._device import stream_handle

        if self.n == 0:
            return self.w_out
        if self.graph is not None:
            self.graph.replay()
        else:
            self._launch(stream_handle())
        return self.w_out

    def capture(self):
        """Capture queue reset + persistent kernel + energy diagnostic in one CUDA
        graph (the schedule is computed once, eagerly); run() then replays it."""
        import torch

        from ._device import stream_handle

        if self.n == 0:
            return self
        self._prepare(stream_handle(), exact=True)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self._launch(stream_handle(s))   # warm up allocations outside the graph
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._launch(stream_handle())
        self.graph = g
        return self

    def energy_drift(self):
        """|E(t_end) - E(0)| / |E(0)| per orbit (FP64 diagnostic)."""
        return ((self.E1 - self.E0) / self.E0).abs()

    def _taken_slots(self):
        """(start, stop) ranges of the order's slots that the last run took:
        the first min(q[1], n_lead x chunk / 32) blocks of 32 slots of the lead
        region and the first min(q[0], n_chunks - n_lead) chunks after it,
        n_lead = min(n_chunks, 4 x multiprocessors / (chunk / 32)) (the queue of
        the batched kernels)."""
        chunk = self.config["chunk"]
        subs = chunk // 32
        n_chunks = self.order.numel() // chunk
        n_lead = min(n_chunks, 4 * self.sms // subs)
        q_main, q_lead = (int(v) for v in self.counter[:2].tolist())
        lead = min(q_lead, n_lead * subs)
        main = min(q_main, n_chunks - n_lead)
        return [(0, 32 * lead), (n_lead * chunk, (n_lead + main) * chunk)]

    def chunks_taken(self):
        """How many chunks' worth of the order the last run took (all of them
        unless it was cancelled)."""
        return sum(b - a for a, b in self._taken_slots()) // self.config["chunk"]

    def completed(self):
        """(N,) bool CUDA tensor: the orbits the last run integrated.  All of
        them unless the run was cancelled (``gala_gb300.cancel``): a cancelled
        launch takes no further queue chunk, so the orbits of the chunks it
        took are done and the others' rows of the output are untouched."""
        import torch

        done = torch.zeros(self.n, dtype=torch.bool, device=self.dev)
        for a, b in self._taken_slots():
            ids = self.order[a:b].long()
            done[ids[ids >= 0]] = True
        return done

    # ------------------------------------------------------------- autotune
    def _cache_key(self):
        import torch

        return (f"{torch.cuda.get_device_name(self.dev)}|{ENTRY[self.precision]}|"
                f"{_potential_key(self.potential)}")

    def _cached_config(self):
        try:
            return dict(_read_cache()[self._cache_key()])
        except KeyError:
            return dict(DEFAULT_CONFIG[self.precision])

    def autotune(self, work_fraction=0.03, reps=2, persist=True):
        """Time every launch shape of SEARCH on a scaled copy of this workload --
        all orbits, every step count multiplied by `work_fraction` (at least 1),
        so the number of warps and the spread of orbit lengths are those of the
        real run -- keep the fastest and cache it."""
        import torch

        from ._device import stream_handle

        scaled = torch.clamp(torch.ceil(self.n_steps.to(torch.float64) * work_fraction), min=1).to(torch.int64)
        sub = BatchIntegrator(self.potential, self.w0, scaled, self.dt, self.method,
                              config=DEFAULT_CONFIG[self.precision], precision=self.precision)
        results = []
        stream = torch.cuda.current_stream()
        for cfg in SEARCH[self.precision]:
            sub.config = cfg
            sub._launch_integrator(stream_handle())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                sub._launch_integrator(stream_handle())
            e1.record(stream)
            e1.synchronize()
            results.append((e0.elapsed_time(e1) * 1e-3 / reps, cfg))
        best = min(results, key=lambda r: r[0])[1]
        self.config = dict(best)
        self.tune_results = [(t, c) for t, c in sorted(results, key=lambda r: r[0])]
        if persist:
            CACHE.parent.mkdir(parents=True, exist_ok=True)
            try:
                data = json.loads(CACHE.read_text())
            except (FileNotFoundError, ValueError):
                data = {}
            data[self._cache_key()] = best
            # write-then-rename: ranks tuning at once never leave a torn file
            tmp = CACHE.with_name(f"{CACHE.name}.{os.getpid()}.tmp")
            tmp.write_text(json.dumps(data, indent=1))
            os.replace(tmp, CACHE)
        return best


_METHODS = {"leapfrog": LEAPFROG, "ruth4": RUTH4}


_cache_memo = {"stamp": None, "data": {}}


def _read_cache():
    """The autotune records, read again only when the file changes."""
    try:
        st = CACHE.stat()
    except FileNotFoundError:
        return {}
    stamp = (st.st_mtime_ns, st.st_size)
    if _cache_memo["stamp"] != stamp:
        try:
            _cache_memo["data"] = json.loads(CACHE.read_text())
        except (FileNotFoundError, ValueError):
            _cache_memo["data"] = {}
        _cache_memo["stamp"] = stamp
    return _cache_memo["data"]


def _method_codes(integrator, n):
    if isinstance(integrator, str):
        if integrator.lower() not in _METHODS:
            raise ValueError(f"integrator must be 'leapfrog' or 'ruth4', got {integrator!r}")
        return np.full(n, _METHODS[integrator.lower()], dtype=np.int32)
    arr = np.asarray(integrator)
    if arr.dtype.kind in "US":
        bad = sorted({str(x) for x in arr.ravel() if str(x).lower() not in _METHODS})
        if bad:
            raise ValueError(f"unknown integrators {bad}: use 'leapfrog' or 'ruth4'")
        return np.array([_METHODS[str(x).lower()] for x in arr.ravel()], dtype=np.int32)
    return integrator


@traced("integrate_batch")
def integrate_batch(potential, w0, n_steps, dt, integrator, precision="fp32c", config=None, out=None):
    """Integrate N orbits, each with its own ``n_steps``, ``dt`` and integrator,
    in one launch of the persistent batch kernel.

    ``integrator`` is 'leapfrog', 'ruth4', or an (N,) array of those names or of
    codes 0 / 1.  Host inputs (numpy arrays or pinned CPU tensors) are copied
    to the GPU on the current stream; the results come back the same way.

    Returns ``(w, dE_over_E)``: the final states (6, N) at t = n_steps * dt
    and the FP64 relative energy change |E(t_end) - E(0)| / |E(0)| per orbit --
    numpy arrays for host inputs, CUDA tensors for device inputs.  ``out``
    (host, optional) is a pair of pinned CPU tensors (6, N) and (N,) that
    receive the results.
    """
    import torch

    on_host = not (isinstance(w0, torch.Tensor) and w0.is_cuda)
    n = (w0.shape[1] if hasattr(w0, "shape") else np.asarray(w0).shape[1])
    method = _method_codes(integrator, n)
    b = BatchIntegrator(potential, w0, n_steps, dt, method, config=config, precision=precision)
    w = b.run()
    dE = b.energy_drift()
    if not on_host:
        return w, dE
    if out is not None:
        out[0].copy_(w, non_blocking=True)
        out[1].copy_(dE, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return out[0].numpy(), out[1].numpy()
    return w.cpu().numpy(), dE.cpu().numpy()
