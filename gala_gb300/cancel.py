"""Cancelling long GPU calls from the host.

gala's mock-stream loop checks for a keyboard interrupt between releases
(``PyErr_CheckSignals``, src/gala/dynamics/mockstream/mockstream.pyx:277).  A
call here is a single kernel launch, so its kernels poll a flag in mapped host
memory instead: once the flag is set, the persistent kernels take no further
work (orbit chunks, orbits, release systems, DOP853 batches) and a mock stream
in the animate mode stops between intervals.  What each entry point leaves
behind is listed with ``gx_set_cancel_flag`` in include/gala_gb300.h.

    flag = CancelFlag()
    with flag.installed():          # launches from this thread read the flag
        out = integrate_batch(...)  # returns once the launch is queued
        ...
        flag.set()                  # from this or any other thread
        torch.cuda.synchronize()    # the launch ends early
"""
from __future__ import annotations

import contextlib
import ctypes as C

from . import _abi

__all__ = ["CancelFlag"]


class CancelFlag:
    """A cancel flag in pinned, mapped host memory (gx_cancel_flag_create)."""

    def __init__(self):
        lib = _abi.load()
        h, d = C.c_void_p(), C.c_void_p()
        _abi.call("gx_cancel_flag_create", C.addressof(h), C.addressof(d))
        self._host = h.value
        self.device_ptr = d.value
        self._value = C.c_int32.from_address(self._host)
        self._lib = lib

    def set(self):
        """Request cancellation of the launches that read this flag."""
        self._value.value = 1

    def clear(self):
        self._value.value = 0

    @property
    def is_set(self) -> bool:
        return self._value.value != 0

    @contextlib.contextmanager
    def installed(self):
        """Hand the flag to every launch made from the calling thread inside the block."""
        self._lib.gx_set_cancel_flag(self.device_ptr)
        try:
            yield self
        finally:
            self._lib.gx_set_cancel_flag(None)

    def close(self):
        """Free the flag; only after every launch that reads it has completed."""
        if self._host is not None:
            self._lib.gx_cancel_flag_destroy(self._host)
            self._host = None
            self._value = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
