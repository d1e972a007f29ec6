"""Device-resident simulation sessions (``mcxg_session_*`` in include/mcx_gb300.h).

A session uploads labels, properties and detectors once; each ``run`` launches only the
persistent transport kernel over a photon range.  The benchmark times these launches with the
inputs already in HBM; ``mcx_run_simulation`` is built from the same pieces.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._lib import lib
from .api import MCXError, PreparedConfig, _check


class Session:
    def __init__(self, pc: PreparedConfig, device: int = 0):
        self.pc = pc
        lib.mcxg_clear_error()
        self.h = lib.mcxg_session_create(C.byref(pc.c), device)
        _check()
        if not self.h:
            raise MCXError(-1, "session creation failed")

    def autotune(self, nphoton: int) -> None:
        """Pick the deposit-tile size from pilot launches (clears the buffers)."""
        _check(lib.mcxg_session_autotune(self.h, nphoton))

    def reset(self) -> None:
        _check(lib.mcxg_session_reset(self.h))

    def run(self, photon_offset: int, nphoton: int, seed: int) -> float:
        """Launch the transport kernel; returns its CUDA-event time in ms."""
        ms = C.c_float(0.0)
        _check(lib.mcxg_session_run(self.h, photon_offset, nphoton, seed, C.byref(ms)))
        return float(ms.value)

    def read(self, with_field: bool = True, max_records: int = 0):
        nx, ny, nz = self.pc.dims
        st = abi.Stats()
        field = None
        fptr = None
        if with_field:
            maxgate = self.pc.ngates if self.pc.c.maxgate == 0 else min(int(self.pc.c.maxgate), self.pc.ngates)
            field = np.zeros(nx * ny * nz * maxgate, dtype=np.float32)
            fptr = field.ctypes.data_as(C.POINTER(C.c_float))
        detp = None
        dptr = None
        if max_records:
            detp = np.zeros(max_records * max(1, self.pc.reclen), dtype=np.float32)
            dptr = detp.ctypes.data_as(C.POINTER(C.c_float))
        ndet = lib.mcxg_session_read(self.h, fptr, dptr, max_records, C.byref(st))
        _check()
        if field is not None:
            field = field.reshape((nx, ny, nz, -1), order="F")
        return field, detp, int(ndet), st

    def close(self) -> None:
        if self.h:
            lib.mcxg_session_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
