"""ctypes front of the CPU oracle (oracle/mcx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, the smoke check and bench.py's CPU-baseline leg use this
module to check or to time; the engine never imports it.  It runs the CPU restatement of MCX's
transport loop on a Config prepared by ``mcx_gb300.prepare`` (the same object the engine
receives) and returns pmcx-shaped results plus the oracle's FP64 raw field, per-voxel deposit
counts and algorithmic counters.
"""

from __future__ import annotations

import ctypes as C
import os
import struct
from pathlib import Path
from typing import Any

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libmcx_oracle.so"


class OracleProblem(C.Structure):
    _fields_ = [
        ("vol", C.c_void_p), ("dim", C.c_uint32 * 3), ("prop", C.c_void_p), ("medianum", C.c_uint32),
        ("detpos", C.c_void_p), ("detnum", C.c_uint32), ("srcpos", C.c_float * 4), ("srcdir", C.c_float * 4),
        ("src_idx", C.c_uint32), ("src_med", C.c_uint32), ("twin0", C.c_float), ("twin1", C.c_float),
        ("tstep", C.c_float), ("maxgate", C.c_uint32), ("unitinmm", C.c_float), ("isreflect", C.c_int),
        ("isspecular", C.c_int), ("voidtime", C.c_int), ("maxvoidstep", C.c_int), ("save2pt", C.c_int),
        ("outputtype", C.c_int), ("minenergy", C.c_float), ("gscatter", C.c_uint32), ("bc", C.c_uint8 * 12),
        ("savedet", C.c_int), ("savedetflag", C.c_uint32), ("maxdetphoton", C.c_uint32), ("nphoton", C.c_uint64),
        ("photon_offset", C.c_uint64), ("seed", C.c_uint64), ("nthreads", C.c_int), ("seed_mode", C.c_int),
        ("mcx_threads", C.c_uint32), ("srctype", C.c_int), ("srcparam1", C.c_float * 4),
        ("srcparam2", C.c_float * 4), ("srcpattern", C.c_void_p), ("mediaformat", C.c_int),
        ("extrasrc", C.c_void_p), ("nextra", C.c_uint32), ("srcid", C.c_int),
    ]


class OracleResult(C.Structure):
    _fields_ = [
        ("field", C.c_void_p), ("hits", C.c_void_p), ("detp", C.c_void_p), ("e_launch", C.c_double),
        ("e_escape", C.c_double), ("e_detect", C.c_double), ("e_absdep", C.c_double), ("e_absother", C.c_double),
        ("n_steps", C.c_uint64), ("n_scatter", C.c_uint64), ("n_deposit", C.c_uint64), ("n_launch", C.c_uint64),
        ("n_detected", C.c_uint64), ("n_photon", C.c_uint64), ("n_saved", C.c_uint64), ("reclen", C.c_uint32),
        ("seconds", C.c_double),
    ]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            import importlib.util

            spec = importlib.util.spec_from_file_location("mcx_gb300_build", HERE.parent / "mcx_gb300" / "build.py")
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle()   # the recipe lives with the engine's
        _lib = C.CDLL(str(LIB_PATH))
        _lib.oracle_run.argtypes = [C.POINTER(OracleProblem), C.POINTER(OracleResult)]
        _lib.oracle_run.restype = C.c_int
        _lib.oracle_rng_kat.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_float), C.c_int]
        _lib.oracle_rng_kat.restype = None
        _lib.oracle_photon_stream.argtypes = [C.c_uint64, C.c_uint64, C.POINTER(C.c_float), C.c_int]
        _lib.oracle_photon_stream.restype = None
    return _lib


def rng_kat(seeds: list[int], n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float32)
    s = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in seeds])
    load().oracle_rng_kat(s, out.ctypes.data_as(C.POINTER(C.c_float)), n)
    return out


def photon_stream(seed: int, pid: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float32)
    load().oracle_photon_stream(seed, pid, out.ctypes.data_as(C.POINTER(C.c_float)), n)
    return out


def run(pc, nphoton: int | None = None, seed: int | None = None, photon_offset: int = 0, threads: int | None = None,
        hits: bool = False, gate_group: int = 0, mcx_threads: int = 0) -> dict[str, Any]:
    """Run the oracle on a prepared Config (``mcx_gb300.prepare``).  Normalisation follows
    src/mcx_core.cu:3823-3925 in FP64.  ``mcx_threads`` > 0 seeds the RNG the way MCX does for
    that many GPU threads (glibc rand() words after srand(seed), photons split statically)."""
    c = pc.c
    nx, ny, nz = pc.dims
    nvox = nx * ny * nz
    ngates = pc.ngates
    maxgate = ngates if c.maxgate == 0 else min(int(c.maxgate), ngates)
    P = OracleProblem()
    P.vol = pc.vol.ctypes.data
    P.dim[:] = [nx, ny, nz]
    P.prop = pc.prop.ctypes.data
    P.medianum = int(c.medianum)
    if pc.detpos is not None:
        P.detpos = pc.detpos.ctypes.data
    P.detnum = int(c.detnum)
    P.srcpos[:] = [c.srcpos.x, c.srcpos.y, c.srcpos.z, c.srcpos.w]
    P.srcdir[:] = [c.srcdir.x, c.srcdir.y, c.srcdir.z, c.srcdir.w]
    if ord(c.srctype) in (0, 1, 2, 7, 11):     # point sources: launch voxel from preprocessing
        P.src_idx = struct.unpack("<I", struct.pack("<f", c.srcparam2.z))[0]
        P.src_med = struct.unpack("<I", struct.pack("<f", c.srcparam2.w))[0]
    P.twin0 = c.tstart + c.tstep * maxgate * gate_group
    P.twin1 = P.twin0 + c.tstep * maxgate
    P.tstep = c.tstep
    P.maxgate = maxgate
    P.unitinmm = c.unitinmm
    P.isreflect = ord(c.isreflect)
    P.isspecular = ord(c.isspecular)
    P.voidtime = int(c.voidtime)
    P.maxvoidstep = int(c.maxvoidstep)
    P.save2pt = ord(c.issave2pt)
    P.outputtype = ord(c.outputtype)
    P.minenergy = c.minenergy
    P.gscatter = int(c.gscatter)
    P.bc[:] = list(C.string_at(C.addressof(c) + type(c).bc.offset, 12))
    savedet = ord(c.issavedet) != 0 and (int(c.detnum) > 0 or any(bytearray(P.bc)[6:12]))
    P.savedet = 1 if savedet else 0
    P.savedetflag = int(c.savedetflag)
    P.maxdetphoton = int(c.maxdetphoton)
    P.nphoton = int(c.nphoton if nphoton is None else nphoton)
    P.photon_offset = photon_offset
    P.seed = int(c.seed if seed is None else seed) & 0xFFFFFFFF
    P.nthreads = threads or os.cpu_count() or 1
    P.seed_mode = 1 if mcx_threads else 0
    P.mcx_threads = int(mcx_threads)
    P.srctype = ord(c.srctype)
    P.srcparam1[:] = [c.srcparam1.x, c.srcparam1.y, c.srcparam1.z, c.srcparam1.w]
    P.srcparam2[:] = [c.srcparam2.x, c.srcparam2.y, c.srcparam2.z, c.srcparam2.w]
    P.srcpattern = c.srcpattern
    P.mediaformat = int(c.mediabyte)
    P.nextra = int(c.extrasrclen)
    P.extrasrc = c.srcdata if P.nextra else None
    P.srcid = int(c.srcid)
    blocks = P.nextra + 1 if (P.nextra and P.srcid < 0) else 1     # one block of gates per source

    field = np.zeros(nvox * maxgate * blocks, dtype=np.float64)
    hit = np.zeros(nvox * maxgate * blocks, dtype=np.uint64) if hits else None
    reclen = int(pc.reclen)
    detp = np.zeros(max(1, int(c.maxdetphoton)) * max(1, reclen), dtype=np.float32) if savedet else None
    R = OracleResult()
    R.field = field.ctypes.data
    R.hits = hit.ctypes.data if hit is not None else None
    R.detp = detp.ctypes.data if detp is not None else None
    rc = load().oracle_run(C.byref(P), C.byref(R))
    if rc:
        raise RuntimeError(f"oracle_run failed with {rc}")

    etot = R.e_launch
    scale = 1.0
    if c.isnormalized != b"\x00" and etot > 0:
        vvox = float(c.steps.x) * float(c.steps.y) * float(c.steps.z)
        ot = ord(c.outputtype)
        if ot in (0, 1):
            scale = float(c.unitinmm) / (etot * vvox * float(c.tstep))
            if ot == 1:
                scale *= float(c.tstep)
        else:
            scale = 1.0 / etot
        if blocks > 1:
            scale *= blocks          # every source ran a share of the photons (src/mcx_core.cu:3908-3910)
    out: dict[str, Any] = {
        "raw": field.reshape((nx, ny, nz, maxgate * blocks), order="F"),
        "flux": (field * scale).reshape((nx, ny, nz, maxgate * blocks), order="F"),
        "normalizer": scale,
        "stat": {
            "energytot": etot, "energyesc": R.e_escape + R.e_detect, "energyabs": etot - (R.e_escape + R.e_detect),
            "e_launch": R.e_launch, "e_escape": R.e_escape, "e_detect": R.e_detect, "e_absdep": R.e_absdep,
            "e_absother": R.e_absother, "n_steps": R.n_steps, "n_scatter": R.n_scatter, "n_deposit": R.n_deposit,
            "n_launch": R.n_launch, "n_detected": R.n_detected, "n_photon": R.n_photon, "seconds": R.seconds,
            "threads": P.nthreads,
        },
    }
    if hit is not None:
        out["hits"] = hit.reshape((nx, ny, nz, maxgate * blocks), order="F")
    if detp is not None:
        nsaved = int(R.n_saved)
        out["detp"] = detp[: nsaved * reclen].reshape((reclen, nsaved), order="F")
        out["stat"]["detected"] = int(R.n_detected)
    return out
