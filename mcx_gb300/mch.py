"""Detected-photon (.mch) and trajectory (.mct) files in MCX's binary layout.

MCX's command-line front-end writes both with ``mcx_savedetphoton`` (src/mcx_utils.c:982-1017):
the 64-byte ``History`` header of the run (src/mcx_utils.h:115-132; ``abi.History`` here), then
the records as float32, ``colcount`` values per photon, then, when seeds were saved, ``seedbyte``
bytes of RNG state per photon.  A trajectory file carries the same header with ``colcount`` = 6,
``savedphoton`` = the number of records and ``detected`` = 0 (src/mcx_core.cu:3966-3975), which
also gives it MCX's ``.mct`` suffix.  pmcx's ``loadmch`` (pmcx/pmcx/io.py:126) and mcxlab's
``loadmch.m`` read these files.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Any

import numpy as np

from . import abi

HEADER_BYTES = C.sizeof(abi.History)


def _header(pc) -> abi.History:
    h = abi.History()
    C.memmove(C.addressof(h), C.addressof(pc.c.his), HEADER_BYTES)
    return h


def save_mch(fname: str | Path, pc, result: dict[str, Any]) -> Path:
    """Write the detected photons of ``result`` (from ``run_prepared(pc)``) as MCX writes them;
    seeds follow the records when the run saved them."""
    h = _header(pc)
    detp = result.get("detp")
    n = 0 if detp is None else int(detp.shape[1])
    # the fields MCX's CLI sets just before it writes (src/mcx_core.cu:3948-3958)
    h.unitinmm = pc.c.unitinmm
    h.savedphoton = n
    h.totalphoton = int(pc.c.nphoton)
    h.detected = n
    if detp is not None and detp.shape[0] != h.colcount:
        raise ValueError(f"records have {detp.shape[0]} columns, the run's header says {h.colcount}")
    with open(fname, "wb") as f:
        f.write(bytes(h))
        if n:
            f.write(np.asarray(detp, np.float32).tobytes(order="F"))
        seeds = result.get("seeds")
        if seeds is not None and n and h.seedbyte:
            f.write(np.ascontiguousarray(np.asarray(seeds, np.uint8).T).tobytes())
    return Path(fname)


def save_mct(fname: str | Path, pc, result: dict[str, Any]) -> Path:
    """Write the trajectory records of ``result`` (``debuglevel`` M or T) as MCX writes them."""
    traj = np.asarray(result["traj"], np.float32)
    h = _header(pc)
    h.colcount = traj.shape[0]
    h.savedphoton = traj.shape[1]
    h.totalphoton = int(pc.c.nphoton)
    h.detected = 0
    with open(fname, "wb") as f:
        f.write(bytes(h))
        f.write(traj.tobytes(order="F"))
    return Path(fname)


def load_mch(fname: str | Path) -> tuple[dict[str, Any], np.ndarray, np.ndarray | None]:
    """(header fields, records [colcount, n] F-ordered, seeds [seedbyte, n] or None) of an .mch
    or .mct file, for files holding one header (MCX appends further blocks only in multi-pass runs)."""
    raw = Path(fname).read_bytes()
    if len(raw) < HEADER_BYTES or raw[:4] != b"MCXH":
        raise ValueError(f"{fname} is not an MCX history file")
    h = abi.History.from_buffer_copy(raw[:HEADER_BYTES])
    hdr = {name: getattr(h, name) for name, *_ in h._fields_ if name not in ("reserved",)}
    hdr["magic"] = bytes(h.magic)
    n, cols = int(h.savedphoton), int(h.colcount)
    body = raw[HEADER_BYTES:HEADER_BYTES + 4 * n * cols]
    if len(body) != 4 * n * cols:
        raise ValueError(f"{fname} is truncated: {len(body)} of {4 * n * cols} record bytes")
    detp = np.frombuffer(body, np.float32).reshape((cols, n), order="F").copy()
    seeds = None
    rest = raw[HEADER_BYTES + 4 * n * cols:]
    if h.seedbyte and n and len(rest) >= n * h.seedbyte:
        seeds = np.frombuffer(rest[:n * h.seedbyte], np.uint8).reshape(n, h.seedbyte).T.copy()
    return hdr, detp, seeds
