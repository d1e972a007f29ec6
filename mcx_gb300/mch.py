"""Detected-photon (.mch, .jdat) and trajectory (.mct, .jdat) files in MCX's layouts.

MCX's command-line front-end writes both with ``mcx_savedetphoton`` (src/mcx_utils.c:982-1017):
the 64-byte ``History`` header of the run (src/mcx_utils.h:115-132; ``abi.History`` here), then
the records as float32, ``colcount`` values per photon, then, when seeds were saved, ``seedbyte``
bytes of RNG state per photon.  A trajectory file carries the same header with ``colcount`` = 6,
``savedphoton`` = the number of records and ``detected`` = 0 (src/mcx_core.cu:3966-3975), which
also gives it MCX's ``.mct`` suffix.  pmcx's ``loadmch`` (pmcx/pmcx/io.py:126) and mcxlab's
``loadmch.m`` read these files.

With ``-F jnii`` MCX writes the same data as a JSON/JData ``.jdat`` document instead
(``mcx_savejdet``, src/mcx_utils.c:1029-1200): ``MCXData.Info`` holds the header fields by name
and the media table, ``MCXData.PhotonData`` one JData array per column group the save mask
selects (detid, nscat, ppath, mom, p, v, w0, s; plus ``seed``), ``MCXData.Trajectory`` the
trajectory columns (photonid, p, w0, srcid).  Each array is photon-major ``[count, columns]``,
zlib-compressed and base64-encoded (``mcx_jdataencode``, src/mcx_utils.c:4538-4614).
"""

from __future__ import annotations

import base64
import ctypes as C
import json
import zlib
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


# -- JSON/JData (.jdat) -------------------------------------------------------------------------
# column groups of a detected-photon record in save-mask bit order (src/mcx_utils.c:1087-1089);
# `None` columns are per-medium (maxmedia of them)
_DET_GROUPS = (("detid", 1, "uint32"), ("nscat", None, "uint32"), ("ppath", None, "single"),
               ("mom", None, "single"), ("p", 3, "single"), ("v", 3, "single"), ("w0", 1, "single"),
               ("s", 4, "single"))
# trajectory columns (src/mcx_utils.c:1064-1066); "iquv" only when the run has several sources
_TRAJ_GROUPS = (("photonid", 1, "uint32"), ("p", 3, "single"), ("w0", 1, "single"), ("srcid", 1, "uint32"),
                ("iquv", 4, "single"))
_JD_TYPES = {"uint8": np.uint8, "int8": np.int8, "uint16": np.uint16, "int16": np.int16, "uint32": np.uint32,
             "int32": np.int32, "uint64": np.uint64, "int64": np.int64, "single": np.float32, "double": np.float64}


def jdata_encode(a: np.ndarray, jtype: str, zip: str = "zlib") -> dict[str, Any]:
    """A JData annotated array: type, size, compression, compressed bytes in base64 (row-major)."""
    a = np.ascontiguousarray(a, _JD_TYPES[jtype])
    raw = a.tobytes()
    if zip == "zlib":
        packed = zlib.compress(raw)
    elif zip == "gzip":
        c = zlib.compressobj(wbits=31)
        packed = c.compress(raw) + c.flush()
    elif zip == "base64":
        packed = raw
    else:
        raise ValueError(f"unsupported JData compression {zip!r} (zlib, gzip or base64)")
    return {"_ArrayType_": jtype, "_ArraySize_": [int(d) for d in a.shape], "_ArrayZipType_": zip,
            "_ArrayZipSize_": int(a.size), "_ArrayZipData_": base64.b64encode(packed).decode("ascii")}


def jdata_decode(obj: dict[str, Any]) -> np.ndarray:
    """The array of a JData annotated array written by `jdata_encode` or by MCX (zlib, gzip or
    base64 payloads; ``_ArrayOrder_`` "c" marks column-major data)."""
    dt = _JD_TYPES[obj["_ArrayType_"]]
    size = [int(d) for d in obj["_ArraySize_"]]
    zt = obj.get("_ArrayZipType_", "base64")
    data = base64.b64decode(obj["_ArrayZipData_"])
    if zt == "zlib":
        data = zlib.decompress(data)
    elif zt == "gzip":
        data = zlib.decompress(data, wbits=31)
    elif zt != "base64":
        raise ValueError(f"unsupported JData compression {zt!r}")
    order = "F" if obj.get("_ArrayOrder_", "r") == "c" else "C"
    return np.frombuffer(data, dt).reshape(size, order=order).copy()


def _media(pc) -> list[dict[str, float]]:
    """The media table in 1/mm, as MCX lists it: the engine's copy is scaled by the voxel size."""
    n = int(pc.c.medianum)
    prop = np.ctypeslib.as_array((C.c_float * (4 * n)).from_address(pc.c.prop)).reshape(n, 4)
    u = float(pc.c.unitinmm)
    return [{"mua": float(r[0]) / u, "mus": float(r[1]) / u, "g": float(r[2]), "n": float(r[3])} for r in prop]


def _info(h: abi.History, count: int, media: list[dict[str, float]]) -> dict[str, Any]:
    return {"Version": h.version, "MediaNum": h.maxmedia, "DetNum": h.detnum, "ColumnNum": h.colcount,
            "TotalPhoton": h.totalphoton, "DetectedPhoton": count, "SavedPhoton": h.savedphoton,
            "LengthUnit": h.unitinmm, "SeedByte": h.seedbyte, "Normalizer": h.normalizer, "Repeat": h.respin,
            "SrcNum": h.srcnum, "SaveDetFlag": h.savedetflag, "TotalSource": h.totalsource, "Media": media}


def save_jdet(fname: str | Path, pc, result: dict[str, Any], trajectory: bool = False, zip: str = "zlib") -> Path:
    """Write the detected photons of ``result`` (``trajectory=False``; seeds too when the run saved
    them) or its trajectory records (``trajectory=True``) as MCX's ``-F jnii`` front-end does
    (``mcx_savejdet``, src/mcx_utils.c:1029-1200): the header fields of the run, then one JData
    array per column group, integers as uint32."""
    h = _header(pc)
    h.unitinmm = pc.c.unitinmm
    h.totalphoton = int(pc.c.nphoton)
    media = _media(pc)
    if trajectory:
        rec = np.asarray(result["traj"], np.float32)
        h.colcount, h.savedphoton, h.detected = rec.shape[0], rec.shape[1], 0
        groups = _TRAJ_GROUPS[:len(_TRAJ_GROUPS) - (h.totalsource == 1)]
        section = "Trajectory"
    else:
        detp = result.get("detp")
        rec = np.zeros((h.colcount, 0), np.float32) if detp is None else np.asarray(detp, np.float32)
        if rec.shape[0] != h.colcount:
            raise ValueError(f"records have {rec.shape[0]} columns, the run's header says {h.colcount}")
        h.savedphoton = h.detected = rec.shape[1]
        groups = [(name, h.maxmedia if k is None else k, t)
                  for bit, (name, k, t) in enumerate(_DET_GROUPS) if (h.savedetflag >> bit) & 1]
        section = "PhotonData"
    count = rec.shape[1]
    out: dict[str, Any] = {}
    col = 0
    for name, k, jtype in groups:
        if col + k > rec.shape[0]:
            break
        block = rec[col:col + k].T                                   # [count, k], photon-major
        if jtype == "uint32":
            block = block.astype(np.uint32)
            # several sources: the writer splits the second column group's high 16 bits off as
            # "srcid" (src/mcx_utils.c:1095, 1119-1142)
            if section == "PhotonData" and name == "nscat" and h.totalsource > 1:
                out["srcid"] = jdata_encode(block >> 16, "uint32", zip)
                block = block & 0xFFFF
        out[name] = jdata_encode(block, jtype, zip)
        col += k
    seeds = result.get("seeds")
    if not trajectory and seeds is not None and count and h.seedbyte:
        out["seed"] = jdata_encode(np.asarray(seeds, np.uint8).T, "uint8", zip)
    doc = {"MCXData": {"Info": _info(h, count, media), section: out}}
    Path(fname).write_text(json.dumps(doc, indent="\t") + "\n")
    return Path(fname)


def load_jdet(fname: str | Path) -> tuple[dict[str, Any], np.ndarray, np.ndarray | None]:
    """(Info, records [ColumnNum, count] F-ordered float32, seeds [SeedByte, count] or None) of a
    ``.jdat`` file written by `save_jdet` or by MCX's front-end: the column groups are put back in
    record order, so the result reads like `load_mch`'s and can seed a replay."""
    doc = json.loads(Path(fname).read_text())["MCXData"]
    info = doc["Info"]
    count = int(info["DetectedPhoton"])
    if "Trajectory" in doc:
        groups, data = [(n, k) for n, k, _ in _TRAJ_GROUPS], doc["Trajectory"]
    else:
        m = int(info["MediaNum"])
        data = doc.get("PhotonData", {})
        groups = [(n, m if k is None else k) for bit, (n, k, _) in enumerate(_DET_GROUPS)
                  if (int(info["SaveDetFlag"]) >> bit) & 1]
    cols = []
    for name, k in groups:
        if name not in data:
            continue
        a = jdata_decode(data[name]).reshape(count, -1)
        if name == "nscat" and "srcid" in data:
            a = a | (jdata_decode(data["srcid"]).reshape(count, -1) << 16)
        cols.append(a.astype(np.float32).T)
    rec = np.concatenate(cols, axis=0) if cols else np.zeros((0, count), np.float32)
    if rec.shape[0] != int(info["ColumnNum"]):
        raise ValueError(f"{fname}: {rec.shape[0]} columns decoded, the header says {info['ColumnNum']}")
    seeds = None
    if "seed" in data:
        seeds = jdata_decode(data["seed"]).reshape(count, -1).T.copy()
    return info, np.asfortranarray(rec), seeds
