"""ctypes mirror of the structs in include/mcx_abi.h (MCX's Config / GPUInfo layouts).

Layouts are built with explicit padding (``_pack_ = 1``) so that CUDA's 16-byte alignment of
``float4`` is reproduced exactly; tests/test_abi_layout.py checks every offset against a C
probe compiled from the header.
"""

from __future__ import annotations

import ctypes as C

SESSION_LEN = 256
PATH_LEN = 1024
MAX_DEVICE = 256
LANG_LEN = 32


def _layout(name: str, spec: list[tuple[str, type, int]]) -> type:
    """A packed ctypes Structure whose members sit at C's natural offsets."""
    fields = []
    off = 0
    npad = 0
    maxal = 1
    for fname, ctype, align in spec:
        maxal = max(maxal, align)
        if off % align:
            n = align - off % align
            fields.append((f"_pad{npad}", C.c_uint8 * n))
            npad += 1
            off += n
        fields.append((fname, ctype))
        off += C.sizeof(ctype)
    if off % maxal:
        fields.append((f"_pad{npad}", C.c_uint8 * (maxal - off % maxal)))
    cls = type(name, (C.Structure,), {"_pack_": 1, "_fields_": fields, "_align": maxal})
    return cls


class float4(C.Structure):
    _pack_ = 1
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class float3(C.Structure):
    _pack_ = 1
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class uint3(C.Structure):
    _pack_ = 1
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


Medium = _layout("Medium", [("mua", C.c_float, 4), ("mus", C.c_float, 4), ("g", C.c_float, 4), ("n", C.c_float, 4)])

ExtraSrc = _layout("ExtraSrc", [("srcpos", float4, 16), ("srcdir", float4, 16), ("srcparam1", float4, 16),
                                ("srcparam2", float4, 16)])

POLMedium = _layout("POLMedium", [("mua", C.c_float, 4), ("r", C.c_float, 4), ("rho", C.c_float, 4),
                                  ("nsph", C.c_float, 4), ("nmed", C.c_float, 4)])

History = _layout("History", [
    ("magic", C.c_char * 4, 1), ("version", C.c_uint, 4), ("maxmedia", C.c_uint, 4), ("detnum", C.c_uint, 4),
    ("colcount", C.c_uint, 4), ("totalphoton", C.c_uint, 4), ("detected", C.c_uint, 4), ("savedphoton", C.c_uint, 4),
    ("unitinmm", C.c_float, 4), ("seedbyte", C.c_uint, 4), ("normalizer", C.c_float, 4), ("respin", C.c_int, 4),
    ("srcnum", C.c_uint, 4), ("savedetflag", C.c_uint, 4), ("totalsource", C.c_uint, 4), ("reserved", C.c_int * 1, 4),
])

Replay = _layout("Replay", [("detid", C.c_void_p, 8), ("seed", C.c_void_p, 8), ("weight", C.c_void_p, 8),
                            ("tof", C.c_void_p, 8)])

GPUInfo = _layout("GPUInfo", [
    ("name", C.c_char * SESSION_LEN, 1), ("id", C.c_int, 4), ("devcount", C.c_int, 4), ("major", C.c_int, 4),
    ("minor", C.c_int, 4), ("globalmem", C.c_size_t, 8), ("constmem", C.c_size_t, 8), ("sharedmem", C.c_size_t, 8),
    ("regcount", C.c_int, 4), ("clock", C.c_int, 4), ("sm", C.c_int, 4), ("core", C.c_int, 4),
    ("autoblock", C.c_int, 4), ("autothread", C.c_int, 4), ("maxgate", C.c_uint, 4), ("maxmpthread", C.c_int, 4),
])

_P = C.c_void_p
_CONFIG_SPEC = [
    ("nphoton", C.c_size_t, 8), ("nblocksize", C.c_uint, 4), ("nthread", C.c_uint, 4), ("seed", C.c_int, 4),
    ("srcpos", float4, 16), ("srcdir", float4, 16), ("srciquv", float4, 16),
    ("tstart", C.c_float, 4), ("tstep", C.c_float, 4), ("tend", C.c_float, 4), ("steps", float3, 4),
    ("dim", uint3, 4), ("crop0", uint3, 4), ("crop1", uint3, 4),
    ("medianum", C.c_uint, 4), ("polmedianum", C.c_uint, 4), ("detnum", C.c_uint, 4), ("maxdetphoton", C.c_uint, 4),
    ("detradius", C.c_float, 4), ("sradius", C.c_float, 4),
    ("prop", _P, 8), ("polprop", _P, 8), ("detpos", _P, 8), ("smatrix", _P, 8),
    ("maxgate", C.c_uint, 4), ("respin", C.c_int, 4), ("printnum", C.c_int, 4), ("gpuid", C.c_int, 4),
    ("vol", _P, 8), ("session", C.c_char * SESSION_LEN, 1),
    ("isrowmajor", C.c_char, 1), ("isreflect", C.c_char, 1), ("isref3", C.c_char, 1), ("isrefint", C.c_char, 1),
    ("isnormalized", C.c_char, 1), ("issavedet", C.c_char, 1), ("issave2pt", C.c_char, 1), ("isgpuinfo", C.c_char, 1),
    ("isspecular", C.c_char, 1), ("issrcfrom0", C.c_char, 1), ("isdumpmask", C.c_char, 1), ("autopilot", C.c_char, 1),
    ("issaveseed", C.c_char, 1), ("issaveexit", C.c_char, 1), ("issaveref", C.c_char, 1), ("ismomentum", C.c_char, 1),
    ("istrajstokes", C.c_char, 1), ("isdumpjson", C.c_char, 1), ("internalsrc", C.c_char, 1),
    ("zipid", C.c_int, 4), ("srctype", C.c_char, 1), ("outputtype", C.c_char, 1), ("outputformat", C.c_char, 1),
    ("faststep", C.c_char, 1), ("minenergy", C.c_float, 4), ("unitinmm", C.c_float, 4), ("omega", C.c_float, 4),
    ("lambda_", C.c_float, 4), ("flog", _P, 8), ("his", History, 4), ("exportfield", _P, 8),
    ("exportdetected", _P, 8), ("detectedcount", C.c_ulong, 8), ("rootpath", C.c_char * PATH_LEN, 1),
    ("shapedata", _P, 8), ("extrajson", _P, 8), ("maxvoidstep", C.c_int, 4), ("voidtime", C.c_int, 4),
    ("srcparam1", float4, 16), ("srcparam2", float4, 16), ("srcnum", C.c_uint, 4), ("srcpattern", _P, 8),
    ("replay", Replay, 8), ("seeddata", _P, 8), ("replaydet", C.c_int, 4), ("seedfile", C.c_char * PATH_LEN, 1),
    ("jsonfile", C.c_char * PATH_LEN, 1), ("debuglevel", C.c_uint, 4), ("savedetflag", C.c_uint, 4),
    ("deviceid", C.c_char * MAX_DEVICE, 1), ("workload", C.c_float * MAX_DEVICE, 4), ("parentid", C.c_int, 4),
    ("runtime", C.c_uint, 4), ("langid", C.c_char * LANG_LEN, 1),
    ("energytot", C.c_double, 8), ("energyabs", C.c_double, 8), ("energyesc", C.c_double, 8),
    ("normalizer", C.c_float, 4), ("maxjumpdebug", C.c_uint, 4), ("debugdatalen", C.c_uint, 4),
    ("gscatter", C.c_uint, 4), ("exportdebugdata", _P, 8), ("mediabyte", C.c_uint, 4),
    ("dx", _P, 8), ("dy", _P, 8), ("dz", _P, 8), ("bc", C.c_char * 13, 1), ("nphase", C.c_uint, 4),
    ("invcdf", _P, 8), ("nangle", C.c_uint, 4), ("angleinvcdf", _P, 8), ("srcid", C.c_int, 4),
    ("extrasrclen", C.c_uint, 4), ("srcdata", _P, 8),
]
Config = _layout("Config", _CONFIG_SPEC)
CONFIG_FIELDS = [name for name, _, _ in _CONFIG_SPEC]


class Stats(C.Structure):
    """mirror of mcxg_stats (include/mcx_gb300.h)"""
    _fields_ = [
        ("e_launch", C.c_double), ("e_escape", C.c_double), ("e_detect", C.c_double), ("e_absdep", C.c_double),
        ("e_absother", C.c_double), ("n_steps", C.c_uint64), ("n_scatter", C.c_uint64), ("n_deposit", C.c_uint64),
        ("n_launch", C.c_uint64), ("n_photon", C.c_uint64), ("n_detected", C.c_uint64), ("n_tile_deposit", C.c_uint64),
        ("kernel_ms", C.c_double), ("total_ms", C.c_double), ("grid", C.c_int), ("block", C.c_int), ("chunk", C.c_int),
        ("launches", C.c_int), ("error_flags", C.c_uint32),
    ]


def offsets(struct: type) -> dict[str, int]:
    """Byte offset of every named (non-padding) member."""
    return {f[0]: getattr(struct, f[0]).offset for f in struct._fields_ if not f[0].startswith("_pad")}
