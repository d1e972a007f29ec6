"""pmcx-style Python interface of the GB300 engine.

``run(cfg)`` takes the same dictionary ``pmcx.run`` takes (src/pmcx.cpp:400-1065 parse_config,
1066-1357 pmcx_interface) and returns the same outputs: ``flux`` as an F-ordered
``[Nx, Ny, Nz, Nt]`` float32 array, ``detp`` as an F-ordered ``[reclen, ndetected]`` array and
``stat`` with runtime / nphoton / energytot / energyabs / normalizer / unitinmm / workload.
Internally it fills an MCX ``Config`` through ctypes, prepares it with ``mcxg_validatecfg`` and
calls the drop-in entry points ``mcx_list_gpu`` and ``mcx_run_simulation`` of libmcx_gb300.so,
exactly as pmcx drives MCX's own core.
"""

from __future__ import annotations

import ctypes as C
import os
from typing import Any

import numpy as np

from . import abi
from ._lib import lib, libc

# MCX's output-type letters (src/mcx_utils.c:150) and pmcx's long names
_OUTPUT_TYPES = {"x": 0, "flux": 0, "f": 1, "fluence": 1, "e": 2, "energy": 2, "j": 3, "jacobian": 3, "p": 4,
                 "nscat": 4, "m": 5, "r": 6, "l": 7, "length": 7, "s": 8, "t": 9, "b": 10}
SEED_FROM_FILE = -999
SEED_BYTES = 16          # xorshift128+ state saved per detected photon
_SRC_TYPES = ["pencil", "isotropic", "cone", "gaussian", "planar", "pattern", "fourier", "arcsine", "disk",
              "fourierx", "fourierx2d", "zgaussian", "line", "slit", "pencilarray", "pattern3d", "hyperboloid", "ring"]
_SAVEDET_CHARS = "dspmxvwi"      # detid, nscat, ppath, momentum, exit pos, exit dir, w0, iquv (src/mcx_utils.c)

_SCALARS_INT = ["nphoton", "nblocksize", "nthread", "maxdetphoton", "maxgate", "respin", "printnum", "maxvoidstep",
                "maxjumpdebug", "gscatter", "srcnum", "srcid", "replaydet", "gpuid", "voidtime"]
_DEBUG_CHARS = "RMPT"            # -D letters: RNG test, trajectories, progress, trajectories only (src/mcx_utils.c:159)
_SCALARS_FLOAT = ["tstart", "tstep", "tend", "sradius", "minenergy", "unitinmm", "omega", "lambda"]
_SCALARS_CHAR = ["isreflect", "isref3", "isrefint", "isnormalized", "issrcfrom0", "autopilot", "issaveref",
                 "issaveexit", "ismomentum", "isspecular", "issave2pt", "issavedet", "isgpuinfo", "isrowmajor",
                 "issaveseed", "faststep", "istrajstokes"]


class MCXError(RuntimeError):
    """An error reported by the engine (the MCX error id is in ``.id``)."""

    def __init__(self, id_: int, msg: str):
        super().__init__(f"MCX error {id_}: {msg}")
        self.id = id_


def _check(rc: int | None = None) -> None:
    eid = lib.mcxg_last_error_id()
    if eid:
        raise MCXError(eid, lib.mcxg_last_error().decode(errors="replace"))
    if rc:
        raise MCXError(rc, "engine call failed")


def _f2h_mcx(x: np.ndarray) -> np.ndarray:
    """float32 -> binary16 bits as MCX packs them (mcx_float2half2, src/mcx_utils.c:5490-5540):
    the mantissa truncated, values below 2^-14 handled by its denormal branch."""
    i = np.asarray(x, np.float32).view(np.uint32).astype(np.int64)
    m = (i >> 13) & 0x3FF
    e = (i >> 23) & 0xFF
    normal = e > 0x70
    h = np.where(normal, ((i >> 31) << 15) | (((e - 0x70) & 0x1F) << 10) | m, 0)
    sign = (i >> 16) & 0x8000
    md = ((i >> 12) & 0x7FF) | 0x800
    s1 = np.clip(114 - e, 0, 31)
    s2 = np.clip(113 - e, 0, 31)
    den = sign | ((md >> s1) + ((md >> s2) & 1))
    h = np.where(~normal & (m < 0x10), den, np.where(normal, h, ((i >> 31) << 15) | m))
    return (h & 0xFFFF).astype(np.uint32)


def pack_media(vol: np.ndarray, unitinmm: float = 1.0) -> tuple[np.ndarray, int]:
    """The 32-bit voxel words and MCX mediabyte of a volume, as pmcx and mcx_utils.c pack them
    (src/pmcx.cpp:120-380, src/mcx_utils.c:3537-3594):

      integer (nx, ny, nz)        labels (mediabyte 1, 2 or 4)
      float   (nx, ny, nz)        mua per voxel, MEDIA_MUA_FLOAT (101): float bits of mua x unitinmm,
                                  0 -> FLT_EPSILON (not void), NaN -> 0 (void)
      float   (2, nx, ny, nz)     mua, mus per voxel, MEDIA_AS_F2H (100): two binary16 halves
      float   (3, nx, ny, nz)     value, field (0-3: mua, mus, g, n) and label per voxel,
                                  MEDIA_LABEL_HALF (99): the label's properties with one field replaced
      float   (4, nx, ny, nz)     mua, mus, g, n per voxel, MEDIA_ASGN_F2H (96): four binary16 halves in
                                  two words per voxel (the second words follow all the first ones)
      uint8   (4, nx, ny, nz)     interpolation bytes for mua, mus, g, n, MEDIA_ASGN_BYTE (103)
      uint8   (8, nx, ny, nz)     split voxels, MEDIA_2LABEL_SPLIT (97): lower label, upper label, plane
                                  point x, y, z (0-255 across the voxel), plane normal x, y, z
                                  (0-255 for -1..1); two words per voxel as mcx_preprocess lays them out
      [u]int16 (2, nx, ny, nz)    interpolation shorts for mua, mus, MEDIA_AS_SHORT (104)
      [u]int16 (3, nx, ny, nz)    label 0, label 1 and the fraction (0-32767) of label 1 per voxel,
                                  MEDIA_2LABEL_MIX (98)

    The words come back as an (nx, ny, nz) array, or (nx, ny, nz, 2) for the two-word formats."""
    v = np.asarray(vol)
    if v.ndim == 3 and v.dtype.kind in "iub":
        return np.asfortranarray(v.astype(np.uint32, copy=False)), {1: 1, 2: 2, 4: 4, 8: 4}[v.dtype.itemsize]
    if v.ndim == 3 and v.dtype.kind == "f":
        f = (v.astype(np.float32) * np.float32(unitinmm)).astype(np.float32)
        w = f.view(np.uint32).copy()
        w[w == 0] = np.array(np.finfo(np.float32).eps, np.float32).view(np.uint32)
        w[np.isnan(f) | (w == 0x80000000)] = 0
        return np.asfortranarray(w), 101
    if v.ndim == 4 and v.dtype.kind == "f" and v.shape[0] == 2:
        mua = (v[0].astype(np.float32) * np.float32(unitinmm)).astype(np.float32)
        mus = (v[1].astype(np.float32) * np.float32(unitinmm)).astype(np.float32)
        w = _f2h_mcx(mua) | (_f2h_mcx(mus) << 16)
        w[np.isnan(mua) | np.isnan(mus)] = 0
        return np.asfortranarray(w.astype(np.uint32)), 100
    if v.ndim == 4 and v.dtype.kind == "f" and v.shape[0] == 3:
        # src/pmcx.cpp:266-300: [binary16 value][2-bit field | 14-bit label]; fields 1 and 2 are
        # scaled by unitinmm as pmcx scales them
        val, fld, lab = (v[k].astype(np.float32) for k in range(3))
        if (fld < 0).any() or (fld >= 4).any() or (lab < 0).any():
            raise MCXError(-4, "the 2nd volume must have an integer value between 0 and 3")
        val = np.where((fld >= 1) & (fld <= 2), val * np.float32(unitinmm), val).astype(np.float32)
        lo = ((fld.astype(np.uint8).astype(np.uint32) & 3) << 14) | (lab.astype(np.uint32) & 0xFFFF)
        w = (lo & 0xFFFF) | (_f2h_mcx(val).astype(np.uint32) << 16)
        return np.asfortranarray(w.astype(np.uint32)), 99
    if v.ndim == 4 and v.dtype.kind == "f" and v.shape[0] == 4:
        # src/pmcx.cpp:305-336: [mus][mua] halves (x unitinmm), then [n][g]; NaN mua / mus is void
        mua = (v[0].astype(np.float32) * np.float32(unitinmm)).astype(np.float32)
        mus = (v[1].astype(np.float32) * np.float32(unitinmm)).astype(np.float32)
        w0 = (_f2h_mcx(mua) | (_f2h_mcx(mus) << 16)).astype(np.uint32)
        w1 = (_f2h_mcx(v[2].astype(np.float32)) | (_f2h_mcx(v[3].astype(np.float32)) << 16)).astype(np.uint32)
        void = np.isnan(mua) | np.isnan(mus)
        w0[void] = 0
        w1[void] = 0
        return np.asfortranarray(np.stack([w0, w1], axis=-1)), 96
    if v.ndim == 4 and v.dtype in (np.int16, np.uint16) and v.shape[0] == 3:
        # src/pmcx.cpp:156-170: [15-bit fraction of label 1][label 1][label 0]
        b = v.astype(np.int64)
        w = (b[0] & 0xFF) | ((b[1] & 0xFF) << 8) | ((b[2] & 0x7FFF) << 16)
        return np.asfortranarray(w.astype(np.uint32)), 98
    if v.ndim == 4 and v.dtype == np.int16 and v.shape[0] == 2:
        b = v.astype(np.uint16).astype(np.uint32)
        return np.asfortranarray(b[0] | (b[1] << 16)), 104
    if v.ndim == 4 and v.dtype == np.uint8 and v.shape[0] == 8:
        # src/mcx_utils.c:1708-1731: [lower][upper][point x][point y], then [point z][normal x, y, z]
        b = v.astype(np.uint32)
        w0 = (b[0] << 24) | (b[1] << 16) | (b[2] << 8) | b[3]
        w1 = (b[4] << 24) | (b[5] << 16) | (b[6] << 8) | b[7]
        return np.asfortranarray(np.stack([w0, w1], axis=-1).astype(np.uint32)), 97
    if v.ndim == 4 and v.dtype == np.uint8 and v.shape[0] == 4:
        b = v.astype(np.uint32)
        return np.asfortranarray(b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24)), 103
    if v.ndim == 4 and v.dtype == np.uint16 and v.shape[0] == 2:
        b = v.astype(np.uint32)
        return np.asfortranarray(b[0] | (b[1] << 16)), 104
    raise MCXError(-4, "the 'vol' field must be a 3-D label array, a 3-D float mua array, or a 4-D per-voxel property array")


def _set_vec(dst, vals, n) -> None:
    vals = list(np.asarray(vals, dtype=np.float64).ravel())
    for i, name in enumerate("xyzw"[:n]):
        if i < len(vals):
            setattr(dst, name, vals[i])


class PreparedConfig:
    """A filled and validated ``Config`` plus the numpy buffers it points into."""

    def __init__(self, cfg: dict[str, Any], verbose: bool = False):
        self.c = abi.Config()
        lib.mcxg_initcfg(C.byref(self.c))
        self.keep: list[Any] = []
        c = self.c
        c.flog = C.c_void_p.in_dll(libc, "stderr").value if verbose else None
        for k in _SCALARS_INT:
            if k in cfg:
                setattr(c, k, int(float(cfg[k])))
        if "debuglevel" in cfg:
            # pmcx takes the -D letters (mcx_parsedebugopt, src/mcx_utils.c:5333-5348); a number is the bit mask
            d = cfg["debuglevel"]
            if isinstance(d, str) and not d.strip().isdigit():
                c.debuglevel = sum(1 << _DEBUG_CHARS.index(ch) for ch in set(d.upper()) if ch in _DEBUG_CHARS)
            else:
                c.debuglevel = int(d)
        for k in _SCALARS_FLOAT:
            if k in cfg:
                setattr(c, "lambda_" if k == "lambda" else k, float(cfg[k]))
        for k in _SCALARS_CHAR:
            if k in cfg:
                setattr(c, k, bytes([int(cfg[k]) & 0xFF]))
        self.seeds = None
        if "seed" in cfg:
            seed = cfg["seed"]
            if isinstance(seed, np.ndarray) or isinstance(seed, (list, tuple)):
                # replay: the seeds pmcx returns, (16, n) uint8 -- one column per detected photon
                sd = np.asarray(seed, dtype=np.uint8)
                if sd.ndim == 2 and sd.shape[0] == SEED_BYTES and sd.shape[1] != SEED_BYTES:
                    sd = sd.T
                # a private copy: mcxg_replayinit compacts it in place
                self.seeds = np.array(sd.reshape(-1, SEED_BYTES), dtype=np.uint8, order="C", copy=True)
                c.seed = SEED_FROM_FILE
                c.replay.seed = self.seeds.ctypes.data
                c.nphoton = self.seeds.shape[0]
            else:
                c.seed = int(seed)
        if "session" in cfg:
            c.session = str(cfg["session"]).encode()[: abi.SESSION_LEN - 1]
        if "srctype" in cfg:
            st = cfg["srctype"]
            c.srctype = bytes([_SRC_TYPES.index(st.lower()) if isinstance(st, str) else int(st)])
        if "outputtype" in cfg:
            ot = cfg["outputtype"]
            c.outputtype = bytes([_OUTPUT_TYPES[ot.lower()] if isinstance(ot, str) else int(ot)])
        if "savedetflag" in cfg:
            f = cfg["savedetflag"]
            if isinstance(f, str):
                f = sum(1 << _SAVEDET_CHARS.index(ch) for ch in f.lower() if ch in _SAVEDET_CHARS)
            c.savedetflag = int(f)
        if "bc" in cfg:
            c.bc = str(cfg["bc"]).encode()[:12]
        if "workload" in cfg:            # per-device photon shares (pmcx's cfg.workload)
            for i, x in enumerate(np.asarray(cfg["workload"], np.float32).reshape(-1)[: abi.MAX_DEVICE]):
                c.workload[i] = float(x)
        for key, n in (("srcpos", 4), ("srcdir", 4), ("srcparam1", 4), ("srcparam2", 4), ("srciquv", 4)):
            if key in cfg:
                _set_vec(getattr(c, key), np.asarray(cfg[key], np.float64).reshape(-1)[:4]
                         if np.ndim(cfg[key]) < 2 else np.asarray(cfg[key])[0], n)
        # several sources: rows 1.. of srcpos / srcdir / srcparam1 / srcparam2 (src/pmcx.cpp:470-600)
        nsrc = max((len(cfg[k]) for k in ("srcpos", "srcdir", "srcparam1", "srcparam2")
                    if k in cfg and np.ndim(cfg[k]) == 2), default=1)
        if nsrc > 1:
            self.srcdata = (abi.ExtraSrc * (nsrc - 1))()
            for k, field in (("srcpos", "srcpos"), ("srcdir", "srcdir"), ("srcparam1", "srcparam1"), ("srcparam2", "srcparam2")):
                if k in cfg and np.ndim(cfg[k]) == 2:
                    rows = np.asarray(cfg[k], np.float64)
                    for i in range(1, min(nsrc, len(rows))):
                        _set_vec(getattr(self.srcdata[i - 1], field), rows[i], 4)
            c.srcdata = C.addressof(self.srcdata)
            c.extrasrclen = nsrc - 1
        if "steps" in cfg:
            _set_vec(c.steps, cfg["steps"], 3)
        if "polprop" in cfg and cfg["polprop"] is not None and np.asarray(cfg["polprop"]).size:
            # sphere populations of the polarised media, one row per medium after the background:
            # mua, radius (um), number density (1/um^3), sphere and background indices (src/pmcx.cpp:689-725)
            pp = np.asarray(cfg["polprop"], dtype=np.float32).reshape(-1, 5)
            self.polprop = (abi.POLMedium * len(pp))(*[abi.POLMedium(*map(float, r)) for r in pp])
            c.polprop = C.addressof(self.polprop)
            c.polmedianum = len(pp)
        if cfg.get("invcdf") is not None and np.asarray(cfg["invcdf"]).size:
            # user phase function: the inverse CDF of cos(theta) between the ends -1 and 1 that
            # pmcx adds (src/pmcx.cpp:843-866)
            inv = np.asarray(cfg["invcdf"], np.float32).ravel(order="F")
            if (inv < -1).any() or (inv > 1).any() or (np.diff(inv) < 0).any():
                raise MCXError(-4, "cfg.invcdf contains invalid data; it must be a monotonically increasing vector with all values between -1 and 1")
            tab = np.concatenate([[-1.0], inv, [1.0]]).astype(np.float32)
            self.keep.append(tab)
            c.invcdf = tab.ctypes.data
            c.nphase = tab.size
        if cfg.get("angleinvcdf") is not None and np.asarray(cfg["angleinvcdf"]).size:
            # launch zenith angles / pi as an inverse CDF (src/pmcx.cpp:868-890)
            ang = np.ascontiguousarray(np.asarray(cfg["angleinvcdf"], np.float32).ravel(order="F"))
            if (ang < 0).any() or (ang > 1).any() or (np.diff(ang) < 0).any():
                raise MCXError(-4, "cfg.angleinvcdf contains invalid data; it must be a monotonically increasing vector with all values between 0 and 1")
            self.keep.append(ang)
            c.angleinvcdf = ang.ctypes.data
            c.nangle = ang.size
        if "srcpattern" in cfg and cfg["srcpattern"] is not None:
            # x fastest, as pmcx passes a (param1.w, param2.w) or (nx, ny, nz) array (src/pmcx.cpp)
            pat = np.asarray(cfg["srcpattern"], dtype=np.float32).ravel(order="F").copy()
            self.keep.append(pat)
            c.srcpattern = pat.ctypes.data

        if "vol" not in cfg or "prop" not in cfg:
            raise MCXError(-4, "the 'vol' and 'prop' fields are required")
        vol = np.asarray(cfg["vol"])
        if vol.ndim == 3 and vol.dtype.kind in "iub" and vol.flags.c_contiguous and not int(cfg.get("isrowmajor", 0)):
            # C-ordered labels: widened in their own order, and the engine's preparation transposes
            # them to MCX's x-fastest order (MCX's isrowmajor input, src/mcx_utils.c:1620-1631)
            vol32 = vol.astype(np.uint32).reshape(-1)
            mediabyte = {1: 1, 2: 2, 4: 4, 8: 4}[vol.dtype.itemsize]
            c.dim.x, c.dim.y, c.dim.z = (int(s) for s in vol.shape)
            c.isrowmajor = b"\x01"
        else:
            words, mediabyte = pack_media(vol, float(cfg.get("unitinmm", 1.0)))
            vol32 = words.ravel(order="F").copy()
            c.dim.x, c.dim.y, c.dim.z = (int(s) for s in words.shape[:3])
        c.mediabyte = mediabyte
        self.vol = vol32
        c.vol = vol32.ctypes.data

        # a private copy: preparation rewrites the rows of polarised media in place
        prop = np.array(cfg["prop"], dtype=np.float32).reshape(-1, 4)
        self.prop = prop
        c.prop = prop.ctypes.data
        c.medianum = prop.shape[0]

        if "detpos" in cfg and np.asarray(cfg["detpos"]).size:
            dp = np.asarray(cfg["detpos"], dtype=np.float32)
            dp = dp.reshape(-1, dp.shape[-1]) if dp.ndim > 1 else dp.reshape(1, -1)
            if dp.shape[1] == 3:
                dp = np.hstack([dp, np.full((dp.shape[0], 1), float(cfg.get("detradius", 1.0)), np.float32)])
            self.detpos = np.ascontiguousarray(dp[:, :4])
            c.detpos = self.detpos.ctypes.data
            c.detnum = self.detpos.shape[0]
        else:
            self.detpos = None
            c.detnum = 0
        if "issavedet" not in cfg and c.detnum == 0:
            c.issavedet = b"\x00"

        lib.mcxg_clear_error()
        rc = lib.mcxg_validatecfg(C.byref(c))
        _check(rc)
        if self.seeds is not None:
            if "detphotons" not in cfg:
                raise MCXError(-6, "you give cfg.seed for replay, but did not specify cfg.detphotons")
            dp = np.asarray(cfg["detphotons"], dtype=np.float32)
            dims = (C.c_int * 2)(dp.shape[0], dp.shape[1])
            self.detps = np.ascontiguousarray(dp.T)       # one detected record after another
            _check(lib.mcxg_replayinit(C.byref(c), self.detps.ctypes.data_as(C.POINTER(C.c_float)), dims, SEED_BYTES))
            # MCX allocates these with malloc; they live as long as this object
            self._replay_bufs = (c.replay.weight, c.replay.tof, c.replay.detid)

    def __del__(self):
        # replay buffers mcxg_replayinit allocated with malloc (MCX frees them in mcx_clearcfg)
        c = getattr(self, "c", None)
        if c is not None and getattr(self, "seeds", None) is not None:
            for name in ("weight", "tof", "detid"):
                ptr = getattr(c.replay, name)
                if ptr:
                    libc.free(C.c_void_p(ptr))
                    setattr(c.replay, name, None)
        # the Mueller tables the polarised-media preparation allocated with malloc
        if c is not None and c.smatrix:
            libc.free(C.c_void_p(c.smatrix))
            c.smatrix = None

    @property
    def dims(self) -> tuple[int, int, int]:
        return int(self.c.dim.x), int(self.c.dim.y), int(self.c.dim.z)

    @property
    def ngates(self) -> int:
        return max(1, int((self.c.tend - self.c.tstart) / self.c.tstep + 0.5))

    @property
    def reclen(self) -> int:
        return int(self.c.his.colcount)


def prepare(cfg: dict[str, Any], verbose: bool = False) -> PreparedConfig:
    """Fill and validate a Config (no GPU needed); the oracle consumes the same object."""
    return PreparedConfig(cfg, verbose=verbose)


def gpuinfo() -> list[dict[str, Any]]:
    """Device list as ``pmcx.gpuinfo()`` reports it (src/pmcx.cpp:1404)."""
    c = abi.Config()
    lib.mcxg_initcfg(C.byref(c))
    c.flog = None
    c.isgpuinfo = bytes([3])
    info = C.POINTER(abi.GPUInfo)()
    lib.mcxg_clear_error()
    n = lib.mcx_list_gpu(C.byref(c), C.byref(info))
    _check()
    out = []
    if info:
        count = info[0].devcount if n else 0
        for i in range(count):
            g = info[i]
            out.append({f[0]: (getattr(g, f[0]).decode() if f[0] == "name" else getattr(g, f[0]))
                        for f in abi.GPUInfo._fields_ if not f[0].startswith("_pad")})
        libc.free(info)
    return out


def run(cfg: dict[str, Any], verbose: bool = False, fp64_field: bool = False,
        devices: list[int] | None = None) -> dict[str, Any]:
    """Run one simulation on the GPU; same inputs and outputs as ``pmcx.run``.

    ``fp64_field`` accumulates the fluence in FP64 on the device (the reference-accuracy twin of
    the FP32 production path, used to state its accumulation error).  ``devices`` lists the
    0-based CUDA devices to split the photons over (MCX's multi-GPU run; a device may be listed
    more than once), in place of ``gpuid``; ``cfg["workload"]`` weights their shares."""
    pc = prepare(cfg, verbose=verbose)
    return run_prepared(pc, fp64_field=fp64_field, devices=devices)


def _active_devices(c) -> None:
    """mcx_list_gpu compacts cfg.deviceid into the active-device list, as the front-ends call it."""
    info = C.POINTER(abi.GPUInfo)()
    lib.mcxg_clear_error()
    nact = lib.mcx_list_gpu(C.byref(c), C.byref(info))
    _check()
    return nact, info


def _srctype_code(c) -> int:
    v = c.srctype
    return v[0] if isinstance(v, bytes) else int(v)


def _attach_field(pc: PreparedConfig):
    c = pc.c
    nx, ny, nz = pc.dims
    maxgate = pc.ngates if c.maxgate == 0 else min(int(c.maxgate), pc.ngates)
    if int(c.seed) == SEED_FROM_FILE and int(c.replaydet) == -1:
        maxgate *= max(1, int(c.detnum))     # one block of gates per detector
    if ord(c.outputtype) in (6, 8):
        maxgate *= 2                         # RF replay: real blocks, then imaginary blocks
    if int(c.extrasrclen) and int(c.srcid) < 0:
        maxgate *= int(c.extrasrclen) + 1    # every source apart: one block of gates per source
    # photon sharing: one channel per pattern, adjacent per voxel (src/mcx_core.cu:2782)
    pc.chans = int(c.srcnum) if (_srctype_code(c) in (5, 15) and int(c.srcnum) > 1) else 1
    flux = None
    if c.issave2pt != b"\x00":
        flux = np.zeros(nx * ny * nz * maxgate * pc.chans, dtype=np.float32)
        c.exportfield = flux.ctypes.data
    return flux, maxgate


def _take_seeds(pc: PreparedConfig):
    """The saved seeds of the detected photons, (16, n) uint8 as pmcx returns them."""
    c = pc.c
    ptr = c.seeddata
    if not ptr:
        return None
    n = int(c.detectedcount)
    seeds = None
    if n and c.issaveseed != b"\x00":
        buf = (C.c_uint8 * (SEED_BYTES * n)).from_address(ptr)
        seeds = np.frombuffer(buf, dtype=np.uint8).copy().reshape(n, SEED_BYTES).T
    libc.free(C.c_void_p(ptr))
    c.seeddata = None
    return seeds


def _take_traj(pc: PreparedConfig):
    """Trajectory records (-D M / T) as pmcx's `traj`: float32 [6, n], rows id (uint32 bits), x, y, z,
    weight, source id."""
    c = pc.c
    ptr, n = c.exportdebugdata, int(c.debugdatalen)
    traj = None
    if ptr:
        rl = 10 if c.istrajstokes != b"\x00" else 6          # with the Stokes vector: 10 floats
        buf = (C.c_float * (rl * n)).from_address(ptr) if n else None
        traj = np.frombuffer(buf, dtype=np.float32).copy().reshape((rl, n), order="F") if n else np.zeros((rl, 0), np.float32)
        libc.free(C.c_void_p(ptr))
        c.exportdebugdata = None
        c.debugdatalen = 0
    elif int(c.debuglevel) & 10:
        traj = np.zeros((6, 0), np.float32)
    return traj


def _take_detected(pc: PreparedConfig):
    c = pc.c
    det_ptr = c.exportdetected
    ndet = int(c.detectedcount)
    detp = None
    if det_ptr:
        reclen = pc.reclen
        if ndet and reclen:
            buf = (C.c_float * (reclen * ndet)).from_address(det_ptr)
            detp = np.frombuffer(buf, dtype=np.float32).copy().reshape((reclen, ndet), order="F")
        libc.free(C.c_void_p(det_ptr))
        c.exportdetected = None
    return detp


def _result(pc: PreparedConfig, flux, maxgate, detp, st) -> dict[str, Any]:
    c = pc.c
    nx, ny, nz = pc.dims
    out: dict[str, Any] = {}
    if flux is not None:
        ch = getattr(pc, "chans", 1)
        # pmcx's shape: photon-sharing channels folded into the first axis, (srcnum * nx, ny, nz, nt)
        out["flux"] = flux.reshape((ch * nx, ny, nz, maxgate), order="F")
        c.exportfield = None
        if c.issaveref != b"\x00":
            # diffuse reflectance as pmcx splits it off (src/pmcx.cpp:1268-1290): the negated field
            # in void voxels, which the fluence then leaves at zero
            void = (pc.vol[:nx * ny * nz] == 0).reshape((nx, ny, nz), order="F")
            f5 = flux.reshape((ch, nx, ny, nz, maxgate), order="F")
            d5 = np.zeros_like(f5)
            d5[:, void] = -f5[:, void]
            f5[:, void] = 0.0
            out["dref"] = d5.reshape((ch * nx, ny, nz, maxgate), order="F")
            out["flux"] = f5.reshape((ch * nx, ny, nz, maxgate), order="F")
    if c.issavedet != b"\x00" and detp is not None:
        out["detp"] = detp
    out["stat"] = {
        "runtime": int(c.runtime),
        "nphoton": int(c.nphoton) * (int(c.respin) if c.respin > 1 else 1),
        "energytot": float(c.energytot),
        "energyabs": float(c.energyabs),
        "normalizer": float(c.normalizer),
        "unitinmm": float(c.unitinmm),
        "workload": [1.0],
        "detected": int(c.his.detected),
        # beyond pmcx: FP64 tallies and the GPU's own counters
        "e_launch": st.e_launch, "e_escape": st.e_escape, "e_detect": st.e_detect,
        "e_absdep": st.e_absdep, "e_absother": st.e_absother,
        "n_steps": st.n_steps, "n_scatter": st.n_scatter, "n_deposit": st.n_deposit,
        "n_launch": st.n_launch, "n_photon": st.n_photon, "n_detected": st.n_detected,
        "n_tile_deposit": st.n_tile_deposit, "kernel_ms": st.kernel_ms, "total_ms": st.total_ms,
        "grid": st.grid, "block": st.block, "chunk": st.chunk, "launches": st.launches,
        "error_flags": st.error_flags,
    }
    return out


def run_prepared(pc: PreparedConfig, fp64_field: bool = False, devices: list[int] | None = None) -> dict[str, Any]:
    c = pc.c
    nact, info = _active_devices(c)
    if nact == 0:
        if info:
            libc.free(info)
        raise MCXError(-1, "no active GPU device found")
    if devices:
        if len(devices) > abi.MAX_DEVICE - 1:
            raise MCXError(-1, "too many devices")
        ids = bytes(int(d) + 1 for d in devices)
        C.memmove(C.addressof(c) + abi.Config.deviceid.offset, ids + b"\x00", len(ids) + 1)
    flux, maxgate = _attach_field(pc)
    try:
        (lib.mcxg_run_simulation_fp64 if fp64_field else lib.mcx_run_simulation)(C.byref(c), info)
        _check()
    finally:
        libc.free(info)
        seeds = _take_seeds(pc)
        detp = _take_detected(pc)
        traj = _take_traj(pc)
    st = abi.Stats()
    lib.mcxg_get_stats(C.byref(st))
    out = _result(pc, flux, maxgate, detp, st)
    if seeds is not None:
        out["seeds"] = seeds
    if traj is not None:
        out["traj"] = traj
    return out


def run_batch(cfgs: list[dict[str, Any]], streams: int = 4, device_fields: list | None = None
              ) -> tuple[list[dict[str, Any]], float]:
    """Run many independent simulations in one CUDA graph on one GPU (``mcxg_run_batch``).

    Returns the per-simulation results -- the same dicts ``run`` gives -- and the graph time in
    ms (all waves: repetitions and gate groups run as further graphs).

    ``device_fields``: one contiguous float32 CUDA tensor per simulation (or None for a host
    field), of the simulation's field size (nx * ny * nz * gates); the normalised fluence is
    stored there on the device (``mcxg_run_batch_device``) and the result has no ``flux``.  Each
    such simulation runs one repetition of one gate group."""
    if len(cfgs) > 1:
        # the preparations are independent and spend their time in numpy copies and the engine's
        # host preparation, both of which run without the interpreter lock
        from concurrent.futures import ThreadPoolExecutor

        with ThreadPoolExecutor(max_workers=min(8, len(cfgs), os.cpu_count() or 1)) as ex:
            pcs = list(ex.map(prepare, cfgs))
    else:
        pcs = [prepare(cfg) for cfg in cfgs]
    for pc in pcs:
        nact, info = _active_devices(pc.c)
        if info:
            libc.free(info)
        if nact == 0:
            raise MCXError(-1, "no active GPU device found")
    if device_fields is not None and len(device_fields) != len(pcs):
        raise MCXError(-4, f"{len(device_fields)} device fields for {len(pcs)} simulations")
    fields, ptrs = [], None
    if device_fields is not None:
        ptrs = (C.c_void_p * len(pcs))()
    for i, pc in enumerate(pcs):
        dev = None if device_fields is None else device_fields[i]
        if dev is None:
            fields.append(_attach_field(pc))
            continue
        flux, maxgate = _attach_field(pc)
        pc.c.exportfield = None
        if flux is None:
            raise MCXError(-4, "a device field was given for a simulation that saves no field")
        if not (getattr(dev, "is_cuda", False) and dev.dtype.is_floating_point and dev.element_size() == 4
                and dev.is_contiguous() and dev.numel() == flux.size):
            raise MCXError(-4, f"device field {i} must be a contiguous float32 CUDA tensor of {flux.size} elements")
        ptrs[i] = dev.data_ptr()
        fields.append((None, maxgate))
    arr = (C.POINTER(abi.Config) * len(pcs))(*[C.pointer(pc.c) for pc in pcs])
    stats = (abi.Stats * len(pcs))()
    ms = C.c_double(0.0)
    try:
        if ptrs is None:
            _check(lib.mcxg_run_batch(arr, len(pcs), int(streams), stats, C.byref(ms)))
        else:
            _check(lib.mcxg_run_batch_device(arr, len(pcs), int(streams), ptrs, stats, C.byref(ms)))
    finally:
        for pc in pcs:
            _take_seeds(pc)
        dets = [_take_detected(pc) for pc in pcs]
        trajs = [_take_traj(pc) for pc in pcs]
    out = [_result(pc, f, g, d, stats[i]) for i, (pc, (f, g), d) in enumerate(zip(pcs, fields, dets))]
    for o, t in zip(out, trajs):
        if t is not None:
            o["traj"] = t
    return out, float(ms.value)


def version() -> str:
    return "mcx-gb300 0.1 (MCX v2025.10 compatible)"
