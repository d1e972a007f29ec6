"""Recipe and driver for the reference MCX CUDA build (the speed bar and a statistical oracle).

MCX's transport exists only as CUDA (src/mcx_core.cu); on a GB300 the reference itself is that
file compiled for sm_103a with the shipped configuration (xorshift128+, `-DUSE_ATOMIC
-DSAVE_DETECTORS -use_fast_math`, src/Makefile's `fermi` target).  This module

  stage()  copies the reference's src/ tree from a reference checkout into baseline/_ref/src
           (git-ignored: an install of the reference, never part of this repository's history);
  build()  compiles baseline/_ref/src into baseline/_ref/bin/mcx with nvcc and gcc directly
           (the reference's own makefiles are not run);
  run()    writes an MCX JSON input for a workload dict of mcx_gb300.problems, runs the binary
           and returns its own speed report, energies, the flux (.mc2) and detected photons
           (.mch).

Test and benchmark infrastructure only: the engine never calls it.
"""

from __future__ import annotations

import json
import os
import platform
import re
import shutil
import struct
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path
from typing import Any

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
REF = ROOT / "baseline" / "_ref"
SRC = REF / "src"
BIN = REF / "bin" / "mcx"

C_FILES = ["mcx_utils.c", "mcx_shapes.c", "mcx_tictoc.c", "mcx.c", "mcx_bench.c", "mcx_lang.c", "cjson/cJSON.c",
           "ubj/ubjw.c"]
CPP_FILES = ["mcx_neurojson.cpp", "mcx_mie.cpp"]
ZMAT_FILES = ["zmat/zmatlib.c", "zmat/miniz/miniz.c", "zmat/lz4/lz4.c", "zmat/lz4/lz4hc.c"]


def reference_root(reference: str | Path | None = None) -> Path:
    """The reference checkout: the argument, else the MCX_REFERENCE_ROOT environment variable."""
    root = reference or os.environ.get("MCX_REFERENCE_ROOT")
    if not root:
        raise RuntimeError("name the MCX checkout: stage(<path>), `ref_mcx.py stage <path>` or MCX_REFERENCE_ROOT=<path>")
    return Path(root)


def stage(reference: str | Path | None = None) -> Path:
    """Copy the reference's src/ tree into baseline/_ref/src (run where the checkout exists)."""
    src = reference_root(reference) / "src"
    if SRC.exists():
        shutil.rmtree(SRC)
    SRC.parent.mkdir(parents=True, exist_ok=True)
    shutil.copytree(src, SRC, ignore=shutil.ignore_patterns("*.o", "*.a", "pybind11", "mcx_doxygen.cfg"))
    for p in SRC.rglob("*"):
        if p.is_file():
            p.chmod(0o644)
    return SRC


def available() -> bool:
    return SRC.exists() and (SRC / "mcx_core.cu").exists()


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return Path(nvcc).resolve().parent.parent


def _run(cmd: list[str], cwd: Path) -> None:
    p = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("reference build step failed:\n" + " ".join(cmd) + "\n" + p.stdout[-3000:] + p.stderr[-3000:])


def _object_jobs(with_core: bool) -> tuple[list[list[str]], list[Path]]:
    """Compile commands and objects of the reference's `mcx` binary: its CUDA translation unit
    (src/mcx_core.cu) when `with_core`, and its host files (CLI, input parsing, output writers)."""
    if not available():
        raise RuntimeError("the reference sources are not staged in baseline/_ref/src")
    cuda = _cuda_home()
    obj = REF / "obj"
    stamp = obj / "machine.txt"
    if stamp.exists() and stamp.read_text() != platform.machine():
        shutil.rmtree(obj)          # objects of another host architecture
    obj.mkdir(parents=True, exist_ok=True)
    stamp.write_text(platform.machine())
    inc = ["-Izmat", "-Izmat/easylzma", "-Izmat/miniz", "-Iubj", f"-I{cuda}/include"]
    jobs = []
    objs = []
    if with_core:
        o = obj / "mcx_core.o"
        objs.append(o)
        jobs.append([str(cuda / "bin" / "nvcc"), "-c", "-DUSE_ATOMIC", "-use_fast_math", "-DSAVE_DETECTORS",
                     "-arch=sm_103a", "-Xcompiler", "-fopenmp", "-DMCX_TARGET_NAME=\"Kilo-Kelvin\"", "-lineinfo", *inc,
                     "-o", str(o), "mcx_core.cu"])
    for f in C_FILES:
        o = obj / (f.replace("/", "_") + ".o")
        objs.append(o)
        jobs.append(["gcc", "-std=c99", "-g", "-fopenmp", *inc, "-c", "-o", str(o), f])
    for f in CPP_FILES:
        o = obj / (f.replace("/", "_") + ".o")
        objs.append(o)
        jobs.append(["g++", "-g", "-fopenmp", *inc, "-c", "-o", str(o), f])
    lzma = sorted(str(p.relative_to(SRC)) for p in (SRC / "zmat" / "easylzma").rglob("*.c"))
    for f in ZMAT_FILES + lzma:
        o = obj / (f.replace("/", "_") + ".o")
        objs.append(o)
        jobs.append(["gcc", "-O3", "-fPIC", "-DNO_ZLIB", "-DNO_ZSTD", "-DNO_BLOSC2", *inc, "-Izmat/easylzma/pavlov",
                     "-c", "-o", str(o), f])
    # objects already built from the same sources are kept (the CUDA file dominates the build)
    return [j for j in jobs if not Path(j[j.index("-o") + 1]).exists()], objs


def _compile(jobs: list[list[str]]) -> None:
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(lambda c: _run(c, SRC), jobs))


def build(force: bool = False) -> Path:
    """Compile the reference `mcx` binary for sm_103a from baseline/_ref/src."""
    if BIN.exists() and not force:
        return BIN
    jobs, objs = _object_jobs(with_core=True)
    _compile(jobs)
    BIN.parent.mkdir(parents=True, exist_ok=True)
    _run(["g++", "-o", str(BIN), *map(str, objs), "-fopenmp", f"-L{_cuda_home()}/lib64", "-lcudart_static", "-ldl",
          "-lrt", "-lpthread", "-lm"], SRC)
    return BIN


FRONTEND_BIN = REF / "bin" / "mcx_on_gb300"


def build_frontend(engine_lib: str | Path, force: bool = False) -> Path:
    """MCX's own command-line front-end (src/mcx.c with the unchanged input parsing, output
    writers and error handler of src/mcx_utils.c and their helpers) linked against the GB300
    engine's shared library in place of the reference's src/mcx_core.cu: the drop-in boundary
    (mcx_run_simulation / mcx_list_gpu, src/mcx_core.h:200-201) exercised by the real caller.
    The executable exports its symbols so the engine's weak mcx_error / mcx_savedata /
    mcx_savedetphoton references bind to the front-end's own."""
    engine_lib = Path(engine_lib).resolve()
    if FRONTEND_BIN.exists() and not force and FRONTEND_BIN.stat().st_mtime >= engine_lib.stat().st_mtime:
        return FRONTEND_BIN
    jobs, objs = _object_jobs(with_core=False)
    _compile(jobs)
    FRONTEND_BIN.parent.mkdir(parents=True, exist_ok=True)
    # only the front-end's handlers are exported to the engine; the CUDA runtime the front-end's
    # timer (src/mcx_tictoc.c) links stays private to the executable
    dyn = REF / "obj" / "frontend_exports.txt"
    dyn.write_text("{ mcx_error; mcx_savedata; mcx_savedetphoton; };\n")
    _run(["g++", "-o", str(FRONTEND_BIN), *map(str, objs), "-fopenmp", f"-Wl,--dynamic-list={dyn}", str(engine_lib),
          f"-Wl,-rpath,{engine_lib.parent}", f"-L{_cuda_home()}/lib64", "-lcudart_static", "-ldl", "-lrt", "-lpthread",
          "-lm"], SRC)
    return FRONTEND_BIN


MIE_LIB = REF / "lib" / "libmcxmie.so"

# mcx_mie.cpp reports bad sizes through MCX's error handler; the library gets this one instead
_MIE_STUB = r"""
#include <stdio.h>
#include <stdlib.h>
extern "C" void mcx_error(const int id, const char* msg, const char* file, const int linenum) {
    fprintf(stderr, "mcx_error %d: %s (%s:%d)\n", id, msg, file, linenum);
    exit(1);
}
"""


def build_mie(force: bool = False) -> Path:
    """Compile the reference's Mie routines (src/mcx_mie.cpp, ``Mie`` and ``small_Mie``) into a
    host shared library, so the Mueller tables of polarised media can be checked without a GPU."""
    if MIE_LIB.exists() and not force:
        return MIE_LIB
    if not (SRC / "mcx_mie.cpp").exists():
        raise RuntimeError("the reference sources are not staged in baseline/_ref/src")
    obj = REF / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    stub = obj / "mie_error_stub.cpp"
    stub.write_text(_MIE_STUB)
    MIE_LIB.parent.mkdir(parents=True, exist_ok=True)
    _run(["g++", "-O2", "-shared", "-fPIC", f"-I{_cuda_home() / 'include'}", "-o", str(MIE_LIB), "mcx_mie.cpp",
          str(stub)], SRC)
    return MIE_LIB


_SRC_NAMES = ["pencil", "isotropic", "cone", "gaussian", "planar", "pattern", "fourier", "arcsine", "disk",
              "fourierx", "fourierx2d", "zgaussian", "line", "slit", "pencilarray", "pattern3d", "hyperboloid", "ring"]


def _src_name(t) -> str:
    """MCX's source-type keyword (src/mcx_utils.c:211)."""
    return t.lower() if isinstance(t, str) else _SRC_NAMES[int(t)]


def _json_input(cfg: dict[str, Any], session: str, volfile: str) -> dict:
    vol = np.asarray(cfg["vol"])
    prop = np.asarray(cfg["prop"], dtype=float)
    flag = cfg.get("savedetflag", "dp")
    issavedet = int(cfg.get("issavedet", 1 if "detpos" in cfg else 0))
    session_keys = {
        "ID": session, "Photons": int(cfg["nphoton"]), "RNGSeed": int(cfg.get("seed", 1648335518)),
        "DoMismatch": int(cfg.get("isreflect", 1)), "DoSaveVolume": 1, "DoNormalize": 1,
        "DoPartialPath": issavedet, "OutputFormat": "mc2", "OutputType": "x", "DoAutoThread": 1,
        "SaveDataMask": flag if isinstance(flag, str) else int(flag),
    }
    if "maxdetphoton" in cfg:
        session_keys["MaxDetPhoton"] = int(cfg["maxdetphoton"])
    if cfg.get("issaveseed"):
        session_keys["DoSaveSeed"] = 1
    if cfg.get("issaveref"):
        session_keys["DoSaveRef"] = int(cfg["issaveref"])
    if cfg.get("debuglevel"):
        session_keys["DebugFlag"] = str(cfg["debuglevel"])       # -D letters, e.g. "M" for trajectories
    svmc = vol.ndim == 4 and vol.dtype == np.uint8 and vol.shape[0] == 8
    out = {
        "Session": session_keys,
        "Domain": {"Dim": list(vol.shape[1:] if svmc else vol.shape), "OriginType": 1 if cfg.get("issrcfrom0", 0) else 0,
                   "LengthUnit": float(cfg.get("unitinmm", 1.0)),
                   "MediaFormat": "svmc" if svmc else "byte", "VolumeFile": volfile,
                   "Media": [{"mua": float(r[0]), "mus": float(r[1]), "g": float(r[2]), "n": float(r[3])} for r in prop]},
        "Forward": {"T0": float(cfg["tstart"]), "T1": float(cfg["tend"]), "Dt": float(cfg["tstep"])},
        "Optode": {"Source": {"Type": _src_name(cfg.get("srctype", "pencil")),
                              "Pos": [float(x) for x in cfg["srcpos"][:3]],
                              "Dir": [float(x) for x in list(cfg["srcdir"])[:4]]}},
    }
    for key, name in (("srcparam1", "Param1"), ("srcparam2", "Param2")):
        if key in cfg:
            out["Optode"]["Source"][name] = [float(x) for x in cfg[key]]
    if cfg.get("srcpattern") is not None:
        # Optode.Source.Pattern {Nx, Ny, Nz, Data} with SrcNum patterns interleaved per pixel
        # (src/mcx_utils.c:2878, 2906-2935)
        pat = np.asarray(cfg["srcpattern"], np.float32)
        ns = int(cfg.get("srcnum", 1))
        shape = pat.shape[1:] if ns > 1 else pat.shape
        dims = list(shape) + [1] * (3 - len(shape))
        out["Optode"]["Source"]["SrcNum"] = ns
        out["Optode"]["Source"]["Pattern"] = {"Nx": int(dims[0]), "Ny": int(dims[1]), "Nz": int(dims[2]),
                                              "Data": [float(x) for x in pat.ravel(order="F")]}
    if "detpos" in cfg and np.asarray(cfg["detpos"]).size:
        out["Optode"]["Detector"] = [{"Pos": [float(d[0]), float(d[1]), float(d[2])], "R": float(d[3])}
                                     for d in np.asarray(cfg["detpos"], float).reshape(-1, 4)]
    if "bc" in cfg:
        out["Session"]["BCFlags"] = cfg["bc"]
    if cfg.get("invcdf") is not None:
        # user phase function (src/mcx_utils.c:2456-2475; MCX adds the ends -1 and 1)
        out["Domain"]["InverseCDF"] = [float(x) for x in np.asarray(cfg["invcdf"], float).ravel()]
    if "polprop" in cfg and np.asarray(cfg["polprop"]).size:
        # polarised media: Domain.MieScatter, Optode.Source.WaveLength / IQUV (src/mcx_utils.c:2360-2400, 2731, 2873)
        out["Domain"]["MieScatter"] = [{"mua": float(r[0]), "radius": float(r[1]), "rho": float(r[2]),
                                        "nsph": float(r[3]), "nmed": float(r[4])}
                                       for r in np.asarray(cfg["polprop"], float).reshape(-1, 5)]
        out["Optode"]["Source"]["WaveLength"] = float(cfg["lambda"])
        if "srciquv" in cfg:
            out["Optode"]["Source"]["IQUV"] = [float(x) for x in cfg["srciquv"]]
    return out


def run(cfg: dict[str, Any], workdir: str | Path | None = None, keep_field: bool = True,
        timeout: float = 900.0) -> dict[str, Any]:
    """Run the reference binary on a workload dict; returns its speed report, energies, flux
    (F-ordered [Nx,Ny,Nz,Nt], normalised as MCX normalises) and detected records."""
    exe = build()
    tmp = (Path(workdir) if workdir else Path(tempfile.mkdtemp(prefix="mcxref_"))).resolve()
    tmp.mkdir(parents=True, exist_ok=True)
    vol = np.asarray(cfg["vol"]).astype(np.uint8)
    volfile = tmp / "vol.bin"
    if vol.ndim == 4 and vol.shape[0] == 8:
        # split voxels (MediaFormat "svmc", src/mcx_utils.c:3527, 1708-1731): 8 bytes per voxel,
        # [lower label, upper label, plane point x, y, z, normal x, y, z], voxels x fastest
        vol.reshape(8, -1, order="F").T.copy().tofile(volfile)
        vol = vol[0]
    else:
        vol.ravel(order="F").tofile(volfile)
    session = "ref"
    (tmp / "in.json").write_text(json.dumps(_json_input(cfg, session, str(volfile))))
    p = subprocess.run([str(exe), "-f", "in.json"], cwd=tmp, capture_output=True, text=True, timeout=timeout)
    log = p.stdout + p.stderr
    # the CLI writes its report to <session>.log (the session is unnamed when the log opens)
    for lf in sorted(tmp.glob("*.log")):
        log += lf.read_text(errors="replace")
    if p.returncode != 0:
        raise RuntimeError(f"reference mcx failed ({p.returncode}):\n{log[-3000:]}")
    clean = re.sub(r"\x1b\[[0-9;]*m", "", log)
    res: dict[str, Any] = {"log": clean}
    m = re.search(r"MCX simulation speed:\s*([0-9.]+)\s*photon/ms", clean)
    res["speed"] = float(m.group(1)) if m else None
    m = re.search(r"kernel complete:\s*([0-9]+)\s*ms", clean)
    res["kernel_ms_cum"] = int(m.group(1)) if m else None
    m = re.search(r"data normalization complete\s*:\s*([0-9]+)\s*ms", clean)
    res["normalized_ms"] = int(m.group(1)) if m else None
    m = re.search(r"total simulated energy:\s*([0-9.]+)\s*absorbed:\s*([0-9.]+)%", clean)
    if m:
        res["energytot"] = float(m.group(1))
        res["absorbed"] = float(m.group(2)) / 100.0
    m = re.search(r"detected\s+([0-9]+)\s+photons", clean)
    res["detected"] = int(m.group(1)) if m else 0
    m = re.search(r"with\s+([0-9]+)\s+threads", clean)
    res["threads"] = int(m.group(1)) if m else None
    if keep_field:
        ng = max(1, int((cfg["tend"] - cfg["tstart"]) / cfg["tstep"] + 0.5))
        f = np.fromfile(tmp / f"{session}.mc2", dtype=np.float32)
        # photon-sharing channels fold into the first axis, (srcnum * nx, ny, nz, nt), as pmcx shapes it
        res["flux"] = f.reshape((f.size // (vol.shape[1] * vol.shape[2] * ng),) + vol.shape[1:] + (ng,), order="F")
    mct = tmp / f"{session}.mct"
    if mct.exists():
        # trajectory records after a History header (src/mcx_utils.c:982-1017): 6 floats each
        raw = mct.read_bytes()
        n = struct.unpack("<4s7If1I", raw[:40])[7]
        res["traj"] = np.frombuffer(raw[64:64 + 24 * n], dtype=np.float32).reshape((6, n), order="F").copy()
    mch = tmp / f"{session}.mch"
    if mch.exists():
        raw = mch.read_bytes()
        res["mch_header"] = raw[:64]
        # History header (src/mcx_utils.h:115-132): magic, version, maxmedia, detnum, colcount,
        # totalphoton, detected, savedphoton, unitinmm, seedbyte, ...
        hdr = struct.unpack("<4s7If1I", raw[:40])
        colcount, saved, seedbyte = hdr[4], hdr[7], hdr[9]
        body = raw[64:64 + 4 * colcount * saved]
        res["detp"] = np.frombuffer(body, dtype=np.float32).reshape((colcount, saved), order="F")
        if seedbyte and cfg.get("issaveseed"):
            sd = np.frombuffer(raw[64 + 4 * colcount * saved:64 + (4 * colcount + seedbyte) * saved], dtype=np.uint8)
            res["seeds"] = sd.reshape(saved, seedbyte).T       # (seedbyte, n), as pmcx returns
    if not workdir:
        shutil.rmtree(tmp, ignore_errors=True)
    return res


if __name__ == "__main__":
    import sys

    if len(sys.argv) > 1 and sys.argv[1] == "stage":
        print(stage(sys.argv[2] if len(sys.argv) > 2 else None))
    else:
        print(build(force="--force" in sys.argv))
