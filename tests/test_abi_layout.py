"""The drop-in boundary on CPU: struct layouts, exported symbols, Config preparation."""

from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent

def _reference_src() -> Path:
    """MCX's src/ tree: $MCX_REFERENCE_ROOT/src when set, else the copy oracle/ref_mcx.py stages
    into baseline/_ref/src."""
    import os

    root = os.environ.get("MCX_REFERENCE_ROOT")
    return Path(root) / "src" if root else ROOT / "baseline" / "_ref" / "src"


REFERENCE_SRC = _reference_src()

def _probe_offsets(include_dir: Path, header: str, tmp_path: Path) -> dict[str, int]:
    """Compile a C probe printing offsetof() of every Config field and the struct sizes."""
    from mcx_gb300 import abi

    lines = [f'#include <stdio.h>\n#include <stddef.h>\n#include "{header}"\nint main(void){{']
    for name in abi.CONFIG_FIELDS:
        cname = "lambda" if name == "lambda_" else name
        lines.append(f'printf("{name} %zu\\n", offsetof(Config, {cname}));')
    lines.append('printf("sizeof_Config %zu\\n", sizeof(Config));')
    lines.append('printf("sizeof_GPUInfo %zu\\n", sizeof(GPUInfo));')
    lines.append('printf("sizeof_History %zu\\n", sizeof(History));')
    lines.append('printf("sizeof_Medium %zu\\n", sizeof(Medium));')
    lines.append('printf("sizeof_POLMedium %zu\\n", sizeof(POLMedium));')
    lines.append('printf("sizeof_ExtraSrc %zu\\n", sizeof(ExtraSrc));')
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    cuda_inc = "/usr/local/cuda/include"
    subprocess.run(["gcc", "-I", str(include_dir), "-I", cuda_inc, str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (ln.split() for ln in out.splitlines())}


def test_ctypes_mirror_matches_header(engine, tmp_path):
    from mcx_gb300 import abi

    c = _probe_offsets(ROOT / "include", "mcx_abi.h", tmp_path)
    offs = abi.offsets(abi.Config)
    for name in abi.CONFIG_FIELDS:
        assert offs[name] == c[name], name
    assert C.sizeof(abi.Config) == c["sizeof_Config"]
    assert C.sizeof(abi.GPUInfo) == c["sizeof_GPUInfo"]
    assert C.sizeof(abi.History) == c["sizeof_History"]
    assert C.sizeof(abi.Medium) == c["sizeof_Medium"]
    assert C.sizeof(abi.POLMedium) == c["sizeof_POLMedium"]
    assert C.sizeof(abi.ExtraSrc) == c["sizeof_ExtraSrc"]


@pytest.mark.skipif(not (REFERENCE_SRC / "mcx_utils.h").exists(), reason="reference headers not present")
def test_header_matches_reference_layout(engine, tmp_path):
    """include/mcx_abi.h against MCX's own src/mcx_utils.h, field by field."""
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    ours = _probe_offsets(ROOT / "include", "mcx_abi.h", tmp_path / "a")
    ref = _probe_offsets(REFERENCE_SRC, "mcx_utils.h", tmp_path / "b")
    assert ours == ref


def test_library_exports_every_declared_symbol(engine):
    """Every function declared in include/*.h is exported by libmcx_gb300.so."""
    from mcx_gb300._lib import LIB_PATH

    declared = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b((?:mcx|mcxg)_\w+)\s*\(", text, flags=re.M):
            declared.add(m.group(1))
    out = subprocess.run(["nm", "-D", "--defined-only", str(LIB_PATH)], check=True, capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert {"mcx_run_simulation", "mcx_list_gpu"} <= declared
    missing = declared - exported
    assert not missing, missing


def test_validatecfg_shifts_and_masks(engine):
    from mcx_gb300 import problems

    cfg = problems.cube60(1000)
    cfg["issrcfrom0"] = 0
    cfg["srcpos"] = [30.0, 30.0, 1.0]
    pc = engine.prepare(cfg)
    c = pc.c
    # origin shift to C indices (src/mcx_utils.c:3761-3773)
    assert (c.srcpos.x, c.srcpos.y, c.srcpos.z) == (29.0, 29.0, 0.0)
    assert abs(pc.detpos[0, 0] - 28.0) < 1e-6
    # launch voxel and label in srcparam2.z/.w as integer bit patterns
    idx = np.frombuffer(np.float32(c.srcparam2.z).tobytes(), np.uint32)[0]
    med = np.frombuffer(np.float32(c.srcparam2.w).tobytes(), np.uint32)[0]
    assert idx == 29 + 29 * 60 and med == 1
    # mus==0 media become (EPS, g=1)
    assert pc.prop[0, 1] == np.float32(np.finfo(np.float32).eps) and pc.prop[0, 2] == 1.0
    # detector voxels are masked only next to the detectors on the z=0 surface
    det = (pc.vol & 0x80000000).reshape(60, 60, 60, order="F") != 0
    assert det[:, :, 0].sum() > 0 and det[:, :, 2:].sum() == 0
    xs, ys, _ = np.nonzero(det)
    near = np.min([np.hypot(xs + 0.5 - d[0], ys + 0.5 - d[1]) for d in pc.detpos], axis=0)
    assert near.max() < 3.0


def test_maskdet_interior_detector_marks_nothing(engine):
    from mcx_gb300 import problems

    cfg = problems.cube60(1000)
    cfg["detpos"] = np.array([[30.0, 30.0, 30.0, 1.0]], np.float32)   # inside the medium, no interface
    pc = engine.prepare(cfg)
    assert not np.any(pc.vol & 0x80000000)


@pytest.mark.parametrize("bad,msg", [
    ({"tstart": 5e-9}, "time gate"),
    ({"srctype": "pattern"}, "srcpattern"),
    ({"srcnum": 2}, "photon sharing"),
    ({"respin": 0}, "respin"),
    ({"srcdir": [0.0, 0.0, 0.0]}, "direction"),
])
def test_validatecfg_errors(engine, bad, msg):
    from mcx_gb300 import problems

    cfg = problems.cube60(1000)
    cfg.update(bad)
    with pytest.raises(engine.MCXError, match=msg):
        engine.prepare(cfg)


def test_label_range_checked_on_host(engine):
    from mcx_gb300 import problems

    cfg = problems.cube60(1000)
    cfg["vol"] = (cfg["vol"] * 5).astype(np.uint8)
    with pytest.raises(engine.MCXError, match="labels"):
        engine.prepare(cfg)


def test_replayinit_filters_and_weights(engine):
    """mcxg_replayinit (restating src/mcx_utils.c:3624-3690) on hand-made records."""
    import ctypes as C

    from mcx_gb300 import problems

    cfg = problems.sphere60b(10)
    cfg.update(savedetflag="dp")
    rng = np.random.default_rng(3)
    n = 6
    detp = np.zeros((3, n), np.float32)                  # detid | ppath(2)
    detp[0] = [1, 2, 3, 2, 4, 2]
    detp[1] = rng.uniform(1, 50, n)
    detp[2] = rng.uniform(0, 20, n)
    detp[1, 5] = 5000.0                                  # time of flight beyond the 5 ns window
    seeds = np.arange(16 * n, dtype=np.uint8).reshape(n, 16).T
    cfg.update(seed=seeds, detphotons=detp, replaydet=2)
    pc = engine.prepare(cfg)
    c = pc.c
    assert c.nphoton == 2 and c.seed == -999             # detector 2, in time: records 1 and 3
    w = np.frombuffer((C.c_float * 2).from_address(c.replay.weight), np.float32)
    tof = np.frombuffer((C.c_float * 2).from_address(c.replay.tof), np.float32)
    mua = np.asarray(cfg["prop"], np.float32)[1:, 0]
    nidx = np.asarray(cfg["prop"], np.float32)[1:, 3]
    for k, i in enumerate((1, 3)):
        assert abs(w[k] - np.exp(-(mua * detp[1:, i]).sum())) < 1e-6
        assert abs(tof[k] - (detp[1:, i] * nidx).sum() * 3.335640951981520e-12) < 1e-15
    got = np.frombuffer((C.c_uint8 * 32).from_address(c.replay.seed), np.uint8).reshape(2, 16)
    assert np.array_equal(got, seeds.T[[1, 3]])


def test_pack_media_layouts():
    """pack_media: the 32-bit words and mediabyte of each per-voxel format (pmcx's packing)."""
    from mcx_gb300.api import pack_media

    b = np.zeros((4, 1, 1, 2), np.uint8)
    b[:, 0, 0, 0] = [1, 2, 3, 4]
    w, f = pack_media(b)
    assert f == 103 and w[0, 0, 0] == 0x04030201 and w[0, 0, 1] == 0
    s = np.zeros((2, 1, 1, 1), np.uint16)
    s[:, 0, 0, 0] = [0x1234, 0x5678]
    w, f = pack_media(s)
    assert f == 104 and w[0, 0, 0] == 0x56781234
    m = np.array([[[0.0, 0.25, np.nan]]], np.float32)
    w, f = pack_media(m, unitinmm=2.0)
    assert f == 101
    assert w[0, 0, 0] == np.array(np.finfo(np.float32).eps, np.float32).view(np.uint32)   # 0 is not void
    assert w[0, 0, 1] == np.array(0.5, np.float32).view(np.uint32) and w[0, 0, 2] == 0  # scaled; NaN void
    w, f = pack_media(np.ones((3, 3, 3), np.uint16))
    assert f == 2 and w.dtype == np.uint32
    lh = np.zeros((3, 1, 1, 2), np.float32)
    lh[:, 0, 0, 0] = [0.25, 1, 5]           # mus of label 5 replaced by 0.25 (x unitinmm)
    lh[:, 0, 0, 1] = [1.5, 3, 2]            # n of label 2 replaced by 1.5
    w, f = pack_media(lh, unitinmm=2.0)
    assert f == 99
    assert w[0, 0, 0] == (0x3800 << 16) | (1 << 14) | 5     # binary16 0.5 = 0x3800
    assert w[0, 0, 1] == (0x3E00 << 16) | (3 << 14) | 2     # binary16 1.5 = 0x3E00
    a4 = np.zeros((4, 1, 1, 2), np.float32)
    a4[:, 0, 0, 0] = [0.25, 2.0, 0.5, 1.5]
    a4[:, 0, 0, 1] = [np.nan, 1.0, 0.5, 1.5]
    w, f = pack_media(a4)
    assert f == 96 and w.shape == (1, 1, 2, 2)
    assert w[0, 0, 0, 0] == (0x4000 << 16) | 0x3400 and w[0, 0, 0, 1] == (0x3E00 << 16) | 0x3800   # halves
    assert w[0, 0, 1, 0] == 0 and w[0, 0, 1, 1] == 0                                          # NaN: void
    mx = np.zeros((3, 1, 1, 1), np.int16)
    mx[:, 0, 0, 0] = [3, 7, 16384]
    w, f = pack_media(mx)
    assert f == 98 and w[0, 0, 0] == (16384 << 16) | (7 << 8) | 3
    sh = np.zeros((2, 1, 1, 1), np.int16)
    sh[:, 0, 0, 0] = [-1, 5]
    w, f = pack_media(sh)
    assert f == 104 and w[0, 0, 0] == (5 << 16) | 0xFFFF
    sp = np.zeros((8, 1, 1, 1), np.uint8)
    sp[:, 0, 0, 0] = [1, 2, 10, 20, 30, 40, 50, 60]
    w, f = pack_media(sp)
    assert f == 97 and w.shape == (1, 1, 1, 2)
    assert w[0, 0, 0, 0] == 0x0102_0A14 and w[0, 0, 0, 1] == 0x1E28_323C     # mcx_preprocess's two words
    with pytest.raises(Exception):
        pack_media(np.ones((5, 3, 3, 3), np.float32))
    bad = np.ones((3, 2, 2, 2), np.float32)
    bad[1] = 4
    with pytest.raises(Exception):
        pack_media(bad)


def test_debug_flags_and_trajectory_only(engine):
    """-D letters as pmcx parses them (src/mcx_utils.c:5333-5348); -D T turns the fluence and
    detector outputs off as mcx_preprocess does (src/mcx_utils.c:1539-1542)."""
    from mcx_gb300 import problems

    for flag, bits in (("M", 2), ("mp", 6), ("T", 8), ("RMPT", 15), (2, 2), ("10", 10)):
        pc = engine.prepare(problems.cube60(100) | {"debuglevel": flag})
        assert pc.c.debuglevel == bits, (flag, pc.c.debuglevel)
    pc = engine.prepare(problems.cube60(100) | {"debuglevel": "T", "issavedet": 1,
                                                  "detpos": np.array([[29, 34, 0, 2]], np.float32)})
    assert pc.c.issave2pt == b"\x00" and pc.c.issavedet == b"\x00"


def test_photon_shares_over_devices(built):
    """The multi-device photon split (src/mcx_core.cu:2980-3007): shares in proportion to the
    workload, or to the core counts when none is given; the last device takes the remainder."""
    from mcx_gb300 import abi, prepare, problems
    from mcx_gb300._lib import lib

    pc = prepare(problems.cube60(1000))
    c = pc.c

    def shares(ids, n, work=None, cores=None):
        C.memmove(C.addressof(c) + abi.Config.deviceid.offset, bytes(ids) + b"\0", len(ids) + 1)
        for i in range(len(ids)):
            c.workload[i] = 0.0 if work is None else work[i]
        info = None
        if cores is not None:
            info = (abi.GPUInfo * max(ids))()
            for i, k in enumerate(cores):
                info[i].core = k
        off = (C.c_uint64 * len(ids))()
        cnt = (C.c_uint64 * len(ids))()
        rc = lib.mcxg_photon_shares(C.byref(c), info, n, off, cnt)
        return rc, list(off), list(cnt)

    assert shares([1], 1000) == (1, [0], [1000])
    assert shares([1, 2], 1001) == (2, [0, 500], [500, 501])
    assert shares([1, 2], 1000, work=[3.0, 1.0]) == (2, [0, 750], [750, 250])
    rc, off, cnt = shares([1, 2, 3], 10 ** 9 + 7, cores=[19456, 19456, 9728])
    assert rc == 3 and sum(cnt) == 10 ** 9 + 7 and off == [0, cnt[0], cnt[0] + cnt[1]]
    assert cnt[0] == cnt[1] == (10 ** 9 + 7) * 2 // 5 and list(c.workload[:3]) == [19456.0, 19456.0, 9728.0]
    assert shares([1, 1], 7) == (2, [0, 3], [3, 4])          # one device listed twice
    rc, _, _ = shares([1, 2], 100, work=[1.0, 0.0])
    assert rc == -1 and b"workload" in lib.mcxg_last_error()


@pytest.mark.parametrize("shape,dtype", [((7, 5, 3), np.uint8), ((130, 90, 100), np.uint8), ((4, 6, 8), np.int16)])
def test_row_major_labels_transposed_by_preparation(engine, shape, dtype):
    """A C-ordered label array goes to the engine as it lies, with MCX's isrowmajor flag: the
    preparation (threaded, tiled above 2^20 voxels) leaves the same x-fastest words as the
    Fortran-ordered copy of the same array, which takes the column-major path."""
    rng = np.random.default_rng(sum(shape))
    vol = rng.integers(0, 3, shape).astype(dtype)
    base = {"nphoton": 10, "prop": [[0, 0, 1, 1], [0.01, 1, 0.9, 1.37], [0.02, 2, 0.8, 1.4]], "tstart": 0.0,
            "tend": 1e-9, "tstep": 1e-9, "srcpos": [1.0, 1.0, 0.0], "srcdir": [0.0, 0.0, 1.0]}
    a = engine.prepare(dict(base, vol=vol))
    b = engine.prepare(dict(base, vol=np.asfortranarray(vol)))
    assert a.c.isrowmajor == b"\x00" and tuple(a.dims) == shape
    assert np.array_equal(a.vol, b.vol)
    assert np.array_equal(a.vol[: vol.size], vol.ravel(order="F").astype(np.uint32))


def test_batch_entry_points_refuse_bad_calls_before_any_device_work(engine):
    """mcxg_run_batch / mcxg_run_batch_device check their arguments on the host first: an empty
    batch and a missing device-field array come back as MCX error -4 with a message."""
    import ctypes as C

    from mcx_gb300 import abi
    from mcx_gb300._lib import lib

    arr = (C.POINTER(abi.Config) * 1)()
    stats = (abi.Stats * 1)()
    ms = C.c_double(0.0)
    assert lib.mcxg_run_batch(arr, 0, 4, stats, C.byref(ms)) == -4
    assert b"empty batch" in lib.mcxg_last_error()
    assert lib.mcxg_run_batch_device(arr, 1, 4, None, stats, C.byref(ms)) == -4
    assert b"no device fields" in lib.mcxg_last_error()
