"""Host preparation (mcxg_validatecfg, mcxg_maskdet) against MCX's own mcx_preprocess and
mcx_maskdet, on the CPU.

MCX's command-line front-end, built from the reference sources (`oracle/ref_mcx.py:
build_frontend`), runs its unchanged preprocessing -- mcx_preprocess and mcx_maskdet
(src/mcx_utils.c:1525-1820, 4214-4340) -- while it parses the input, and with `-M 1` writes the
masked volume (label and detector bit per voxel, src/mcx_utils.c:4354-4390) and exits before it
looks for a GPU; with `--dumpjson 3` it prints the prepared configuration instead
(src/mcx_utils.c:1929-1932, 3250-3400).  The engine's preparation of the same deck
(`mcx_gb300.prepare`, which runs mcxg_validatecfg) must leave the same labels and detector bits
(bit 31) in every voxel, and the same source position, direction, launch voxel and label
(srcparam2.z / .w bit patterns, src/mcx_utils.c:1737-1746), detectors and media.
"""

from __future__ import annotations

import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import ref_mcx

pytestmark = pytest.mark.skipif(not ref_mcx.available(), reason="reference sources not staged in baseline/_ref/src")

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def cli(built):
    return ref_mcx.build_frontend(ROOT / "mcx_gb300" / "libmcx_gb300.so")


def _reference_mask(cli, cfg, tmp_path) -> np.ndarray:
    vol = np.asarray(cfg["vol"]).astype(np.uint8)
    vol.ravel(order="F").tofile(tmp_path / "vol.bin")
    (tmp_path / "in.json").write_text(json.dumps(ref_mcx._json_input(cfg, "mask", str(tmp_path / "vol.bin"))))
    p = subprocess.run([str(cli), "-f", "in.json", "-M", "1", "-F", "nii"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    raw = (tmp_path / "mask_vol.nii").read_bytes()
    off = int(np.frombuffer(raw[108:112], "<f4")[0])
    # NIfTI uint16 pairs per voxel, x fastest: (label, detector bit)
    return np.frombuffer(raw[off:off + 4 * vol.size], "<u2").reshape(-1, 2)


def _deck(vol, detpos, **kw):
    cfg = {"nphoton": 1000, "seed": 1, "vol": vol, "prop": np.array([[0, 0, 1, 1], [0.01, 1.0, 0.9, 1.37],
                                                                       [0.02, 2.0, 0.8, 1.4], [0.03, 3.0, 0.7, 1.45]],
                                                                      np.float32),
           "tstart": 0.0, "tend": 5e-9, "tstep": 5e-9, "srcpos": [2.0, 2.0, 0.0], "srcdir": [0.0, 0.0, 1.0],
           "issrcfrom0": 1, "detpos": np.asarray(detpos, np.float32), "issavedet": 1}
    cfg.update(kw)
    return cfg


def _decks():
    from mcx_gb300 import problems

    yield "cube60b", problems.cube60b(1000)
    yield "cube60b-halfmm", dict(problems.cube60b(1000), unitinmm=0.5)
    yield "sphere60b", problems.sphere60b(1000)
    # a void pocket inside the medium and detectors on its wall, on the outer faces and outside
    v = np.ones((40, 30, 20), np.uint8)
    v[15:25, 10:20, 8:14] = 0
    v[:, :, 15:] = 2
    yield "pocket", _deck(v, [[15, 15, 10, 2.0], [20, 10, 11, 1.5], [0, 15, 10, 3.0], [39.5, 29.5, 19.5, 2.5],
                              [20, 15, 25, 2.0], [20, 15, 0, 4.0]])
    # random labels with scattered void voxels and random detectors, origin at 1 (MATLAB indices)
    rng = np.random.default_rng(7)
    v = rng.integers(1, 4, (24, 18, 16)).astype(np.uint8)
    v[rng.random(v.shape) < 0.08] = 0
    det = np.column_stack([rng.uniform(-2, 26, 8), rng.uniform(-2, 20, 8), rng.uniform(-2, 18, 8),
                           rng.uniform(0.5, 4.0, 8)])
    yield "random", _deck(v, det, issrcfrom0=0, srcpos=[3.0, 3.0, 1.0])


@pytest.mark.parametrize("name", ["cube60b", "cube60b-halfmm", "sphere60b", "pocket", "random"])
def test_detector_mask_matches_mcx(engine, cli, tmp_path, name):
    cfg = dict(_decks())[name]
    want = _reference_mask(cli, cfg, tmp_path)
    pc = engine.prepare(cfg)
    n = np.asarray(cfg["vol"]).size
    got = np.asarray(pc.vol[:n])
    assert np.array_equal((got & 0x7FFFFFFF).astype(np.uint16), want[:, 0])
    marked = (got >> 31).astype(np.uint16)
    print(name, "detector voxels", int(marked.sum()), "MCX", int(want[:, 1].sum()))
    assert marked.sum() > 0
    assert np.array_equal(marked, want[:, 1])


def _reference_prepared(cli, cfg, tmp_path) -> dict:
    vol = np.asarray(cfg["vol"]).astype(np.uint8)
    vol.ravel(order="F").tofile(tmp_path / "vol.bin")
    (tmp_path / "in.json").write_text(json.dumps(ref_mcx._json_input(cfg, "prep", str(tmp_path / "vol.bin"))))
    p = subprocess.run([str(cli), "-f", "in.json", "--dumpjson", "3"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    return json.loads(p.stdout[p.stdout.index("{"):])


def _prep_decks():
    from mcx_gb300 import problems

    yield "cube60b", problems.cube60b(1000)
    yield "sphere60b", problems.sphere60b(1000)
    yield "outside", dict(problems.cube60b(1000), srcpos=[29.5, 29.5, -3.0])
    yield "oblique", dict(problems.sphere60b(1000), srcpos=[10.25, 40.75, 12.5], srcdir=[1.0, -2.0, 3.0])
    yield "origin1", dict(problems.cube60b(1000), issrcfrom0=0, srcpos=[30.0, 30.0, 1.0])
    yield "halfmm", dict(problems.sphere60b(1000), unitinmm=0.5)


@pytest.mark.parametrize("name", ["cube60b", "sphere60b", "outside", "oblique", "origin1", "halfmm"])
def test_prepared_source_detectors_media_match_mcx(engine, cli, tmp_path, name):
    cfg = dict(_prep_decks())[name]
    ref = _reference_prepared(cli, cfg, tmp_path)
    pc = engine.prepare(cfg)
    c = pc.c
    src = ref["Optode"]["Source"]
    f32 = lambda v: np.asarray(v, np.float64).astype(np.float32)  # noqa: E731
    assert np.array_equal(f32(src["Pos"]), f32([c.srcpos.x, c.srcpos.y, c.srcpos.z])), (src["Pos"], c.srcpos.x)
    np.testing.assert_array_max_ulp(f32(src["Dir"][:3]), f32([c.srcdir.x, c.srcdir.y, c.srcdir.z]), maxulp=1)
    # the launch voxel and its label, kept as integer bit patterns in srcparam2.z / .w
    bits = f32(src["Param2"][2:4]).view(np.uint32)
    mine = np.array([c.srcparam2.z, c.srcparam2.w], np.float32).view(np.uint32)
    assert np.array_equal(bits, mine), (bits, mine)
    det = np.array([[d["Pos"][0], d["Pos"][1], d["Pos"][2], d["R"]] for d in ref["Optode"]["Detector"]], np.float32)
    assert np.array_equal(det, np.asarray(pc.detpos, np.float32).reshape(-1, 4))
    media = np.array([[m["mua"], m["mus"], m["g"], m["n"]] for m in ref["Domain"]["Media"]], np.float64)
    prop = np.ctypeslib.as_array((__import__("ctypes").c_float * (4 * c.medianum)).from_address(c.prop))
    prop = prop.reshape(-1, 4).astype(np.float64)
    prop[:, :2] /= np.float64(np.float32(c.unitinmm))
    np.testing.assert_allclose(prop, media, rtol=1e-6, atol=1e-12)
