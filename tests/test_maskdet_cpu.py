"""Detector masking (mcxg_maskdet) bit for bit against MCX's own mcx_maskdet, on the CPU.

MCX's command-line front-end, built from the reference sources (`oracle/ref_mcx.py:
build_frontend`), runs its unchanged preprocessing -- mcx_preprocess and mcx_maskdet
(src/mcx_utils.c:1525-1820, 4214-4340) -- while it parses the input, and with `-M 1` writes the
masked volume (label and detector bit per voxel, src/mcx_utils.c:4354-4390) and exits before it
looks for a GPU.  The engine's preparation of the same deck (`mcx_gb300.prepare`, which runs
mcxg_validatecfg) must leave the same labels and the same detector bits (bit 31) in every voxel.
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
