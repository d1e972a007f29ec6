"""Seed saving and photon replay (src/mcx_core.cu:375-377, 1203-1215, 2018-2066, 2207-2226).

A baseline run saves every detected photon's generator state at launch; a replay run starts
the same photons from those states, so each follows its baseline path exactly and is detected
again with the same record.  Along the way it adds the replay outputs, whose sums are known from
the baseline records:
  * Jacobian (j): sum over the voxels of medium m = sum_i w_i ppath_i(m),
    w_i = exp(-sum_m mua_m ppath_i(m)) the detected weight;
  * scattering counts (p): sum over the voxels of medium m = sum_i w_i nscat_i(m).
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu


def _baseline(n, flags="dsp"):
    cfg = problems.sphere60b(n)
    cfg.update(issaveseed=1, savedetflag=flags, seed=31337)
    return cfg


def _expect(base_detp, prop, col0, replaydet=0):
    """sum_i w_i x column block starting at col0 (per medium), from the baseline records."""
    det = base_detp
    M = prop.shape[0] - 1
    ppath = det[1 + M:1 + 2 * M]                         # 'dsp': id | nscat(M) | ppath(M)
    w = np.exp(-(prop[1:, 0:1].astype(np.float64) * ppath).sum(axis=0))
    keep = np.ones(det.shape[1], bool) if replaydet <= 0 else (det[0].astype(int) == replaydet)
    return (det[col0:col0 + M][:, keep].astype(np.float64) * w[keep]).sum(axis=1), w[keep].sum()


@pytest.fixture(scope="module")
def base(engine):
    r = engine.run(_baseline(1_000_000))
    assert r["seeds"].shape == (16, r["stat"]["detected"])
    return r


@pytest.mark.parametrize("ot,col", [("j", "ppath"), ("p", "nscat")])
def test_replay_reproduces_detected_photons(engine, base, ot, col):
    cfg = _baseline(1)
    cfg.update(seed=base["seeds"], detphotons=base["detp"], outputtype=ot, isnormalized=0)
    r = engine.run(cfg)
    n = r["stat"]["nphoton"]
    # replayed: the baseline photons detected within the time window (all but a few at its end)
    assert n > 0.99 * base["detp"].shape[1]
    # every replayed photon is detected again with the same record
    assert r["stat"]["detected"] == n
    baseline = set(map(tuple, base["detp"].T.tolist()))
    assert all(rec in baseline for rec in map(tuple, r["detp"].T.tolist()))
    # per-medium sums of the replay output equal the replayed records' weighted sums
    prop = np.asarray(cfg["prop"], np.float32)
    M = prop.shape[0] - 1
    col0 = 1 + M if col == "ppath" else 1
    expect, _ = _expect(r["detp"], prop, col0)
    field = r["flux"][..., 0].astype(np.float64)
    labels = cfg["vol"]
    got = np.array([field[labels == m].sum() for m in range(1, M + 1)])
    np.testing.assert_allclose(got, expect, rtol=2e-5)


def test_replay_normalisation_and_detector_blocks(engine, base):
    cfg = _baseline(1)
    cfg.update(seed=base["seeds"], detphotons=base["detp"], outputtype="j", replaydet=-1)
    r = engine.run(cfg)
    prop = np.asarray(cfg["prop"], np.float32)
    M = prop.shape[0] - 1
    assert r["flux"].shape[-1] == 4                      # one block per detector, 1 gate each
    for d in range(1, 5):
        expect, wsum = _expect(r["detp"], prop, 1 + M, replaydet=d)
        blk = r["flux"][..., d - 1].astype(np.float64)
        # normalised by unitinmm / (sum of detected weights of detector d)
        np.testing.assert_allclose(blk.sum(), expect.sum() / wsum, rtol=2e-5)


def test_replay_single_detector(engine, base):
    cfg = _baseline(1)
    cfg.update(seed=base["seeds"], detphotons=base["detp"], outputtype="j", replaydet=2, isnormalized=0)
    r = engine.run(cfg)
    assert r["stat"]["nphoton"] == int((base["detp"][0] == 2).sum())
    assert set(np.unique(r["detp"][0]).astype(int)) == {2}


def test_replay_in_mcx_seeding_mode(engine):
    from mcx_gb300._lib import lib

    lib.mcxg_set_seeding(1)
    try:
        b = engine.run(_baseline(300_000, flags="dp"))
        cfg = _baseline(1, flags="dp")
        cfg.update(seed=b["seeds"], detphotons=b["detp"], outputtype="j")
        r = engine.run(cfg)
    finally:
        lib.mcxg_set_seeding(0)
    assert r["stat"]["detected"] == r["stat"]["nphoton"] > 0.99 * b["detp"].shape[1]
    baseline = set(map(tuple, b["detp"].T.tolist()))
    assert all(rec in baseline for rec in map(tuple, r["detp"].T.tolist()))


@pytest.mark.parametrize("ot,col,sign", [("r", "ppath", -1.0), ("s", "nscat", 1.0)])
def test_rf_replay_outputs(engine, base, ot, col, sign):
    """Frequency-domain replay (src/mcx_core.cu:1700-1703, 2018-2066, 2207-2256): the real half of
    the field holds sign x w_i cos(omega t_i) x (path or scattering count), the imaginary half the
    same with sin; t_i the detected photon's time of flight from its partial paths."""
    omega = 2 * np.pi * 100e6
    cfg = _baseline(1)
    cfg.update(seed=base["seeds"], detphotons=base["detp"], outputtype=ot, isnormalized=0, omega=omega)
    r = engine.run(cfg)
    prop = np.asarray(cfg["prop"], np.float32)
    M = prop.shape[0] - 1
    det = r["detp"].astype(np.float64)
    ppath = det[1 + M:1 + 2 * M]
    w = np.exp(-(prop[1:, 0:1].astype(np.float64) * ppath).sum(axis=0))
    tof = (ppath * prop[1:, 3:4].astype(np.float64)).sum(axis=0) * 3.335640951981520e-12
    q = det[1 + M:1 + 2 * M] if col == "ppath" else det[1:1 + M]
    assert r["flux"].shape[-1] == 2
    labels = cfg["vol"]
    for half, trig in ((0, np.cos), (1, np.sin)):
        field = r["flux"][..., half].astype(np.float64)
        got = np.array([field[labels == m].sum() for m in range(1, M + 1)])
        expect = sign * (q * (w * trig(omega * tof))).sum(axis=1)
        np.testing.assert_allclose(got, expect, rtol=1e-4, atol=1e-6 * np.abs(expect).max())
