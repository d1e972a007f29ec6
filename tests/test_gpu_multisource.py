"""Several sources in one run (extrasrclen, srcid) on the GPU.

Two pencil beams into cube60's medium at different points:
* srcid -1 keeps one block of gates per source, each normalised as if its source had all the
  photons: block k equals a run of source k alone;
* srcid 0 merges them: the field is the mean of the two single-source fields, and the detected
  photons carry their source above bit 16 of the detector id;
* srcid 2 runs the second source only.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu

POS = [[20.0, 30.0, 0.0, 1.0], [40.0, 30.0, 0.0, 1.0]]
DIR = [[0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 1.0, 0.0]]


def _deck(n, **kw):
    cfg = problems.cube60(n)
    cfg.update(kw)
    return cfg


def _coarse(f):
    return f.astype(np.float64).reshape(10, 6, 10, 6, 10, 6).sum((1, 3, 5))


def _check(a, b, what):
    ca, cb = _coarse(a), _coarse(b)
    big = cb > 0.01 * cb.max()
    print(what, ca.sum(), cb.sum(), np.abs(ca[big] / cb[big] - 1).max())
    assert ca.sum() == pytest.approx(cb.sum(), rel=0.01)
    assert np.abs(ca[big] / cb[big] - 1).max() < 0.1


def test_sources(engine):
    n = 2_000_000
    singles = [engine.run(_deck(n, srcpos=POS[k], srcdir=DIR[k]))["flux"][..., 0] for k in range(2)]
    apart = engine.run(_deck(n, srcpos=POS, srcdir=DIR, srcid=-1))["flux"]
    assert apart.shape[3] == 2
    for k in range(2):
        _check(apart[..., k], singles[k], f"srcid -1, block {k}")
    merged = engine.run(_deck(n, srcpos=POS, srcdir=DIR, srcid=0))
    _check(merged["flux"][..., 0], 0.5 * (singles[0] + singles[1]), "srcid 0")
    ids = merged["detp"][0].astype(np.int64)
    src, det = ids >> 16, ids & 0xFFFF
    assert set(np.unique(src)) == {1, 2} and det.min() >= 1 and det.max() <= 4
    second = engine.run(_deck(n, srcpos=POS, srcdir=DIR, srcid=2))["flux"][..., 0]
    _check(second, singles[1], "srcid 2")


# -- replay of a several-source run (src/mcx_core.cu:1203-1231) -----------------------------------
def _ms_replay_deck(base, keep=None, **kw):
    cfg = _deck(1, srcpos=POS, srcdir=DIR, savedetflag="dsp")
    keep = np.ones(base["detp"].shape[1], bool) if keep is None else keep
    cfg.update(seed=base["seeds"][:, keep], detphotons=base["detp"][:, keep], outputtype="j", isnormalized=0)
    cfg.update(kw)
    return cfg


@pytest.fixture(scope="module")
def msbase(engine):
    r = engine.run(_deck(1_000_000, srcpos=POS, srcdir=DIR, srcid=0, issaveseed=1, savedetflag="dsp", seed=4242))
    src = r["detp"][0].astype(np.int64) >> 16
    assert set(np.unique(src)) == {1, 2}
    return r


def _records(detp, mask_source=False):
    d = detp.copy()
    if mask_source:
        d[0] = (d[0].astype(np.int64) & 0xFFFF).astype(np.float32)
    return set(map(tuple, d.T.tolist()))


def test_replay_draws_the_recorded_source(engine, msbase):
    """srcid 0: a replayed photon draws its source from its restored generator state, as the
    recorded run did, so it follows the recorded path and is detected again with its record."""
    r = engine.run(_ms_replay_deck(msbase, srcid=0))
    n = r["stat"]["nphoton"]
    assert n > 0.99 * msbase["detp"].shape[1] and r["stat"]["detected"] == n
    assert _records(r["detp"]) <= _records(msbase["detp"])


def test_replay_of_one_source_skips_the_source_draw(engine, msbase):
    """srcid 2: the photons the recorded run launched from source 2, replayed from source 2 alone,
    skip the draw that picked their source (src/mcx_core.cu:1229-1231) and are detected again."""
    mine = (msbase["detp"][0].astype(np.int64) >> 16) == 2
    r = engine.run(_ms_replay_deck(msbase, keep=mine, srcid=2))
    n = r["stat"]["nphoton"]
    assert n > 0.99 * mine.sum() and r["stat"]["detected"] == n
    assert _records(r["detp"]) <= _records(msbase["detp"][:, mine], mask_source=True)


def test_replay_every_source_and_detector_apart(engine, msbase):
    """srcid -1 with replaydet -1: one block per (source, detector), sources outermost; each block
    holds the Jacobian of that source's photons detected by that detector.  Normalised, MCX scales
    the first source's detector blocks by their replayed weight and leaves the others as summed
    (src/mcx_core.cu:3845-3873)."""
    r = engine.run(_ms_replay_deck(msbase, srcid=-1, replaydet=-1))
    assert r["flux"].shape[-1] == 8
    # every replayed photon detected again: its record carries its source and detector
    prop = np.asarray(_deck(1)["prop"], np.float32)
    M = prop.shape[0] - 1
    det = r["detp"]
    assert r["stat"]["detected"] == r["stat"]["nphoton"]
    ids = det[0].astype(np.int64)
    ppath = det[1 + M:1 + 2 * M].astype(np.float64)
    w = np.exp(-(prop[1:, 0:1].astype(np.float64) * ppath).sum(axis=0))
    raw = {}
    for s in (1, 2):
        for d in range(1, 5):
            sel = ((ids >> 16) == s) & ((ids & 0xFFFF) == d)
            blk = r["flux"][..., (s - 1) * 4 + d - 1].astype(np.float64)
            raw[s, d] = blk
            np.testing.assert_allclose(blk.sum(), (ppath[:, sel] * w[sel]).sum(), rtol=2e-5, atol=1e-9)
    n = engine.run(_ms_replay_deck(msbase, srcid=-1, replaydet=-1, isnormalized=1))["flux"]
    for d in range(1, 5):
        wsum = w[(ids & 0xFFFF) == d].sum()          # the replayed weight of detector d
        np.testing.assert_allclose(n[..., d - 1].astype(np.float64).sum(), raw[1, d].sum() / wsum, rtol=2e-5)
        np.testing.assert_allclose(n[..., 4 + d - 1].astype(np.float64).sum(), raw[2, d].sum(), rtol=2e-5)


def test_sources_against_the_oracle(engine, oracle):
    """srcid -1 on the engine and on the oracle's restatement of the source draw and the
    per-source blocks: each block's total within 1% and its 6^3 sums within 10%."""
    n = 1_000_000
    e = engine.run(_deck(n, srcpos=POS, srcdir=DIR, srcid=-1))["flux"]
    o = oracle.run(engine.prepare(_deck(n, srcpos=POS, srcdir=DIR, srcid=-1)), seed=97531)["flux"]
    assert e.shape == o.shape
    for k in range(2):
        _check(e[..., k], o[..., k], f"srcid -1, block {k}, engine against the oracle")
