"""The oracle's extra sources (src/mcx_core.cu:1217-1227, 2225-2227, 3908-3910) on the CPU: two
pencil beams into cube60's medium.  With srcid -1 each source's block of gates, normalised as if
the source had all the photons, is that source's run alone; srcid 0 merges them into the mean
field and marks the detected photons' source above bit 16; srcid 2 runs the second source only
(with the same random streams the second source's own run has)."""

from __future__ import annotations

import numpy as np

from mcx_gb300 import problems

POS = [[20.0, 30.0, 0.0, 1.0], [40.0, 30.0, 0.0, 1.0]]
DIR = [[0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 1.0, 0.0]]
N = 200_000


def _deck(**kw):
    cfg = problems.cube60(N)
    cfg.update(kw)
    return cfg


def _coarse(f):
    return f.astype(np.float64).reshape(10, 6, 10, 6, 10, 6).sum((1, 3, 5))


def _close(a, b, tol_total=0.02, tol_block=0.15):
    ca, cb = _coarse(a), _coarse(b)
    big = cb > 0.02 * cb.max()
    assert abs(ca.sum() / cb.sum() - 1) < tol_total, (ca.sum(), cb.sum())
    assert np.abs(ca[big] / cb[big] - 1).max() < tol_block


def test_sources_apart_merged_and_alone(engine, oracle):
    singles = [oracle.run(engine.prepare(_deck(srcpos=POS[k], srcdir=DIR[k])))["flux"][..., 0] for k in range(2)]
    apart = oracle.run(engine.prepare(_deck(srcpos=POS, srcdir=DIR, srcid=-1)))["flux"]
    assert apart.shape[3] == 2
    for k in range(2):
        _close(apart[..., k], singles[k])
    merged = oracle.run(engine.prepare(_deck(srcpos=POS, srcdir=DIR, srcid=0)))
    _close(merged["flux"][..., 0], 0.5 * (singles[0] + singles[1]))
    ids = merged["detp"][0].astype(np.int64)
    assert set(np.unique(ids >> 16)) == {1, 2} and (ids & 0xFFFF).min() >= 1 and (ids & 0xFFFF).max() <= 4
    # srcid 2 draws no source: its photons are the second source's own run, photon for photon
    second = oracle.run(engine.prepare(_deck(srcpos=POS, srcdir=DIR, srcid=2)))["flux"][..., 0]
    alone = oracle.run(engine.prepare(_deck(srcpos=POS[1], srcdir=DIR[1])))["flux"][..., 0]
    np.testing.assert_allclose(second.sum(), alone.sum(), rtol=1e-9)
