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
