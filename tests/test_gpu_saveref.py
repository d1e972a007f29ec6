"""Diffuse reflectance (issaveref = 1) on the GPU.

* the reflectance map holds exactly the weight that left the medium: in a medium wrapped in a
  void shell every escaping photon ends in a void voxel, so the raw (un-normalised) reflectance
  summed over the grid equals the FP64 escaped-energy tally;
* it is non-negative, lives only on void voxels, and the fluence there is zero (pmcx's split);
* against the reference build (Session.DoSaveRef): the total reflectance and its distribution
  over the six faces of the shell agree.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu


def test_reflectance_is_the_escaped_weight(engine):
    r = engine.run(problems.reflectance_cube(1_000_000))
    dref, flux, st = r["dref"], r["flux"], r["stat"]
    void = np.ones((62, 62, 62), bool)
    void[1:-1, 1:-1, 1:-1] = False
    assert (dref >= 0).all() and not dref[~void].any() and not flux[void].any()
    raw = dref.astype(np.float64).sum() / st["normalizer"]
    print("reflectance", raw, "escaped", st["e_escape"], "launched", st["e_launch"])
    assert raw == pytest.approx(st["e_escape"], rel=2e-3)
    assert dref[:, :, 0].sum() > 0.5 * dref.sum()          # most light returns through the entry face


def test_without_saveref_unchanged(engine):
    # the fluence inside the medium is the same with and without the reflectance output (the
    # runs differ in kernel variant, so photon for photon only in distribution)
    cfg = problems.reflectance_cube(1_000_000)
    a = engine.run(cfg)
    b = engine.run(cfg | {"issaveref": 0})
    assert "dref" not in b
    inner = (slice(1, -1),) * 3
    fa, fb = a["flux"][inner].astype(np.float64), b["flux"][inner].astype(np.float64)
    assert fa.sum() == pytest.approx(fb.sum(), rel=5e-3)


def test_against_reference_build(engine):
    from oracle import ref_mcx

    if not ref_mcx.available():
        pytest.skip("reference sources are not staged in baseline/_ref/src")
    ref_mcx.build()
    n = 1_000_000
    ours = engine.run(problems.reflectance_cube(n))["dref"][..., 0].astype(np.float64)
    f = ref_mcx.run(problems.reflectance_cube(n))["flux"][..., 0].astype(np.float64)
    void = np.ones((62, 62, 62), bool)
    void[1:-1, 1:-1, 1:-1] = False
    theirs = np.where(void, -f, 0.0)
    assert (theirs >= 0).all()
    faces = lambda d: np.array([d[0].sum(), d[-1].sum(), d[:, 0].sum(), d[:, -1].sum(),  # noqa: E731
                                d[:, :, 0].sum(), d[:, :, -1].sum()])
    print("total", ours.sum(), theirs.sum(), "faces", faces(ours), faces(theirs))
    assert ours.sum() == pytest.approx(theirs.sum(), rel=0.01)
    np.testing.assert_allclose(faces(ours), faces(theirs), rtol=0.05, atol=0.002 * theirs.sum())
    # the radial profile on the entry face, in 2-voxel rings
    yy, xx = np.meshgrid(np.arange(62) + 0.5, np.arange(62) + 0.5, indexing="ij")
    ring = np.minimum((np.hypot(xx - 31, yy - 31) / 2).astype(int), 10)
    po = np.bincount(ring.ravel(), ours[:, :, 0].ravel(), 11)
    pt = np.bincount(ring.ravel(), theirs[:, :, 0].ravel(), 11)
    np.testing.assert_allclose(po, pt, rtol=0.05, atol=0.002 * pt.sum())


def test_exit_paths_equal_detected_sums(engine):
    # issaveref = 2: one detected record per voxel holding the summed exit weight and weighted
    # partial paths of the photons that ended there (MCX's slots: weight and medium-1 path share
    # slot 0), detection itself off.  The same sum over photons comes from an ordinary detector
    # run whose disk covers the whole medium surface: sum of w0 exp(-mua L) (1 + L).
    n = 1_000_000
    cfg = problems.reflectance_cube(n) | {"issaveref": 2, "issavedet": 1, "detpos": [[31.0, 31.0, 61.0, 1.0]],
                                           "maxdetphoton": 62 ** 3}
    d = engine.run(cfg)["detp"].astype(np.float64)
    assert d.shape == (2, 62 ** 3)
    void = np.ones((62, 62, 62), bool)
    void[1:-1, 1:-1, 1:-1] = False
    v = void.ravel(order="F")
    assert not d[:, ~v].any() and not d[1].any()
    det = engine.run(problems.reflectance_cube(n) | {"issaveref": 0, "issavedet": 1, "savedetflag": "dpw",
                                                     "detpos": [[31.0, 31.0, 31.0, 100.0]], "maxdetphoton": n})
    p = det["detp"].astype(np.float64)            # detid, path in medium 1, w0
    est = (p[2] * np.exp(-0.005 * p[1]) * (1.0 + p[1])).sum()
    se = (p[2] * np.exp(-0.005 * p[1]) * (1.0 + p[1])).std() * np.sqrt(p.shape[1])
    print("slot 0 sum", d[0].sum(), "detector estimate", est, "SE", se, "detected", p.shape[1])
    assert abs(d[0].sum() - est) <= 5 * se * np.sqrt(2)
