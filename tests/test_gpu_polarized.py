"""Polarised light on the GPU: Mie phase-function sampling and Stokes-vector tracking.

* every detected photon carries a Stokes vector of unit intensity that stays fully polarised
  (sphere scattering maps fully polarised light to fully polarised light);
* runs are deterministic for a fixed seed (the same set of detected records, in the order the
  photons happened to finish, and the same fluence up to the order of float atomic additions);
* against the reference build of MCX on the polarised slab deck
  (mcxlab/examples/demo_polarized_photon.m): absorbed fraction, detected count, the path length
  and exit-direction statistics of detected photons, and the reflected Stokes vector R = sum of
  the detector-frame Stokes vectors times the detected weights over the launched photons, each
  within five standard errors of the two runs combined.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu

MUA = [0.005, 0.005]


def test_detected_stokes_vectors(engine):
    cfg = problems.polarized_slab(200_000)
    r = engine.run(cfg)
    d = r["detp"]
    assert d.shape[0] == 13 and d.shape[1] > 1000
    iquv = d[9:13].astype(np.float64)
    np.testing.assert_allclose(iquv[0], 1.0, atol=1e-5)
    np.testing.assert_allclose((iquv[1:] ** 2).sum(0), 1.0, atol=2e-4)
    v = d[5:8].astype(np.float64)
    np.testing.assert_allclose((v ** 2).sum(0), 1.0, atol=1e-4)
    assert (v[2] < 0).all()                                     # leaving through z = 0
    assert (d[2:4] >= 0).all() and (d[2:4] <= 100).all() and np.abs(d[4]).max() < 1e-3
    # light scattered back from a horizontally polarised beam keeps a positive Q on average
    st, w = problems.rotated_stokes(d, 2, 0.1, MUA)
    assert (st[1] * w).sum() > 0


def test_deterministic(engine):
    a = engine.run(problems.polarized_slab(50_000))
    b = engine.run(problems.polarized_slab(50_000))
    da, db = a["detp"], b["detp"]
    assert da.shape == db.shape
    assert np.array_equal(da[:, np.lexsort(da)], db[:, np.lexsort(db)])
    fa, fb = a["flux"], b["flux"]
    np.testing.assert_allclose(fa, fb, rtol=1e-4, atol=1e-6 * np.abs(fa).max())


def test_against_reference_build(engine):
    from oracle import ref_mcx

    if not ref_mcx.available():
        pytest.skip("reference sources are not staged in baseline/_ref/src")
    ref_mcx.build()
    n = 1_000_000
    ours = engine.run(problems.polarized_slab(n))
    theirs = ref_mcx.run(problems.polarized_slab(n), keep_field=False)
    do, dr = ours["detp"], theirs["detp"]
    assert dr.shape[0] == do.shape[0] == 13
    no, nr = do.shape[1], dr.shape[1]
    print("detected: engine", no, "MCX", nr, "absorbed: engine", (ours["stat"]["energyabs"] / ours["stat"]["energytot"]), "MCX", theirs["absorbed"])
    assert abs(no - nr) <= 5 * np.sqrt(no + nr)
    assert (ours["stat"]["energyabs"] / ours["stat"]["energytot"]) == pytest.approx(theirs["absorbed"], rel=0.03, abs=2e-4)

    def close(a, b, what):
        se = np.sqrt(a.var() / a.size + b.var() / b.size)
        print(what, a.mean(), b.mean(), "SE", se)
        assert abs(a.mean() - b.mean()) <= 5 * se + 1e-6, what

    for k, what in ((0, "ppath small spheres"), (7, "exit v_z"), (8, "w0")):
        close(do[k].astype(np.float64), dr[k].astype(np.float64), what)
    so, wo = problems.rotated_stokes(do, 2, 0.1, MUA)
    sr, wr = problems.rotated_stokes(dr, 2, 0.1, MUA)
    for k, what in enumerate("IQUV"):
        # R_k = sum(s_k w) / n: compare the per-launched-photon contributions (zero for the undetected)
        a = np.zeros(n)
        a[:no] = so[k] * wo
        b = np.zeros(n)
        b[:nr] = sr[k] * wr
        close(a, b, "R_" + what)


def test_trajectories_with_stokes(engine):
    # istrajstokes: trajectory records of polarised runs carry the Stokes vector (10 floats);
    # without it, the plain 6-float records
    cfg = problems.polarized_slab(2000) | {"debuglevel": "M", "maxjumpdebug": 200_000}
    t = engine.run(cfg | {"istrajstokes": 1})["traj"]
    assert t.shape[0] == 10 and t.shape[1] > 2000
    s = t[6:10].astype(np.float64)
    np.testing.assert_allclose(s[0], 1.0, atol=1e-5)
    np.testing.assert_allclose((s[1:] ** 2).sum(0), 1.0, atol=2e-4)
    assert engine.run(cfg)["traj"].shape[0] == 6
