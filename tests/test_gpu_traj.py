"""Photon trajectories (MCX's -D M / -D T, savedebugdata, src/mcx_core.cu:427-442).

A record (id, x, y, z, weight, source id) is written when a photon is launched, at each
scattering event, at each mismatched-index face it meets and when it ends (src/mcx_core.cu:
1681-1687, 2068-2074, 2435-2441, 1116-1122).  Checked: without reflection a run writes exactly
two records per photon plus one per scattering event (the kernel's own scattering counter); ids
run over the photons, each photon's records start at the source with its launch weight and never
gain weight; the record cap drops the excess; -D T leaves the fluence and detector outputs off;
and against MCX's own build the records per photon after the first weight loss, and their mean
depth, agree within statistical error.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu


def _deck(n, reflect=0, seed=7):
    cfg = problems.cube60(n)
    cfg.update(seed=seed, isreflect=reflect, debuglevel="M")
    return cfg


def test_records_per_photon_and_order(engine):
    n = 2000
    r = engine.run(_deck(n))
    traj, st = r["traj"], r["stat"]
    assert traj.shape[0] == 6
    assert traj.shape[1] == 2 * n + st["n_scatter"], (traj.shape, st["n_scatter"])
    ids = traj[0].view(np.uint32)
    assert ids.min() == 1 and ids.max() == n and len(np.unique(ids)) == n
    order = np.argsort(ids, kind="stable")           # records of one photon stay in write order
    ids_s, w_s, pos_s = ids[order], traj[4][order], traj[1:4][:, order]
    first = np.r_[True, ids_s[1:] != ids_s[:-1]]
    src = np.asarray(problems.cube60(1)["srcpos"][:3], np.float32)
    assert np.allclose(pos_s[:, first].T, src, atol=1e-4)
    assert np.allclose(w_s[first], 1.0)
    assert (np.diff(w_s)[~first[1:]] <= 1e-6).all()   # weight never grows along a photon
    assert (traj[5] == 0).all()
    inside = (traj[1:4] >= -1e-3).all(0) & (traj[1:4] <= 60 + 1e-3).all(0)
    assert inside.all()


def test_mismatched_faces_add_records(engine):
    n = 2000
    r0 = engine.run(_deck(n, reflect=0))
    r1 = engine.run(_deck(n, reflect=1))
    # with n = 1.37 against 1.0 every face the photon meets adds a record, and reflections keep
    # photons inside: more records per photon than the 2 + scatterings of the unreflected run
    assert r1["traj"].shape[1] > 2 * n + r1["stat"]["n_scatter"]
    assert r0["traj"].shape[1] == 2 * n + r0["stat"]["n_scatter"]


def test_record_cap_and_trajectory_only(engine):
    r = engine.run(_deck(500) | {"maxjumpdebug": 100})
    assert r["traj"].shape == (6, 100)
    r = engine.run(_deck(500) | {"debuglevel": "T", "issavedet": 1,
                                 "detpos": np.array([[29, 34, 0, 2]], np.float32)})
    assert "flux" not in r and "detp" not in r
    assert r["traj"].shape[1] > 1000


def test_against_reference_build(engine):
    from oracle import ref_mcx

    if not ref_mcx.available():
        pytest.skip("reference sources are not staged in baseline/_ref/src")
    ref_mcx.build()
    n = 20000
    cfg = _deck(n, reflect=1, seed=11)
    ours = engine.run(_deck(n, reflect=1, seed=11))["traj"]
    ref = ref_mcx.run(cfg, keep_field=False)
    theirs = ref["traj"]
    # records after the photon first lost weight (scattering, faces, termination): MCX may also
    # write records at thread start, at the source with the source weight, which this count leaves out
    late_o, late_r = ours[:, ours[4] < 1.0], theirs[:, theirs[4] < 1.0]
    per_ours, per_ref = late_o.shape[1] / n, late_r.shape[1] / n
    ids = late_o[0].view(np.uint32)
    counts = np.bincount(ids, minlength=n + 1)[1:]
    se = counts.std() / np.sqrt(n)
    print("records per photon after the first loss: engine", per_ours, "MCX", per_ref, "SE", se,
          "all records: engine", ours.shape[1], "MCX", theirs.shape[1])
    assert abs(per_ours - per_ref) <= 5 * se * np.sqrt(2)
    # where the interactions happen: the depth profile of the records (records of one photon are
    # correlated, so the photon count is the conservative sample size)
    zo, zr = late_o[3], late_r[3]
    assert abs(zo.mean() - zr.mean()) <= 5 * np.sqrt(zo.var() / n + zr.var() / n), (zo.mean(), zr.mean())
