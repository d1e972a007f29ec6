"""The .mch file of a run against the one the reference build writes for the same deck.

Header fields that do not depend on the random walk (layout, column count, media and detector
counts, photon total, seed size, normalisation, flags) are equal; the detected counts agree
within five standard errors; the file reads back to the run's records and seeds.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu


def test_mch_against_reference_build(engine, tmp_path):
    from oracle import ref_mcx

    from mcx_gb300 import abi, mch

    if not ref_mcx.available():
        pytest.skip("reference sources are not staged in baseline/_ref/src")
    ref_mcx.build()
    cfg = problems.cube60(200_000) | {"issaveseed": 1, "savedetflag": "dp"}
    pc = engine.prepare(cfg)
    res = engine.run_prepared(pc)
    f = mch.save_mch(tmp_path / "ours.mch", pc, res)
    hdr, detp, seeds = mch.load_mch(f)
    assert np.array_equal(detp, res["detp"]) and np.array_equal(seeds, res["seeds"])
    theirs = ref_mcx.run(problems.cube60(200_000) | {"issaveseed": 1, "savedetflag": "dp"}, keep_field=False)
    h = abi.History.from_buffer_copy(theirs["mch_header"])
    print({k: (hdr[k], getattr(h, k)) for k in hdr if k != "magic"})
    for k in ("version", "maxmedia", "detnum", "colcount", "totalphoton", "unitinmm", "seedbyte", "respin",
              "srcnum", "savedetflag", "totalsource"):
        assert hdr[k] == getattr(h, k), k
    assert hdr["magic"] == bytes(h.magic) == b"MCXH"
    assert hdr["normalizer"] == pytest.approx(h.normalizer, rel=1e-6)
    assert abs(hdr["detected"] - h.detected) <= 5 * np.sqrt(hdr["detected"] + h.detected)
    assert hdr["savedphoton"] == hdr["detected"] and h.savedphoton == h.detected
