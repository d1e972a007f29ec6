"""The .mch / .mct writer and reader (mcx_gb300/mch.py) on the CPU.

* the header is MCX's 64-byte History block (src/mcx_utils.h:115-132), checked against a
  struct.pack of the documented field order; records follow as F-ordered float32 and seeds as
  photon-major bytes (src/mcx_utils.c:1009-1014);
* write -> read round trips for detected photons with and without seeds and for trajectories,
  whose header carries colcount 6, the record count and detected = 0 (src/mcx_core.cu:3966-3975).
"""

from __future__ import annotations

import struct

import numpy as np
import pytest

from mcx_gb300 import problems


def _prepared(engine):
    cfg = problems.cube60(1000)
    pc = engine.prepare(cfg)
    h = pc.c.his
    h.colcount, h.detected, h.savedphoton, h.totalphoton = 6, 0, 0, 0
    h.normalizer, h.seedbyte, h.respin = 2.5, 32, 1
    return pc


def test_header_layout_and_round_trip(engine, tmp_path):
    from mcx_gb300 import mch

    pc = _prepared(engine)
    rng = np.random.default_rng(4)
    detp = rng.random((6, 3)).astype(np.float32)
    seeds = rng.integers(0, 256, (32, 3), dtype=np.uint8)
    f = mch.save_mch(tmp_path / "a.mch", pc, {"detp": detp, "seeds": seeds})
    raw = f.read_bytes()
    assert len(raw) == 64 + 6 * 3 * 4 + 32 * 3
    want = struct.pack("<4sIIIIIIIfIfiIIIi", b"MCXH", 1, 2, 4, 6, 1000, 3, 3, 1.0, 32, 2.5, 1, 1,
                       int(pc.c.his.savedetflag), 1, 0)
    assert raw[:64] == want
    assert raw[64:64 + 72] == detp.tobytes(order="F")
    assert raw[136:] == seeds.T.tobytes()
    hdr, d2, s2 = mch.load_mch(f)
    assert hdr["magic"] == b"MCXH" and hdr["colcount"] == 6 and hdr["savedphoton"] == 3 and hdr["maxmedia"] == 2
    assert hdr["normalizer"] == 2.5 and hdr["detnum"] == 4
    assert np.array_equal(d2, detp) and np.array_equal(s2, seeds)
    # without seeds: records only
    f = mch.save_mch(tmp_path / "b.mch", pc, {"detp": detp})
    assert len(f.read_bytes()) == 64 + 72 and mch.load_mch(f)[2] is None
    with pytest.raises(ValueError):
        mch.save_mch(tmp_path / "c.mch", pc, {"detp": detp[:5]})


def test_trajectory_file(engine, tmp_path):
    from mcx_gb300 import mch

    pc = _prepared(engine)
    traj = np.arange(6 * 5, dtype=np.float32).reshape(6, 5)
    f = mch.save_mct(tmp_path / "a.mct", pc, {"traj": traj})
    hdr, d, s = mch.load_mch(f)
    assert hdr["colcount"] == 6 and hdr["savedphoton"] == 5 and hdr["detected"] == 0 and hdr["totalphoton"] == 1000
    assert np.array_equal(d, traj) and s is None
    bad = tmp_path / "bad.mch"
    bad.write_bytes(b"XXXX" + bytes(60))
    with pytest.raises(ValueError):
        mch.load_mch(bad)
