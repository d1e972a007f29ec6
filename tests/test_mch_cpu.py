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


# -- .jdat (MCX's -F jnii detected-photon and trajectory documents) -------------------------------
def _jdat_prepared(engine, unit=1.0, totalsource=1):
    cfg = problems.cube60b(1000)
    cfg.update(unitinmm=unit, savedetflag="dspmxvw", issaveseed=1)
    pc = engine.prepare(cfg)
    h = pc.c.his
    h.maxmedia, h.detnum, h.totalsource, h.srcnum = 2, 4, totalsource, 1
    h.colcount = 1 + 3 * 2 + 3 + 3 + 1          # detid, nscat/ppath/mom per medium, p, v, w0
    h.savedetflag, h.seedbyte, h.normalizer, h.respin, h.version = 0x7F, 16, 3.5, 1, 1
    return pc, cfg


def _records(n, rng):
    detp = rng.random((14, n)).astype(np.float32)
    detp[0] = rng.integers(1, 5, n)              # detector ids
    detp[1:3] = rng.integers(0, 500, (2, n))     # scattering counts per medium
    return detp


def test_jdat_layout_and_round_trip(engine, tmp_path):
    import json

    from mcx_gb300 import mch

    pc, cfg = _jdat_prepared(engine)
    rng = np.random.default_rng(11)
    detp = _records(7, rng)
    seeds = rng.integers(0, 256, (16, 7), dtype=np.uint8)
    f = mch.save_jdet(tmp_path / "x_detp.jdat", pc, {"detp": detp, "seeds": seeds})
    doc = json.loads(f.read_text())["MCXData"]
    info = doc["Info"]
    # the header fields by the names and in the order of src/mcx_utils.c:1040-1055
    assert list(info) == ["Version", "MediaNum", "DetNum", "ColumnNum", "TotalPhoton", "DetectedPhoton",
                          "SavedPhoton", "LengthUnit", "SeedByte", "Normalizer", "Repeat", "SrcNum",
                          "SaveDetFlag", "TotalSource", "Media"]
    assert (info["MediaNum"], info["DetNum"], info["ColumnNum"], info["TotalPhoton"]) == (2, 4, 14, 1000)
    assert (info["DetectedPhoton"], info["SavedPhoton"], info["SeedByte"], info["SaveDetFlag"]) == (7, 7, 16, 0x7F)
    assert info["Normalizer"] == 3.5 and info["LengthUnit"] == 1.0
    # the media table as the run holds it (the background medium's mus is set to FLT_EPSILON, as MCX does)
    want = np.asarray(cfg["prop"], np.float32)
    assert np.allclose([[m["mua"], m["mus"], m["g"], m["n"]] for m in info["Media"]], want, rtol=1e-6, atol=2e-7)
    # one photon-major array per column group of the save mask (bits d s p m x v w)
    pd = doc["PhotonData"]
    assert list(pd) == ["detid", "nscat", "ppath", "mom", "p", "v", "w0", "seed"]
    sizes = {k: pd[k]["_ArraySize_"] for k in pd}
    assert sizes == {"detid": [7, 1], "nscat": [7, 2], "ppath": [7, 2], "mom": [7, 2], "p": [7, 3], "v": [7, 3],
                     "w0": [7, 1], "seed": [7, 16]}
    assert [pd[k]["_ArrayType_"] for k in pd] == ["uint32", "uint32"] + ["single"] * 5 + ["uint8"]
    assert all(pd[k]["_ArrayZipType_"] == "zlib" and pd[k]["_ArrayZipSize_"] == np.prod(sizes[k]) for k in pd)
    assert np.array_equal(mch.jdata_decode(pd["detid"]).ravel(), detp[0].astype(np.uint32))
    assert np.array_equal(mch.jdata_decode(pd["ppath"]), detp[3:5].T)
    assert np.array_equal(mch.jdata_decode(pd["seed"]), seeds.T)
    info2, d2, s2 = mch.load_jdet(f)
    assert info2 == info and np.array_equal(d2, detp) and np.array_equal(s2, seeds)


def test_jdat_media_in_mm_and_other_encodings(engine, tmp_path):
    from mcx_gb300 import mch

    pc, cfg = _jdat_prepared(engine, unit=0.5)
    detp = _records(4, np.random.default_rng(2))
    for zip_type in ("gzip", "base64"):
        f = mch.save_jdet(tmp_path / f"{zip_type}.jdat", pc, {"detp": detp}, zip=zip_type)
        info, d2, s2 = mch.load_jdet(f)
        assert np.array_equal(d2, detp) and s2 is None
        # the engine scales its media table by the voxel size; the document lists 1/mm
        assert np.allclose([[m["mua"], m["mus"]] for m in info["Media"]], np.asarray(cfg["prop"])[:, :2], rtol=1e-6,
                           atol=3e-7)
        assert info["LengthUnit"] == 0.5
    with pytest.raises(ValueError):
        mch.save_jdet(tmp_path / "bad.jdat", pc, {"detp": detp[:5]})
    with pytest.raises(ValueError):
        mch.save_jdet(tmp_path / "bad.jdat", pc, {"detp": detp}, zip="lz4")


def test_jdat_several_sources_split_the_second_group(engine, tmp_path):
    """With more than one source, MCX's writer takes the high 16 bits of the second column group
    off as a "srcid" array (src/mcx_utils.c:1095, 1119-1142); reading puts them back."""
    import json

    from mcx_gb300 import mch

    pc, _ = _jdat_prepared(engine, totalsource=3)
    detp = _records(5, np.random.default_rng(3))
    detp[1] += np.float32(65536 * 2)
    f = mch.save_jdet(tmp_path / "s.jdat", pc, {"detp": detp})
    pd = json.loads(f.read_text())["MCXData"]["PhotonData"]
    assert list(pd)[:3] == ["detid", "srcid", "nscat"]
    assert np.array_equal(mch.jdata_decode(pd["srcid"])[:, 0], np.full(5, 2, np.uint32))
    assert mch.jdata_decode(pd["nscat"]).max() < 65536
    assert np.array_equal(mch.load_jdet(f)[1], detp)


def test_jdat_trajectory(engine, tmp_path):
    import json

    from mcx_gb300 import mch

    pc, _ = _jdat_prepared(engine)
    traj = np.arange(6 * 5, dtype=np.float32).reshape(6, 5)
    f = mch.save_jdet(tmp_path / "x_traj.jdat", pc, {"traj": traj}, trajectory=True)
    doc = json.loads(f.read_text())["MCXData"]
    assert "PhotonData" not in doc
    tr = doc["Trajectory"]
    assert list(tr) == ["photonid", "p", "w0", "srcid"]
    assert [tr[k]["_ArraySize_"] for k in tr] == [[5, 1], [5, 3], [5, 1], [5, 1]]
    assert doc["Info"]["ColumnNum"] == 6 and doc["Info"]["DetectedPhoton"] == 5 and doc["Info"]["SavedPhoton"] == 5
    info, d, s = mch.load_jdet(f)
    assert np.array_equal(d, traj) and s is None


def test_jdata_decode_orders_and_types():
    """JData arrays as MCX's writers emit them: row-major by default, "_ArrayOrder_": "c" for
    column-major volumes (src/mcx_utils.c:4573-4575, 4594-4596), uint8 to double payloads."""
    import base64
    import zlib

    from mcx_gb300 import mch

    a = np.arange(24, dtype=np.float64).reshape(2, 3, 4)
    col = {"_ArrayType_": "double", "_ArraySize_": [2, 3, 4], "_ArrayOrder_": "c", "_ArrayZipType_": "zlib",
           "_ArrayZipSize_": 24, "_ArrayZipData_": base64.b64encode(zlib.compress(a.tobytes(order="F"))).decode()}
    assert np.array_equal(mch.jdata_decode(col), a)
    for jt, dt in (("uint8", np.uint8), ("int16", np.int16), ("uint32", np.uint32), ("single", np.float32)):
        v = (np.arange(6) * 3).astype(dt).reshape(2, 3)
        assert np.array_equal(mch.jdata_decode(mch.jdata_encode(v, jt)), v)
