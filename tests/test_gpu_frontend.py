"""The drop-in boundary exercised by MCX's real caller: the reference's own command-line front-end
(src/mcx.c, with the unchanged input parsing, output writers and error handler of
src/mcx_utils.c) linked against libmcx_gb300.so in place of src/mcx_core.cu.

Each case runs the CLI the way the reference's regression script test/testmcx.sh does and checks
the same printed result (the line of testmcx.sh is given per case), plus the files the CLI writes
through mcx_savedata / mcx_savedetphoton and an engine error routed through mcx_error."""

from __future__ import annotations

import json
import re
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import ref_mcx

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_mcx.available(), reason="reference sources not staged in baseline/_ref/src")]

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def cli(built):
    return ref_mcx.build_frontend(ROOT / "mcx_gb300" / "libmcx_gb300.so")


def run(cli, args, cwd, rc=0):
    """Runs the CLI in `cwd`; returns its report.  MCX's front-end declares its log switch as a
    plain `char` initialised to -1 (src/mcx_utils.c:4783); where char is unsigned (aarch64) that
    reads as "save the log", so the report goes to <session>.log instead of stdout: both are read."""
    for f in Path(cwd).glob("*.log"):
        f.unlink()
    p = subprocess.run([str(cli), *args], cwd=cwd, capture_output=True, text=True, timeout=600)
    out = p.stdout + p.stderr + "".join(f.read_text(errors="replace") for f in sorted(Path(cwd).glob("*.log")))
    out = re.sub(r"\x1b\[[0-9;]*m", "", out)
    assert p.returncode == rc, f"{args}: exit {p.returncode}\n{out[-3000:]}"
    return out


CASES = [
    # (arguments, pattern of testmcx.sh, its line)
    (["--bench", "cube60", "-S", "0"], r"absorbed:.*17\.[0-9]+%", 61),
    (["--bench", "cube60b", "-S", "0"], r"absorbed:.*27\.[0-9]+%", 65),
    (["--bench", "cube60", "-b", "1", "-S", "0"], r"absorbed:.*27\.[0-9]+%", 69),
    (["--bench", "cube60", "-b", "0", "-B", "aarraa", "-S", "0"], r"absorbed:.*27\.[0-9]+%", 73),
    (["--bench", "cube60", "--bc", "cccccc", "-n", "1e3", "-d", "0", "-S", "0"], r"absorbed:.*99\.[0-9]+%", 77),
    (["--bench", "cube60b"], r"detected.*4[0-9]+ photons", 81),
    (["--bench", "cube60planar"], r"absorbed:.*25\.[0-9]+%", 85),
    (["--bench", "cube60", "--json", '{"Optode":{"Source":{"Type":"isotropic","Pos":[29,29,29]}}}', "-d", "0", "-S", "0"],
     r"absorbed:.*88\.[0-9]+%", 89),
    (["--bench", "cube60", "--json",
      '{"Domain":{"Media":[[0,0,1,1],[0.001,0.001,0,1]]},"Optode":{"Source":{"Type":"cone","Param1":[0.5,0,0,0]}}}',
      "-d", "0", "-S", "0"], r"absorbed:.*6\.[0-9]+%", 93),
    (["--bench", "cube60", "--bc", "______111111", "-n", "1e4"], r"detected.*9[7-9][0-9.]+ photons", 112),
    (["--bench", "cube60", "-D", "R"], r"generating 216000 random numbers", 153),
    (["-L"], r"Global [Mm]emory", 34),
]


@pytest.mark.parametrize("args,pattern,line", CASES, ids=[f"testmcx.sh:{c[2]}" for c in CASES])
def test_cli_regression_case(cli, tmp_path, args, pattern, line):
    out = run(cli, args, tmp_path)
    assert re.search(pattern, out), f"testmcx.sh:{line} expects /{pattern}/ in:\n{out[-3000:]}"


def test_cli_rng_payload(cli, tmp_path, goldens):
    """-D R on a 2x2x2 grid: the generator's first 8 uniforms written through the front-end's
    JNIfTI writer, by the engine and by the reference build on the same input, decode to the same
    floats in the same order; they are the values of test/testmcx.sh:155 (the compressed bytes
    depend on the zlib build the front-end links, so the decoded floats are compared)."""
    import base64
    import zlib

    args = ["--bench", "cube60", "-d", "0", "-s", "testrng222", "--json",
            '{"Shapes":[{"Grid":{"Tag":0,"Size":[2,2,2]}}]}', "-F", "jnii", "-D", "R"]

    def decode(path):
        doc = json.loads(path.read_text())
        return np.frombuffer(zlib.decompress(base64.b64decode(doc["NIFTIData"]["_ArrayZipData_"])), np.float32)

    run(cli, args, tmp_path)
    got = decode(tmp_path / "testrng222.jnii")
    ref_dir = tmp_path / "reference"
    ref_dir.mkdir()
    run(ref_mcx.build(), args, ref_dir)
    assert np.array_equal(got, decode(ref_dir / "testrng222.jnii"))
    # the golden values are listed with x slowest, the field's voxels are stored x fastest
    want = np.asarray(goldens["rng_kat"]["values_rowmajor"], np.float32).reshape(2, 2, 2)
    assert np.array_equal(got.reshape(2, 2, 2, order="F"), want), got


def test_cli_seed_replay(cli, tmp_path):
    """Seeds saved by the CLI (-q 1) and replayed from its own detected-photon file (-E): the
    replay simulates exactly the photons the first run detected and detects every one of them
    again (test/testmcx.sh:137, 142)."""
    a = run(cli, ["--bench", "cube60", "-s", "replaytest", "-q", "1", "-S", "0"], tmp_path)
    b = run(cli, ["--bench", "cube60", "-E", "replaytest_detp.jdat", "-S", "0"], tmp_path)
    det_a = int(re.findall(r"detected\s+([0-9]+) photons", a)[-1])
    sim_b = int(float(re.findall(r"simulated\s+([0-9.]+) photons", b)[-1]))
    det_b = int(re.findall(r"detected\s+([0-9]+) photons", b)[-1])
    assert det_a > 0 and sim_b == det_a and det_b == sim_b, (det_a, sim_b, det_b, b[-2000:])
    assert re.search(r"absorbed:.*3[0-8]\.[0-9]+%", b), b[-2000:]


def test_cli_trajectories_against_the_reference(cli, tmp_path):
    """-D M (test/testmcx.sh:161): the trajectory positions the CLI saves per photon agree with
    the reference build's on the same deck within 5% (testmcx.sh's own check, 6000-9999 positions
    for 100 photons, is one draw of a statistic whose spread at that sample size reaches it; the
    count per photon is heavy-tailed -- photons that wander the whole window scatter ~1000 times --
    so 1e5 photons are needed for its mean to settle within a few per cent)."""
    n = 10 ** 5
    args = ["--bench", "cube60", "-D", "M", "-S", "0", "-d", "0", "-n", str(n)]
    ours = int(re.findall(r"saved trajectory positions:\s*([0-9]+)", run(cli, args, tmp_path))[-1])
    ref_dir = tmp_path / "reference"
    ref_dir.mkdir()
    theirs = int(re.findall(r"saved trajectory positions:\s*([0-9]+)", run(ref_mcx.build(), args, ref_dir))[-1])
    assert 60 * n <= ours <= 100 * n and abs(ours / theirs - 1) < 0.05, (ours, theirs)


def test_cli_files_match_the_python_front_end(cli, tmp_path, engine):
    """The .mc2 fluence and .mch detected photons written by the CLI through mcx_savedata /
    mcx_savedetphoton agree with the pmcx-style front-end's run of the same deck."""
    from mcx_gb300 import problems

    out = run(cli, ["--bench", "cube60b", "-F", "mc2", "-s", "cli", "-n", "1e6", "-E", "1234"], tmp_path)
    ndet = int(re.findall(r"detected\s+([0-9]+) photons", out)[-1])
    flux = np.fromfile(tmp_path / "cli.mc2", dtype=np.float32)
    assert flux.size == 60 ** 3
    raw = (tmp_path / "cli.mch").read_bytes()
    magic, _, maxmedia, detnum, colcount, total, detected, saved = struct.unpack("<4s7I", raw[:32])
    assert magic == b"MCXH" and detnum == 4 and saved == ndet and detected == ndet
    recs = np.frombuffer(raw[64:64 + 4 * colcount * saved], np.float32).reshape((colcount, saved), order="F")
    assert set(np.unique(recs[0]).astype(int)) <= {1, 2, 3, 4}

    res = engine.run(problems.cube60b(1e6))
    ref = res["flux"][..., 0].ravel(order="F")
    assert abs(flux.sum() - ref.sum()) / ref.sum() < 0.01
    n_py = res["detp"].shape[1] if res["detp"].ndim == 2 else len(res["detp"])
    assert abs(ndet - n_py) < 5 * np.sqrt(n_py)


def test_cli_engine_error_goes_through_mcx_error(cli, tmp_path):
    """A deck whose volume labels exceed the media table is refused by the engine, which reports
    through the front-end's mcx_error: MCX's message format and exit code -4 (252)."""
    out = run(cli, ["--bench", "cube60", "--json", json.dumps({"Domain": {"Media": [[0, 0, 1, 1]]}}), "-n", "1e3"],
              tmp_path, rc=256 - 4)
    assert re.search(r"MCX ERROR\(-4\):input media optical properties are less than the labels", out), out[-2000:]


def test_cli_jdat_matches_the_python_writer(cli, tmp_path, engine):
    """The detected-photon .jdat the CLI writes through MCX's own writer (mcx_savejdet; -F jnii is
    the front-end's default) and the one mcx_gb300.mch.save_jdet writes for the Python front-end's
    run of the same deck and seed: the same header fields, and -- the engine's photons having
    per-photon random streams -- the same detected records and seeds, as sets."""
    from mcx_gb300 import mch, problems

    run(cli, ["--bench", "cube60b", "-n", "1e5", "-E", "1234", "-s", "jd", "-q", "1", "-S", "0"], tmp_path)
    info_c, rec_c, seed_c = mch.load_jdet(tmp_path / "jd_detp.jdat")
    # -S 0 on the CLI: no field, so no normalisation and the header's normaliser stays 1, as MCX
    # leaves it (src/mcx_core.cu:3823)
    cfg = problems.cube60b(1e5) | {"seed": 1234, "issaveseed": 1, "issave2pt": 0}
    pc = engine.prepare(cfg)
    res = engine.run_prepared(pc)
    info_p, rec_p, seed_p = mch.load_jdet(mch.save_jdet(tmp_path / "py_detp.jdat", pc, res))
    print({k: (info_c[k], info_p[k]) for k in info_c if k != "Media"})
    for k in ("Version", "MediaNum", "DetNum", "ColumnNum", "TotalPhoton", "DetectedPhoton", "SavedPhoton",
              "LengthUnit", "SeedByte", "Repeat", "SrcNum", "SaveDetFlag", "TotalSource"):
        assert info_c[k] == info_p[k], k
    assert info_p["Normalizer"] == pytest.approx(info_c["Normalizer"], rel=1e-6)
    for mc, mp in zip(info_c["Media"], info_p["Media"]):
        assert all(mp[q] == pytest.approx(mc[q], rel=1e-6, abs=1e-9) for q in ("mua", "mus", "g", "n"))

    def rows(rec, seeds):
        return sorted(rec[:, i].tobytes() + seeds[:, i].tobytes() for i in range(rec.shape[1]))

    assert rec_c.shape == rec_p.shape and rows(rec_c, seed_c) == rows(rec_p, seed_p)
