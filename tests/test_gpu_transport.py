"""Parity of the GB300 transport kernel with the CPU oracle and the reference goldens.

Every test here runs the engine through its C-ABI (mcx_run_simulation via mcx_gb300.run, or the
session / RNG entry points) on cuda:0.  Tolerances:
  * integer work (RNG streams, photon counts, launch-shape independence of detected records):
    bit-exact;
  * per-voxel fluence: 16 independent seeds per side, per-voxel means within 3 standard errors
    (tests/stats.py) in voxels with more than 1e3 oracle deposits;
  * energy balance launched = absorbed + escaped + detected: 1e-5 relative (FP64 tallies);
  * FP32 field accumulation against the FP64-accumulated twin: 1e-5 relative on the total,
    1e-4 per voxel in the hottest 1% of voxels.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from mcx_gb300 import problems

from .stats import assert_parity
from .test_oracle_golden import diffusion_ratio, glibc_seed_words

pytestmark = pytest.mark.gpu

SEEDS = [1000 + 17 * i for i in range(16)]


@pytest.fixture(scope="module")
def lib(engine):
    from mcx_gb300._lib import lib as L

    return L


def balance(s):
    return abs(s["e_launch"] - (s["e_absdep"] + s["e_absother"] + s["e_escape"] + s["e_detect"])) / s["e_launch"]


# ----------------------------------------------------------------------------- RNG -------------
def test_rng_kat_gpu_bit_exact(lib, goldens):
    seeds = (C.c_uint32 * 4)(*glibc_seed_words())
    out = (C.c_float * 8)()
    assert lib.mcxg_rng_test(seeds, out, 8) == 0, lib.mcxg_last_error()
    got = np.frombuffer(out, np.float32).reshape(2, 2, 2, order="F")
    expect = np.array(goldens["rng_kat"]["values_rowmajor"], np.float32).reshape(2, 2, 2)
    assert np.array_equal(got, expect)


@pytest.mark.parametrize("pid", [0, 1, 12345, 2**40 + 7])
def test_photon_stream_matches_oracle(lib, oracle, pid):
    out = (C.c_float * 256)()
    assert lib.mcxg_photon_stream(987654321, pid, out, 256) == 0
    assert np.array_equal(np.frombuffer(out, np.float32), oracle.photon_stream(987654321, pid, 256))


# ----------------------------------------------------------------------------- goldens ---------
@pytest.mark.parametrize("deck,idx", [("cube60", 0), ("cube60b", 1)])
def test_absorbed_fraction_golden(engine, goldens, deck, idx):
    g = goldens["absorbed_fraction"][idx]
    r = engine.run(getattr(problems, deck)(1e6))
    s = r["stat"]
    frac = s["energyabs"] / s["energytot"]
    assert g["lo"] <= frac < g["hi"], (frac, g["source"])
    assert abs(s["energytot"] - 1e6) <= 10
    assert s["n_photon"] == 1_000_000 and s["error_flags"] == 0
    assert balance(s) < 1e-5


def test_absorbed_fraction_golden_1e8(engine, goldens):
    for g, deck in ((goldens["absorbed_fraction"][2], problems.cube60), (goldens["absorbed_fraction"][3], problems.sphere60b)):
        r = engine.run(deck(g["nphoton"]))
        s = r["stat"]
        frac = s["energyabs"] / s["energytot"]
        assert abs(frac - g["value"]) <= g["tol"], (frac, g["source"])
        assert abs(s["energytot"] - g["nphoton"]) <= 10
        assert balance(s) < 1e-5


def test_detected_golden(engine, goldens):
    g = goldens["detected"]
    r = engine.run(problems.cube60b(g["nphoton"]))
    assert g["lo"] <= r["stat"]["detected"] <= g["hi"]
    assert r["detp"].shape == (3, r["stat"]["detected"])
    assert set(np.unique(r["detp"][0]).astype(int)) <= {1, 2, 3, 4}


def test_boundary_conditions_golden(engine, goldens):
    g = goldens["boundary_detected"]
    cfg = problems.cube60(g["nphoton"])
    cfg["bc"] = g["bc"]
    r = engine.run(cfg)
    assert g["lo"] <= r["stat"]["detected"] <= g["hi"]
    assert np.all(r["detp"][0] == -1)
    g = goldens["cyclic"]
    cfg = problems.cube60(g["nphoton"])
    cfg.update(bc=g["bc"], issavedet=0)
    s = engine.run(cfg)["stat"]
    assert g["lo"] <= s["energyabs"] / s["energytot"] <= g["hi"]
    g = goldens["reflect_bc"]
    cfg = problems.cube60(g["nphoton"])
    cfg.update(bc=g["bc"], isreflect=g["isreflect"])
    s = engine.run(cfg)["stat"]
    assert g["lo"] <= s["energyabs"] / s["energytot"] < g["hi"]


# ----------------------------------------------------------------------------- parity ----------
def _stack_gpu(engine, cfg_fn, n, seeds):
    out = []
    for sd in seeds:
        r = engine.run(cfg_fn(n, seed=sd))
        assert r["stat"]["error_flags"] == 0
        out.append(r["flux"])
    return np.stack(out)


def _stack_oracle(engine, oracle, cfg_fn, n, seeds):
    out, hits = [], None
    pc = engine.prepare(cfg_fn(n))
    for sd in seeds:
        r = oracle.run(pc, seed=sd, hits=True)
        out.append(r["flux"])
        hits = r["hits"] if hits is None else hits + r["hits"]
    return np.stack(out), hits


@pytest.mark.parametrize("name,n", [("workload0", 100000), ("workload1", 50000)])
def test_voxel_parity_16_seeds(engine, oracle, name, n):
    fn = getattr(problems, name)
    gpu = _stack_gpu(engine, fn, n, SEEDS)
    cpu, hits = _stack_oracle(engine, oracle, fn, n, [s + 500000 for s in SEEDS])
    rep = assert_parity(gpu, cpu, hits > 1000)
    print(name, rep)


def _small_layered(n, seed=0):
    cfg = problems.workload2(n, seed=seed, n=64)
    return cfg


def test_voxel_parity_layered_skipvoid(engine, oracle):
    gpu = _stack_gpu(engine, _small_layered, 20000, SEEDS)
    cpu, hits = _stack_oracle(engine, oracle, _small_layered, 20000, [s + 500000 for s in SEEDS])
    rep = assert_parity(gpu, cpu, hits > 1000)
    print("layered64", rep)


def test_step_and_deposit_counts_match_oracle(engine, oracle):
    """Mean steps, scatters and deposits per photon are algorithmic quantities: the GPU's own
    counters must agree with the oracle's within 4 standard errors of the photon mean."""
    for fn, n in ((problems.workload0, 200000), (problems.workload1, 100000)):
        g = engine.run(fn(n, seed=11))["stat"]
        o = oracle.run(engine.prepare(fn(n)), seed=12)["stat"]
        for key in ("n_steps", "n_scatter", "n_deposit"):
            mg, mo = g[key] / g["n_photon"], o[key] / o["n_photon"]
            # per-photon counts have a coefficient of variation below 1.5
            assert abs(mg - mo) <= 4 * 1.5 * mo / np.sqrt(n), (fn.__name__, key, mg, mo)


def test_detected_photons_parity(engine, oracle):
    n = 1_000_000
    g = engine.run(problems.workload1(n, seed=3))
    o = oracle.run(engine.prepare(problems.workload1(n)), seed=4)
    dg, do = g["detp"], o["detp"]
    assert dg.shape[0] == do.shape[0] == 1 + 2 + 2      # detid, nscat(2), ppath(2)
    for det in (1, 2, 3, 4):
        ng, no = int((dg[0] == det).sum()), int((do[0] == det).sum())
        assert abs(ng - no) <= 3 * np.sqrt(ng + no + 1), (det, ng, no)
        if min(ng, no) > 50:
            for row in range(1, 5):
                a, b = dg[row][dg[0] == det], do[row][do[0] == det]
                se = np.sqrt(a.var(ddof=1) / a.size + b.var(ddof=1) / b.size)
                assert abs(a.mean() - b.mean()) <= 4 * se + 1e-6, (det, row, a.mean(), b.mean())


@pytest.mark.parametrize("tile", [-1, 0, 32])
def test_energy_balance_and_fp32_accumulation(engine, lib, tile):
    """FP32 field against the FP64-accumulated twin on identical photon histories, with the
    default, no and a larger shared-memory tile.  The source voxel of cube60 receives ~1e7 equal
    first-flight deposits per 1e7 photons: without the two-copy spill FP32 would drift there by
    ~0.5%; with the exact shared-memory tile and the two-copy spill it stays below 1e-5 there,
    and below 1e-4 in the hottest 1% of voxels."""
    cfg = problems.workload0(10_000_000, seed=77)
    try:
        lib.mcxg_set_launch(0, 0, 0, tile)
        r32 = engine.run(cfg)
        r64 = engine.run(cfg, fp64_field=True)
    finally:
        lib.mcxg_set_launch(0, 0, 0, -1)
    s = r32["stat"]
    assert balance(s) < 1e-5 and balance(r64["stat"]) < 1e-5
    # identical photon histories: the only difference is how the field was accumulated
    assert r32["stat"]["n_steps"] == r64["stat"]["n_steps"]
    f32, f64 = r32["flux"].astype(np.float64), r64["flux"].astype(np.float64)
    tot_err = abs(f32.sum() - f64.sum()) / f64.sum()
    assert tot_err < 1e-5, tot_err
    hot = f64 > np.quantile(f64, 0.99)
    rel = np.abs(f32[hot] - f64[hot]) / f64[hot]
    print("tile", tile, "FP32 vs FP64: total", tot_err, "max rel in hottest 1%", rel.max(), "source voxel",
          f32[29, 29, 0, 0] / f64[29, 29, 0, 0] - 1)
    assert rel.max() < 1e-4, rel.max()
    # sum of flux*mua*Vvox/normaliser recovers the absorbed weight recorded by the kernel
    raw = f32[..., 0] / s["normalizer"]
    assert abs(raw.sum() * 0.005 - s["e_absdep"]) / s["e_absdep"] < 1e-5


def test_diffusion_agreement_gpu(engine):
    r = engine.run(problems.workload0(10_000_000, seed=5))
    ratios = diffusion_ratio(r["flux"], 5e-9)
    assert np.all(np.abs(ratios - 1.0) < 0.05), ratios


# ----------------------------------------------------------------------------- engine ----------
def test_launch_shape_independence(engine, lib):
    """Photons are seeded by index, so block size and refill chunk change nothing but the FP32
    summation order: detected records are bitwise identical, counters identical."""
    cfg = problems.workload1(300000, seed=9)
    try:
        lib.mcxg_set_launch(128, 0, 8, -1)
        a = engine.run(cfg)
        lib.mcxg_set_launch(256, 2, 64, 0)
        b = engine.run(cfg)
    finally:
        lib.mcxg_set_launch(0, 0, 0, -1)
    for key in ("n_steps", "n_scatter", "n_deposit", "n_launch", "n_photon", "n_detected"):
        assert a["stat"][key] == b["stat"][key], key
    da = a["detp"][:, np.lexsort(a["detp"][::-1])]
    db = b["detp"][:, np.lexsort(b["detp"][::-1])]
    assert np.array_equal(da, db)
    # same deposits summed in another order (and, in the second run, with the smallest
    # shared-memory tile, so most hot voxels take plain FP32 atomics): each run's FP32 sum is
    # within ~2e-4 of the FP64 sum in the hottest voxels, so two runs differ by up to twice that
    fa, fb = a["flux"].astype(np.float64), b["flux"].astype(np.float64)
    assert abs(fa.sum() - fb.sum()) / fb.sum() < 1e-5
    hot = fb > np.quantile(fb, 0.99)
    rel = np.abs(fa[hot] - fb[hot]) / fb[hot]
    print("launch shape: max rel diff in hot voxels", rel.max())
    assert rel.max() < 5e-4
    assert abs(a["stat"]["e_absdep"] - b["stat"]["e_absdep"]) / a["stat"]["e_absdep"] < 1e-9


def test_session_matches_run(engine):
    cfg = problems.workload0(200000, seed=21)
    r = engine.run(cfg)
    pc = engine.prepare(problems.workload0(200000, seed=21))
    with engine.Session(pc) as s:
        s.run(0, 200000, 21)
        field, _, _, st = s.read()
    raw = r["flux"] / r["stat"]["normalizer"]
    assert st.n_steps == r["stat"]["n_steps"]
    assert np.allclose(field, raw, rtol=1e-4, atol=1e-6 * raw.max())


def test_respin_accumulates(engine):
    cfg = problems.workload0(100000, seed=31)
    cfg["respin"] = 3
    r = engine.run(cfg)
    assert r["stat"]["n_photon"] == 300000 and r["stat"]["launches"] == 3
    assert abs(r["stat"]["energytot"] - 300000) <= 10


def test_errors_are_reported_not_faulted(engine):
    cfg = problems.workload0(1000)
    cfg["vol"] = cfg["vol"] * 3                      # label 3 with only 2 property rows
    with pytest.raises(engine.MCXError):
        engine.run(cfg)
    cfg = problems.workload0(1000)
    cfg["srctype"] = "pattern"                        # a pattern source without its pattern
    with pytest.raises(engine.MCXError, match="srcpattern"):
        engine.run(cfg)
    # the context is still usable
    assert engine.run(problems.workload0(1000))["stat"]["n_photon"] == 1000


def test_path_length_output_matches_oracle(engine, oracle):
    """Output type 'l' (src/mcx_core.cu:2221-2223): w0 x path per voxel, normalised by the
    launched energy (src/mcx_core.cu:3837-3838); its total is the weighted path length per photon."""
    cfg = problems.workload0(1_000_000, seed=5)
    cfg["outputtype"] = "l"
    g = engine.run(cfg)
    tot_g = float(g["flux"].astype(np.float64).sum())
    pc = engine.prepare(problems.workload0(200_000, seed=6) | {"outputtype": "l"})
    o = oracle.run(pc, seed=6)
    tot_o = float(o["flux"].astype(np.float64).sum())
    assert g["stat"]["error_flags"] == 0
    # per-photon weighted path lengths have a coefficient of variation near 1: 5 SE ~ 1.2%
    assert abs(tot_g - tot_o) <= 0.012 * tot_o, (tot_g, tot_o)


def test_step_cap_stops_photons_and_reports(engine, lib):
    """Failure detection without a GPU fault: a step cap far below what the photons need stops
    them on the device; the kernel returns, the host reports MCX error -6, and the context keeps
    working."""
    try:
        lib.mcxg_set_step_cap(100)
        with pytest.raises(engine.MCXError, match="step cap"):
            engine.run(problems.workload1(200_000, seed=3))
    finally:
        lib.mcxg_set_step_cap(0)
    r = engine.run(problems.workload0(100_000))
    assert r["stat"]["error_flags"] == 0 and r["stat"]["n_photon"] == 100_000


def test_late_time_window_is_deterministic(engine, oracle):
    """A window that starts after t = 0 (here 4-6 ns, 20 gates): every deposit the window test
    admits lands in a gate of the field -- the gate index of t x bin_a - bin_b can round to -1
    right at the window's start and is clamped to the first gate -- so repeated runs give the same
    photons the same paths (bit-identical counters), and the window's absorbed weight agrees with
    the oracle's."""
    def deck():
        c = problems.workload1(600_000, seed=77)
        c.update(tstart=4e-9, tend=6e-9, respin=3, issavedet=0)
        return c

    runs = [engine.run(deck()) for _ in range(3)]
    for k in ("n_steps", "n_scatter", "n_deposit", "n_photon"):
        assert len({r["stat"][k] for r in runs}) == 1, [r["stat"][k] for r in runs]
    assert runs[0]["stat"]["error_flags"] == 0
    o = oracle.run(engine.prepare(problems.workload1(600_000, seed=77) | {"tstart": 4e-9, "tend": 6e-9,
                                                                          "issavedet": 0}),
                   nphoton=600_000, seed=78)
    g = runs[0]["stat"]
    fg, fo = g["e_absdep"] / g["e_launch"], o["stat"]["e_absdep"] / o["stat"]["e_launch"]
    assert abs(fg - fo) < 5 * np.sqrt(fo * (1 - fo) / 600_000) + 1e-4, (fg, fo)
