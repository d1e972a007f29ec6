"""Parity with the reference MCX CUDA build itself, on the same GPU.

MCX's own binary is compiled from its sources for sm_103a (oracle/ref_mcx.py) and run on the
same inputs.  Skipped when the reference sources are not staged in baseline/_ref/src.

  * same seed, MCX seeding mode: the engine draws the same random streams as MCX (one
    xorshift128+ stream per MCX thread, glibc-rand seed words), so absorbed fraction, detected
    count and fluence agree far more tightly than two independent runs could;
  * 16 independent seeds per side, MCX seeding mode: per-voxel mean fluence within 3 standard
    errors in voxels with more than 1e3 oracle deposits (tests/stats.py);
  * the default per-photon seeding: totals within 0.5%.  MCX's seeding draws its first number
    after seeding from a poorly mixed state (its mean is 0.491 instead of 0.5), which lengthens
    the first flight of every thread's first photon; per-photon streams do not share that bias,
    so the per-voxel 3-SE criterion is applied to the MCX seeding mode.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

from .stats import assert_parity, parity_report, voxel_z_full

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_mcx

    if not ref_mcx.available():
        pytest.skip("reference sources are not staged in baseline/_ref/src")
    ref_mcx.build()
    return ref_mcx


@pytest.fixture
def mcx_seeding(engine):
    from mcx_gb300._lib import lib

    lib.mcxg_set_seeding(1)
    yield
    lib.mcxg_set_seeding(0)


def _shells(f):
    i = np.arange(60) + 0.5 - 29.0
    X, Y, Z = np.meshgrid(i, i, np.arange(60) + 0.5, indexing="ij")
    R = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    return np.array([f[(R >= lo) & (R < lo + 2)].sum() for lo in range(0, 30, 2)])


def test_same_seed_same_streams(engine, ref, mcx_seeding):
    cfg = problems.workload0(10_000_000, seed=1234)
    r = ref.run(cfg)
    o = engine.run(problems.workload0(10_000_000, seed=1234))
    o64 = engine.run(problems.workload0(10_000_000, seed=1234), fp64_field=True)
    fo = o["stat"]["energyabs"] / o["stat"]["energytot"]
    print("absorbed reference", r["absorbed"], "engine", fo)
    # independent 1e7-photon runs differ by ~1e-4; shared streams agree far closer
    assert abs(fo - r["absorbed"]) < 3e-5
    fo_, fr_ = o["flux"][..., 0].astype(np.float64), r["flux"][..., 0].astype(np.float64)
    f64 = o64["flux"][..., 0].astype(np.float64)
    ratio = _shells(fo_) / _shells(fr_)
    src = (29, 29, 0)
    print("shell ratios", ratio, "source voxel: engine FP32 vs FP64", fo_[src] / f64[src] - 1,
          "reference vs FP64", fr_[src] / f64[src] - 1)
    assert np.all(np.abs(ratio[1:] - 1.0) < 2e-4)
    # the source voxel receives ~1e7 equal first-flight deposits; against the FP64 sum of the
    # same photons the engine's FP32 field is exact to 1e-5 there, while MCX's own FP32 two-copy
    # accumulation -- whose primary copy drifts far from zero when thousands of threads hit one
    # voxel at once -- is off by a few 1e-3.  Everywhere else the two agree to 2e-4.
    assert abs(fo_[src] / f64[src] - 1) < 1e-5
    assert abs(fr_[src] / f64[src] - 1) < 1e-2
    cfg = problems.cube60b(1_000_000)
    r = ref.run(cfg)
    o = engine.run(problems.cube60b(1_000_000))
    print("detected reference", r["detected"], "engine", o["stat"]["detected"])
    assert abs(o["stat"]["detected"] - r["detected"]) <= max(10, 0.003 * r["detected"])


@pytest.mark.parametrize("name,n", [("workload0", 1_000_000), ("workload1", 1_000_000)])
def test_parity_16_seeds_mcx_seeding(engine, ref, oracle, mcx_seeding, name, n):
    fn = getattr(problems, name)
    ref_stack = np.stack([ref.run(fn(n, seed=5000 + i))["flux"] for i in range(16)])
    eng_stack = np.stack([engine.run(fn(n, seed=9000 + i))["flux"] for i in range(16)])
    hits = oracle.run(engine.prepare(fn(n)), nphoton=16 * n, seed=77, hits=True)["hits"]
    mask = hits > 1000
    # voxels beyond 7 SE may only be the few next to the source, where MCX's own FP32
    # accumulation is off (see test_same_seed_same_streams); they are reported, then excluded
    z = voxel_z_full(eng_stack, ref_stack, mask)
    far = np.argwhere(np.abs(z) > 7.0)
    print(name, "voxels beyond 7 SE:", far.tolist())
    assert len(far) <= 4 and all(abs(c[0] - 29) <= 1 and abs(c[1] - 29) <= 1 and c[2] <= 1 for c in far), far
    for c in far:
        mask[tuple(c)] = False
    rep = assert_parity(eng_stack, ref_stack, mask)
    print(name, rep)


def test_default_seeding_totals(engine, ref):
    cfg = problems.workload1(10_000_000, seed=99)
    r = ref.run(cfg)
    o = engine.run(problems.workload1(10_000_000, seed=99))
    fo = o["stat"]["energyabs"] / o["stat"]["energytot"]
    assert abs(fo - r["absorbed"]) < 0.005 * r["absorbed"]
    tot_r = r["flux"].astype(np.float64).sum()
    tot_o = o["flux"].astype(np.float64).sum()
    assert abs(tot_o - tot_r) / tot_r < 0.005
    print("default seeding vs reference", parity_report(o["flux"][None], r["flux"][None], np.zeros(1, bool)),
          "absorbed", r["absorbed"], fo)


@pytest.mark.parametrize("name,setting", [
    ("planar", {}),
    ("disk", {"srctype": "disk", "srcpos": [29.0, 29.0, 0.0], "srcparam1": [6.0, 0.0, 0.0, 0.0]}),
    ("isotropic", {"srctype": "isotropic", "srcpos": [29.0, 29.0, 29.0]}),
])
def test_source_shapes_same_seed(engine, ref, mcx_seeding, name, setting):
    """Area and angular sources draw their launch numbers from the photon's stream in MCX's order,
    so in MCX seeding mode the engine and MCX simulate the same photons."""
    def deck():
        cfg = problems.cube60planar(1_000_000)
        cfg.update(setting)
        cfg["seed"] = 4711
        return cfg

    r = ref.run(deck(), keep_field=False)
    o = engine.run(deck())
    fo = o["stat"]["energyabs"] / o["stat"]["energytot"]
    print(name, "absorbed reference", r["absorbed"], "engine", fo, "detected", r["detected"], o["stat"]["detected"])
    assert abs(fo - r["absorbed"]) < 5e-5
    assert abs(o["stat"]["detected"] - r["detected"]) <= max(10, 0.003 * r["detected"])


def test_replay_of_reference_seeds(engine, ref, mcx_seeding):
    """Seeds saved by MCX itself are xorshift128+ states in MCX's layout: replayed by the engine in
    MCX seeding mode, MCX's detected photons are detected again with the same records."""
    cfg = problems.cube60b(1_000_000)
    cfg.update(issaveseed=1, savedetflag="dp", seed=2024)
    r = ref.run(cfg, keep_field=False)
    assert r["seeds"].shape == (16, r["detp"].shape[1])
    rep = problems.cube60b(1)
    rep.update(seed=r["seeds"], detphotons=r["detp"], savedetflag="dp", outputtype="j")
    o = engine.run(rep)
    n = o["stat"]["nphoton"]
    assert n > 0.99 * r["detp"].shape[1]
    # the same arithmetic on the same random numbers: nearly every photon retraces MCX's path
    again = set(map(tuple, np.round(r["detp"].T.astype(np.float64), 3).tolist()))
    mine = [tuple(x) for x in np.round(o["detp"].T.astype(np.float64), 3).tolist()]
    same = sum(1 for x in mine if x in again)
    print("replayed", n, "detected again", o["stat"]["detected"], "with MCX's record", same)
    assert o["stat"]["detected"] >= 0.98 * n
    assert same >= 0.95 * n


@pytest.mark.parametrize("seed", list(range(8)))
def test_random_decks_against_the_reference(engine, ref, seed):
    """The randomised decks of tests/test_gpu_fuzz.py (volume, inclusions, void pocket, media,
    boundary conditions, reflection, gates, source shape, detectors) run by MCX itself: absorbed
    fraction and detected count within 5 standard errors of the engine's."""
    from .test_gpu_fuzz import deck

    n = 1_000_000
    cfg = deck(seed, n)
    cfg["outputtype"] = "x"
    r = ref.run(cfg, keep_field=False)
    g = engine.run(deck(seed, n) | {"outputtype": "x"})["stat"]
    fg, fr = g["energyabs"] / g["energytot"], r["absorbed"]
    se = np.sqrt(2 * max(fg * (1 - fg), 1e-4) / n)
    print(seed, cfg["srctype"], cfg["bc"], "absorbed engine", fg, "reference", fr, "detected", g["detected"], r["detected"])
    assert abs(fg - fr) <= 5 * se + 2e-4, (seed, fg, fr)
    if g["detected"] or r["detected"]:
        assert abs(g["detected"] - r["detected"]) <= 5 * np.sqrt(g["detected"] + r["detected"]) + 3, (seed, g["detected"], r["detected"])


def test_layered_256_parity_16_seeds(engine, ref, oracle, mcx_seeding):
    """The large layered workload at its full 256^3 size (five nested ellipsoid shells, the pencil
    beam entering from outside through void skipping, Fresnel reflection): 16 independent seeds
    per side in MCX seeding mode, per-voxel mean fluence within 3 SE of MCX's own build in voxels
    with more than 1e3 deposits (counted by the oracle on a 2e6-photon sample, scaled to the 1.6e7
    photons of each side), and the absorbed fraction against the oracle within 5 SE."""
    n, seeds = 1_000_000, 16

    def moments(fluxes):
        s = s2 = None
        for f in fluxes:
            f = f.astype(np.float64)
            s = f if s is None else s + f
            s2 = f * f if s2 is None else s2 + f * f
        mean = s / seeds
        se = np.sqrt(np.maximum(s2 / seeds - mean * mean, 0.0) * seeds / (seeds - 1) / seeds)
        return mean, se

    absorbed = []

    def engine_runs():
        for i in range(seeds):
            o = engine.run(problems.workload2(n, seed=9000 + i))
            absorbed.append(o["stat"]["energyabs"] / o["stat"]["energytot"])
            yield o["flux"]

    me, se_e = moments(engine_runs())
    mr, se_r = moments(ref.run(problems.workload2(n, seed=5000 + i))["flux"] for i in range(seeds))
    sample = 2_000_000
    orc = oracle.run(engine.prepare(problems.workload2(sample)), nphoton=sample, seed=77, hits=True)
    mask = orc["hits"] * (seeds * n / sample) > 1000
    se = np.sqrt(se_e ** 2 + se_r ** 2)
    ok = mask & (se > 0)
    z = (me[ok] - mr[ok]) / se[ok]
    rep = {"voxels": int(z.size), "frac_beyond_3se": float(np.mean(np.abs(z) > 3)), "mean_z": float(z.mean()),
           "max_abs_z": float(np.abs(z).max())}
    print("workload2 256^3 vs MCX", rep)
    assert rep["voxels"] >= 1000, rep
    # the voxels next to the entry point, where MCX's own FP32 accumulation is off, may exceed 7 SE
    far = np.argwhere((np.abs((me - mr) / np.where(se > 0, se, 1)) > 7) & ok)
    print("voxels beyond 7 SE:", far.tolist())
    assert len(far) <= 4, far
    assert rep["frac_beyond_3se"] <= 0.02 and abs(rep["mean_z"]) <= 0.15, rep
    fo = orc["stat"]["energyabs"] / orc["stat"]["energytot"]
    fa = float(np.mean(absorbed))
    se_a = np.sqrt(fo * (1 - fo) / sample + np.var(absorbed, ddof=1) / seeds)
    print("absorbed engine", fa, "oracle", fo)
    assert abs(fa - fo) <= 5 * se_a, (fa, fo, se_a)
