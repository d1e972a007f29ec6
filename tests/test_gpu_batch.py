"""Batched simulations (mcxg_run_batch): many independent Configs in one CUDA graph.

Photons are seeded by (seed, photon index), so a simulation run inside the batch follows the same
photon histories as the same Config run alone: counters and detected records are identical, the
field differs only by FP32 summation order (the batch also uses the smallest deposit tile).
Repetitions and gate groups run in waves of graphs, with the same photon ranges as a single run.
"""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu


def _small_batch():
    insts = problems.batch_instances(count=10, seed=77, budget_scale=1e-3)
    for c in insts:
        c["nphoton"] = max(c["nphoton"], 20000)
    return insts


def test_batch_matches_single_runs(engine):
    insts = _small_batch()
    res, ms = engine.run_batch(insts, streams=4)
    assert ms > 0 and len(res) == len(insts)
    for cfg, rb in zip(_small_batch(), res):
        ra = engine.run(cfg)
        sa, sb = ra["stat"], rb["stat"]
        for key in ("n_steps", "n_scatter", "n_deposit", "n_launch", "n_photon", "detected"):
            assert sa[key] == sb[key], key
        assert sb["error_flags"] == 0
        for key in ("energytot", "energyabs"):
            assert abs(sa[key] - sb[key]) <= 1e-6 * max(1.0, sa[key]), key
        if "detp" in ra:
            da = ra["detp"][:, np.lexsort(ra["detp"][::-1])]
            db = rb["detp"][:, np.lexsort(rb["detp"][::-1])]
            assert np.array_equal(da, db)
        # same deposits summed in another order: the FP32 accumulation tolerance
        fa, fb = ra["flux"].astype(np.float64), rb["flux"].astype(np.float64)
        assert abs(fa.sum() - fb.sum()) <= 1e-5 * fa.sum()
        hot = fa > np.quantile(fa, 0.99)
        assert np.max(np.abs(fa[hot] - fb[hot]) / fa[hot]) < 5e-4
        assert sb["runtime"] >= 1


def test_batch_energy_balance_and_normalisation(engine):
    insts = _small_batch()
    res, _ = engine.run_batch(insts, streams=2)
    for cfg, r in zip(insts, res):
        s = r["stat"]
        bal = abs(s["e_launch"] - (s["e_absdep"] + s["e_absother"] + s["e_escape"] + s["e_detect"]))
        assert bal <= 1e-5 * s["e_launch"]
        # normalised flux (src/mcx_core.cu:3823-3925): sum(flux * mua * Vvox * tstep) is the
        # weight deposited in the field over the launched weight
        prop = np.asarray(cfg["prop"], np.float32)
        mua = prop[:, 0][cfg["vol"].astype(int)]
        deposited = float((r["flux"][..., 0].astype(np.float64) * mua).sum() * 5e-9)
        # FP32 field sums against the FP64 tally of the same deposits
        assert abs(deposited - s["e_absdep"] / s["e_launch"]) <= 1e-3 * deposited


def test_batch_repetitions_and_gate_groups(engine):
    """Repetitions (respin) and gate groups (maxgate below the gate count) run in waves of
    graphs; each simulation gets what mcx_run_simulation gives it: the same photons (counters and
    detected count identical), energies and the field accumulated over repetitions and groups."""
    insts = _small_batch()[:4]
    insts[1]["respin"] = 3
    insts[2].update(tstep=1e-9, maxgate=2)          # 5 gates in groups of 2: 3 windows
    insts[3].update(respin=-2, tstep=2.5e-9, maxgate=1)
    res, ms = engine.run_batch([dict(c) for c in insts], streams=3)
    assert ms > 0
    for cfg, rb in zip(insts, res):
        ra = engine.run(dict(cfg))
        sa, sb = ra["stat"], rb["stat"]
        assert sb["error_flags"] == 0
        for key in ("n_steps", "n_scatter", "n_photon", "detected", "nphoton"):
            assert sa[key] == sb[key], (key, sa[key], sb[key])
        for key in ("energytot", "energyabs"):
            assert abs(sa[key] - sb[key]) <= 1e-6 * max(1.0, sa[key]), key
        fa, fb = ra["flux"], rb["flux"]
        assert fa.shape == fb.shape
        assert np.abs(fa - fb).max() <= 1e-4 * np.abs(fa).max() + 1e-12


def test_batch_fields_on_the_device(engine):
    """mcxg_run_batch_device: the normalised fields land in the caller's CUDA buffers, equal to
    the host fields of the same batch within FP32 summation order, with the same counters; host
    and device fields can be mixed; the contract's refusals raise MCX errors."""
    import torch

    from mcx_gb300.api import MCXError

    insts = problems.denoise_instances(3, 32, seed=5)
    for c in insts:
        c["nphoton"] = 200_000
    host, _ = engine.run_batch(insts, streams=3)
    bufs = [torch.full((c["vol"].size,), -1.0, device="cuda") for c in insts]
    dev, ms = engine.run_batch(insts, streams=3, device_fields=[bufs[0], None, bufs[2]])
    assert ms > 0 and "flux" not in dev[0] and "flux" in dev[1] and "flux" not in dev[2]
    for i, (h, d) in enumerate(zip(host, dev)):
        for key in ("n_steps", "n_scatter", "n_photon"):
            assert h["stat"][key] == d["stat"][key], key
        for key in ("energytot", "normalizer"):
            assert d["stat"][key] == pytest.approx(h["stat"][key], rel=1e-6), key
        fa = h["flux"][..., 0].ravel(order="F").astype(np.float64)
        fb = (bufs[i].cpu().numpy() if i != 1 else d["flux"][..., 0].ravel(order="F")).astype(np.float64)
        assert (fb >= 0).all()
        assert abs(fa.sum() - fb.sum()) <= 1e-5 * fa.sum()
        hot = fa > np.quantile(fa, 0.99)
        assert np.max(np.abs(fa[hot] - fb[hot]) / fa[hot]) < 5e-4
    with pytest.raises(MCXError):           # wrong size
        engine.run_batch(insts[:1], device_fields=[torch.empty(10, device="cuda")])
    with pytest.raises(MCXError):           # two repetitions
        engine.run_batch([dict(insts[0], respin=2)], device_fields=[bufs[0]])
