"""Several devices in one mcx_run_simulation call, and the FP64 field switch.

MCX splits one run's photons over the devices its front-end lists (src/mcx_core.cu:2980-3007)
and merges fields, energies and detected photons (3645-3666, 3716-3770).  With per-photon RNG
streams the devices' photon ranges together are exactly the single-device photon set, so a split
run must reproduce the single-device run: the same counters, the same detected records, the
fluence within FP32 summation order.  The pool gives one GPU per run, so the devices here are
replicas on that one GPU (the same device listed twice): the host threads, the photon split, the
merge and the shared normalisation all run; the kernels of the two sessions never wait on each
other."""

from __future__ import annotations

import numpy as np
import pytest

from mcx_gb300 import problems

pytestmark = pytest.mark.gpu

KEYS = ("n_steps", "n_scatter", "n_deposit", "n_launch", "n_photon", "n_detected")


def _same_run(a, b, tol_total=1e-5):
    for k in KEYS:
        assert a["stat"][k] == b["stat"][k], k
    for k in ("e_launch", "e_escape", "e_detect", "e_absdep", "e_absother"):
        assert abs(a["stat"][k] - b["stat"][k]) <= 1e-8 * max(1.0, abs(b["stat"][k])), k
    fa, fb = a["flux"].astype(np.float64).ravel(), b["flux"].astype(np.float64).ravel()
    assert abs(fa.sum() - fb.sum()) / fb.sum() < tol_total
    hot = fb > np.quantile(fb, 0.99)
    assert (np.abs(fa[hot] - fb[hot]) / fb[hot]).max() < 2e-3
    if "detp" in b:
        ra, rb = a["detp"], b["detp"]
        assert ra.shape == rb.shape
        assert np.array_equal(ra[:, np.lexsort(ra[::-1])], rb[:, np.lexsort(rb[::-1])])


@pytest.mark.parametrize("workload", [None, [3.0, 1.0]])
def test_two_replicas_equal_one_device(engine, workload):
    one = engine.run(problems.workload1(2_000_000, seed=321), devices=[0])
    cfg = problems.workload1(2_000_000, seed=321)
    if workload:
        cfg["workload"] = workload
    two = engine.run(cfg, devices=[0, 0])
    _same_run(two, one)
    assert two["stat"]["launches"] == 2 * one["stat"]["launches"]


def test_replicas_with_respin_and_gate_groups(engine):
    def deck():
        cfg = problems.workload1(600_000, seed=77)
        cfg.update(respin=3, maxgate=20)          # 3 repetitions in each of 3 gate groups
        return cfg

    one = engine.run(deck(), devices=[0])
    three = engine.run(deck(), devices=[0, 0, 0])
    _same_run(three, one)


def test_field_precision_switch(engine):
    """mcxg_set_field_precision(64): mcx_run_simulation accumulates in FP64 (MCX's USE_DOUBLE
    build) and gives the FP64 twin's output bit for bit; 32 restores the production path."""
    from mcx_gb300._lib import lib

    cfg = lambda: problems.workload0(1_000_000, seed=5)  # noqa: E731
    twin = engine.run(cfg(), fp64_field=True)
    lib.mcxg_set_field_precision(64)
    try:
        sw = engine.run(cfg())
    finally:
        lib.mcxg_set_field_precision(32)
    # the same photons summed in FP64: equal up to the order of the FP64 atomic additions, which
    # can move a value across a float rounding boundary
    a, b = sw["flux"].astype(np.float64), twin["flux"].astype(np.float64)
    assert np.abs(a - b).max() <= 2.5e-7 * np.abs(b).max()
    fp32 = engine.run(cfg())
    assert abs(fp32["flux"].astype(np.float64).sum() / b.sum() - 1) < 1e-5
