"""The allocation-free entry point mcxg_run_noalloc against the session path.

mcxg_run_noalloc exists for callers that may not call cudaMalloc while they run (an
application that owns all device memory through its own pool, or a latency-bound loop that
cannot take cudaMalloc's implicit device synchronisation): the caller passes every buffer and
the kernel keeps its small bookkeeping in a static device array.  This test allocates the
caller's buffers up front (with torch, as such a caller would with its own pool), then calls
the entry point twice in a row through the C-ABI and checks each result against the existing
session entry point: same counters and detected records bit for bit (same photons), fluence
within the FP32 accumulation tolerance used by tests/test_gpu_transport.py.  The second call
checks that the shared static array is cleared between calls.  The file sorts last so that a
run stopping at the first failure has already run every other test.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from mcx_gb300 import abi, problems

pytestmark = pytest.mark.gpu

N = 200_000
SEED = 4711


def byte_labels(vol32: np.ndarray) -> np.ndarray:
    """MCX uint32 voxels (bit 31 = detector mask) in the engine's byte format."""
    lab = (vol32 & 0x7F).astype(np.uint8)
    lab |= np.where(vol32 & 0x80000000, 0x80, 0).astype(np.uint8)
    return lab


def test_noalloc_matches_session_twice(engine):
    torch = pytest.importorskip("torch")
    from mcx_gb300._lib import lib

    cfg = problems.workload1(N, seed=SEED)
    pc = engine.prepare(cfg)
    nx, ny, nz = pc.dims
    nvox = nx * ny * nz
    ngates = pc.ngates
    reclen = pc.reclen
    maxdet = int(pc.c.maxdetphoton)

    with engine.Session(pc) as s:
        s.run(0, N, SEED)
        ref_field, ref_detp, ref_ndet, ref_st = s.read(max_records=maxdet)
    ref_field = ref_field.reshape(-1, order="F").astype(np.float64)
    ref_rec = ref_detp[: ref_ndet * reclen].reshape((reclen, ref_ndet), order="F")

    dev = torch.device("cuda", 0)
    labels = torch.from_numpy(byte_labels(pc.vol)).to(dev)
    assert lib.mcxg_noalloc_scratch_bytes() <= 8192

    for call in range(2):
        field = torch.zeros(nvox * ngates, dtype=torch.float32, device=dev)
        spill = torch.zeros(nvox * ngates, dtype=torch.float32, device=dev)
        detp = torch.zeros(maxdet * reclen, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        st = abi.Stats()
        rc = lib.mcxg_run_noalloc(C.byref(pc.c), labels.data_ptr(), field.data_ptr(), spill.data_ptr(),
                                  detp.data_ptr(), 0, N, 0, None, C.byref(st))
        assert rc == 0, lib.mcxg_last_error()
        torch.cuda.synchronize()
        assert st.error_flags == 0
        for key in ("n_steps", "n_scatter", "n_deposit", "n_launch", "n_photon"):
            assert getattr(st, key) == getattr(ref_st, key), (call, key)
        assert st.n_detected == ref_ndet
        assert abs(st.e_absdep - ref_st.e_absdep) / ref_st.e_absdep < 1e-9
        got = (field + spill).cpu().numpy().astype(np.float64)
        assert abs(got.sum() - ref_field.sum()) / ref_field.sum() < 1e-4, call
        hot = ref_field > np.quantile(ref_field, 0.99)
        assert (np.abs(got[hot] - ref_field[hot]) / ref_field[hot]).max() < 2e-3, call
        rec = detp.cpu().numpy()[: ref_ndet * reclen].reshape((reclen, ref_ndet), order="F")
        assert np.array_equal(rec[:, np.lexsort(rec[::-1])], ref_rec[:, np.lexsort(ref_rec[::-1])]), call


def test_noalloc_reports_errors_without_stats(engine):
    """Errors come back through the return value even when the caller passes no statistics: a
    run stopped by the per-photon step cap, a label past the medium table, MCX seeding."""
    torch = pytest.importorskip("torch")
    from mcx_gb300._lib import lib

    pc = engine.prepare(problems.workload0(20_000, seed=SEED))
    nx, ny, nz = pc.dims
    nvox = nx * ny * nz
    dev = torch.device("cuda", 0)
    field = torch.zeros(nvox * pc.ngates, dtype=torch.float32, device=dev)
    spill = torch.zeros_like(field)

    def call(labels):
        return lib.mcxg_run_noalloc(C.byref(pc.c), labels.data_ptr(), field.data_ptr(), spill.data_ptr(), None,
                                    0, 20_000, 0, None, None)

    good = torch.from_numpy(byte_labels(pc.vol)).to(dev)
    assert call(good) == 0, lib.mcxg_last_error()
    lib.mcxg_set_step_cap(100)
    try:
        assert call(good) == -6 and b"step cap" in lib.mcxg_last_error()
    finally:
        lib.mcxg_set_step_cap(0)
    bad = good.clone()
    bad[nvox // 2] = int(pc.c.medianum)           # one label past the table
    assert call(bad) == -4
    lib.mcxg_set_seeding(1)
    try:
        assert call(good) == -6 and b"seeding" in lib.mcxg_last_error()
    finally:
        lib.mcxg_set_seeding(0)
    assert call(good) == 0, lib.mcxg_last_error()
