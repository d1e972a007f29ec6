"""Statistical comparison helpers shared by the parity tests."""

from __future__ import annotations

import numpy as np


def seed_moments(samples: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Mean and standard error over the leading (seed) axis."""
    n = samples.shape[0]
    return samples.mean(axis=0), samples.std(axis=0, ddof=1) / np.sqrt(n)


def voxel_z(a: np.ndarray, b: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """Per-voxel z-scores of two independent seed stacks (Welch), restricted to `mask`."""
    ma, sa = seed_moments(a)
    mb, sb = seed_moments(b)
    se = np.sqrt(sa ** 2 + sb ** 2)
    ok = mask & (se > 0)
    return (ma[ok] - mb[ok]) / se[ok]


def parity_report(a: np.ndarray, b: np.ndarray, mask: np.ndarray) -> dict:
    z = voxel_z(a, b, mask)
    return {
        "voxels": int(z.size),
        "frac_beyond_3se": float(np.mean(np.abs(z) > 3.0)) if z.size else 0.0,
        "mean_z": float(z.mean()) if z.size else 0.0,
        "max_abs_z": float(np.abs(z).max()) if z.size else 0.0,
    }


def assert_parity(a: np.ndarray, b: np.ndarray, mask: np.ndarray, min_voxels: int = 100) -> dict:
    """Per-voxel means within 3 standard errors.

    With 16 seeds per side the z-scores follow a t-like law with ~30 degrees of freedom, for
    which |z| > 3 has probability ~0.5% per voxel; the test allows 2% of voxels beyond 3 SE,
    no voxel beyond 7 SE, and a mean z (systematic shift) below 0.15."""
    rep = parity_report(a, b, mask)
    assert rep["voxels"] >= min_voxels, rep
    assert rep["frac_beyond_3se"] <= 0.02, rep
    assert rep["max_abs_z"] <= 7.0, rep
    assert abs(rep["mean_z"]) <= 0.15, rep
    return rep


def voxel_z_full(a: np.ndarray, b: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """Per-voxel z-scores over the whole grid (0 outside `mask` or where the SE is 0)."""
    ma, sa = seed_moments(a)
    mb, sb = seed_moments(b)
    se = np.sqrt(sa ** 2 + sb ** 2)
    z = np.zeros(ma.shape)
    ok = mask & (se > 0)
    z[ok] = (ma[ok] - mb[ok]) / se[ok]
    return z
