"""Shared parity helpers for the GPU-vs-oracle tests (test infrastructure)."""
from __future__ import annotations

import numpy as np


def pixel_stats(sum_, sumsq, n):
    n = np.maximum(np.asarray(n, np.float64), 1.0)
    if n.ndim == sum_.ndim - 1:
        n = n[..., None]
    mean = sum_ / n
    var = np.maximum(sumsq / n - mean * mean, 0.0)
    se = np.sqrt(var / n)
    return mean, se


def compare_renders(g_sum, g_sumsq, g_n, o_sum, o_sumsq, o_n):
    """Per-pixel, per-channel comparison of two Monte Carlo renders of the same scene and spp.

    Returns dict(frac_z3, max_abs_z, frac_close, rel_mean_diff): frac_z3 is the fraction of
    pixel channels whose means differ by more than 3 combined standard errors; frac_close the
    fraction agreeing to 1e-4 relative (identical random numbers make most paths identical).
    """
    mg, sg = pixel_stats(g_sum, g_sumsq, g_n)
    mo, so = pixel_stats(o_sum, o_sumsq, o_n)
    d = mg - mo
    se = np.sqrt(sg * sg + so * so)
    tiny = 1e-6 * (1.0 + np.abs(mo))
    z = np.where(se > 0, d / np.maximum(se, 1e-30), np.where(np.abs(d) <= tiny, 0.0, np.inf))
    close = np.abs(d) <= 1e-4 * (1.0 + np.abs(mo))
    return {
        "frac_z3": float(np.mean(np.abs(z) > 3.0)),
        "max_abs_z": float(np.max(np.abs(z))),
        "frac_close": float(np.mean(close)),
        "rel_mean_diff": float(abs(mg.mean() - mo.mean()) / max(abs(mo.mean()), 1e-12)),
        "mean_g": float(mg.mean()),
        "mean_o": float(mo.mean()),
    }


def assert_same_paths(got, want, rtol=1e-4, atol=1e-5, frac=0.999):
    """Two renders of the same paths (same random numbers) by separately compiled kernels: fused
    multiply-adds contracted differently round differently, so values agree to `rtol`; a path whose
    branch (a roulette or lobe decision at a boundary) flips on such a rounding may change a pixel by
    a whole sample, so at least `frac` of the channels must agree and the image means to 1e-5."""
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    close = np.abs(got - want) <= atol + rtol * np.abs(want)
    assert close.mean() >= frac, f"only {close.mean():.5f} of the channels agree"
    assert abs(got.mean() - want.mean()) <= 1e-5 * max(abs(want.mean()), 1e-12) + atol
