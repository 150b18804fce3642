"""Parity metrics of a rendered frame against the oracle's frame."""
from __future__ import annotations

import numpy as np


def psnr(a: np.ndarray, b: np.ndarray, peak: float = 1.0) -> float:
    """PSNR of the clipped values. A NaN in both images (the reference's own 0/0 in a few
    delta-DE orbits) counts as equal; a NaN in one of them as an error of `peak`."""
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    err = np.where(na & nb, 0.0, np.where(na | nb, peak, np.clip(a, 0, peak) - np.clip(b, 0, peak)))
    mse = float(np.mean(err ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def compare(test, ref, rows=None) -> dict:
    """hit/miss mismatch, relative hit-depth error, iteration agreement, shaded PSNR."""
    sl = slice(*rows) if rows else slice(None)
    th, rh = test.hit[sl].astype(bool), ref.hit[sl].astype(bool)
    both = th & rh
    out = {"pixels": int(th.size), "hit_fraction": float(rh.mean()),
           "hit_mismatch": float(np.mean(th != rh))}
    if both.any():
        rel = np.abs(test.depth[sl][both] - ref.depth[sl][both]) / np.abs(ref.depth[sl][both])
        out.update(depth_rel_p50=float(np.percentile(rel, 50)), depth_rel_p99=float(np.percentile(rel, 99)),
                   depth_rel_max=float(rel.max()),
                   iters_agree=float(np.mean(test.iters[sl][both] == ref.iters[sl][both])))
    out["psnr_float"] = psnr(test.image_float[sl], ref.image_float[sl])
    return out
