"""Pixel comparison shared by the GPU-vs-oracle render tests."""
import numpy as np


def compare(name, got, ref):
    """Per-pixel bit equality of two images (rows = pixels), with a report of
    the fraction that is bit-identical, the fraction within 1e-4 and the
    largest error of the rest.  Returns (same, close) boolean arrays."""
    g = np.ascontiguousarray(got, np.float32).reshape(got.shape[0], -1)
    r = np.ascontiguousarray(ref, np.float32).reshape(ref.shape[0], -1)
    same = np.all(g.view(np.uint32) == r.view(np.uint32), axis=1)
    close = np.all(np.abs(g - r) <= 1e-4 * np.maximum(1.0, np.abs(r)), axis=1)
    err = np.abs(g.astype(np.float64) - r.astype(np.float64)).max(axis=1)
    worst = float(err[~same].max()) if (~same).any() else 0.0
    print(f"{name}: {same.mean() * 100:.4f}% of {g.shape[0]} pixels bit-identical, {close.mean() * 100:.4f}% within "
          f"1e-4, largest error elsewhere {worst:.3g}")
    return same, close


def assert_bit_identical(name, got, ref):
    same, _ = compare(name, got, ref)
    assert same.all(), f"{name}: {(~same).sum()} of {same.size} pixels differ"
