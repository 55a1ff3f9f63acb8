"""Comparison helpers shared by the tests."""
import numpy as np

from aurora_gb300 import types as T

GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden")


def load_golden(name):
    z = np.load(GOLDEN + "/" + name + ".npz")
    d = {k: z[k] for k in z.files}
    d["rays"] = np.ascontiguousarray(d["rays"]).view(T.ray_dtype).reshape(-1)
    if "camera" in d:
        d["camera"] = np.ascontiguousarray(d["camera"]).view(T.camera_dtype).reshape(())
    return d


def closest_vs_reference(hits, ref_tuv, ref_prim):
    """Closest-hit results must equal the reference's bit for bit, except that
    on an exact tie in t the lower prim id wins (the reference keeps the first
    tested triangle). Returns the number of tie-resolved differences."""
    t = hits["t"].view(np.uint32)
    assert np.array_equal(t, ref_tuv[:, 0].view(np.uint32)), "t differs from the reference"
    diff = hits["prim"] != ref_prim
    if diff.any():
        assert np.all(hits["prim"][diff] < ref_prim[diff]), "a differing hit is not a lower-id tie"
    same = ~diff
    assert np.array_equal(hits["u"][same].view(np.uint32), ref_tuv[same, 1].view(np.uint32))
    assert np.array_equal(hits["v"][same].view(np.uint32), ref_tuv[same, 2].view(np.uint32))
    return int(diff.sum())


def hits_equal(a, b):
    """Bitwise equality of two hit arrays."""
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))
