"""Shared helpers of the test suite: fixture loading and result comparison."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
TUPLE_DTYPE = np.dtype([("key", "<u4"), ("val", "<u4"), ("ts", "<u8")])


def tuples_from_keys(keys, first=0):
    """Tuples of a stream whose tuple i has val = ts = first + i (the generator's layout)."""
    t = np.empty(len(keys), TUPLE_DTYPE)
    t["key"] = keys
    idx = np.arange(first, first + len(keys), dtype=np.uint64)
    t["val"] = idx.astype(np.uint32)
    t["ts"] = idx
    return t


def load_fixture(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["left"] = tuples_from_keys(out["left_keys"])
    out["right"] = tuples_from_keys(out["right_keys"])
    return out


def sorted_pairs(pairs):
    """Pairs (structured r/s or Nx2) as a sorted uint64 array r<<32|s."""
    if pairs.dtype.names:
        v = (pairs["r"].astype(np.uint64) << np.uint64(32)) | pairs["s"].astype(np.uint64)
    else:
        v = (pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint64)
    return np.sort(v)


def make_tuples(keys, first=0):
    return tuples_from_keys(np.asarray(keys, dtype=np.uint32), first)
