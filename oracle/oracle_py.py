"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; the product package never does.

Two libraries:
  * ``_build/liboracle.so`` - the C restatement (sjb_oracle.c) of the
    reference's CPU joiners plus the result restatement (count, checksums,
    sorted pairs).  Built from source on first use.
  * ``_ref/libsjbref.so`` - the reference's own CPU joiner sources compiled
    against the TBB-API shim (``make -C oracle ref``).  Only available where
    the reference sources are present (``SJB_REF_SRC``); ``ref_lib()``
    returns None elsewhere.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUPLE_DTYPE = np.dtype([("key", "<u4"), ("val", "<u4"), ("ts", "<u8")])
PAIR_DTYPE = np.dtype([("r", "<u4"), ("s", "<u4")])

_lock = threading.Lock()
_lib = None
_ref = None
_ref_tried = False


class OracleResult(C.Structure):
    _fields_ = [("count", C.c_uint64), ("xor_checksum", C.c_uint64),
                ("prod_checksum", C.c_uint64), ("n_pairs", C.c_uint64)]


class WindowDesc(C.Structure):
    _fields_ = [("left_offset", C.c_uint64), ("n_left", C.c_uint64),
                ("right_offset", C.c_uint64), ("n_right", C.c_uint64),
                ("pairs_offset", C.c_uint64), ("pairs_capacity", C.c_uint64)]


def build(force: bool = False) -> str:
    so = os.path.join(HERE, "_build", "liboracle.so")
    if force or not os.path.exists(so):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return so


def build_ref() -> str | None:
    """Compile the reference's CPU joiners when their sources are present
    (the recipe's `ref-if-present` target; the location comes from the
    SJB_REF_SRC environment variable or the recipe's default)."""
    so = os.path.join(HERE, "_ref", "libsjbref.so")
    subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"], check=True, stdout=subprocess.DEVNULL)
    return so if os.path.exists(so) else None


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(build())
            u64, vp, i32 = C.c_uint64, C.c_void_p, C.c_int
            L.oracle_gen_uniform.argtypes = [vp, u64, u64, u64, u64, i32]
            L.oracle_zipf_table.argtypes = [vp, u64, C.c_double]
            L.oracle_gen_zipf.argtypes = [vp, u64, u64, u64, vp, u64, u64, i32]
            L.oracle_perm.argtypes = [u64, u64, u64]
            L.oracle_perm.restype = C.c_uint32
            L.oracle_log_uniform.argtypes = [u64, u64, u64, u64]
            L.oracle_log_uniform.restype = u64
            for f in ("oracle_pair_hash",):
                getattr(L, f).argtypes = [C.c_uint32, C.c_uint32]
                getattr(L, f).restype = u64
            for f in ("oracle_fr", "oracle_gs"):
                getattr(L, f).argtypes = [C.c_uint32]
                getattr(L, f).restype = u64
            L.oracle_lazy_hj_count.argtypes = [vp, u64, vp, u64, u64, u64, i32, C.POINTER(u64)]
            L.oracle_lazy_smj_count.argtypes = [vp, u64, vp, u64, u64, i32, C.POINTER(u64)]
            L.oracle_lazy_nlj_count.argtypes = [vp, u64, vp, u64]
            L.oracle_lazy_nlj_count.restype = u64
            L.oracle_eager_hj.argtypes = [vp, vp, u64, u64, u64, u64, vp, vp, u64]
            L.oracle_eager_hj.restype = C.c_int64
            L.oracle_join.argtypes = [vp, u64, vp, u64, i32, vp, u64, C.POINTER(OracleResult)]
            L.oracle_join_windows.argtypes = [vp, vp, vp, C.c_uint32, i32, vp, vp, i32]
            _lib = L
    return _lib


def ref_lib():
    """The reference's own CPU joiners, or None where they cannot be built."""
    global _ref, _ref_tried
    with _lock:
        if not _ref_tried:
            _ref_tried = True
            try:
                so = build_ref()
            except (OSError, subprocess.CalledProcessError):
                so = None
            if so:
                R = C.CDLL(so)
                u64, vp = C.c_uint64, C.c_void_p
                R.ref_lazy_hj_count.argtypes = [vp, u64, vp, u64, u64, u64, u64, C.POINTER(u64)]
                R.ref_lazy_smj_count.argtypes = [vp, u64, vp, u64, u64, u64, u64, C.POINTER(u64)]
                R.ref_lazy_nlj_count.argtypes = [vp, u64, vp, u64, u64, C.POINTER(u64)]
                R.ref_eager_hj.argtypes = [vp, vp, u64, u64, u64, u64, vp, vp, u64]
                R.ref_eager_hj.restype = C.c_int64
                _ref = R
    return _ref


# ---------------------------------------------------------------- generators
def gen_uniform(first: int, n: int, seed: int, domain: int, threads: int = 8) -> np.ndarray:
    out = np.empty(n, TUPLE_DTYPE)
    lib().oracle_gen_uniform(_p(out), first, n, seed, domain, threads)
    return out


def zipf_table(n: int, z: float) -> np.ndarray:
    t = np.empty(n, np.uint64)
    lib().oracle_zipf_table(_p(t), n, z)
    return t


def gen_zipf(first: int, n: int, seed: int, table: np.ndarray, domain: int, perm_seed: int,
             threads: int = 8) -> np.ndarray:
    out = np.empty(n, TUPLE_DTYPE)
    lib().oracle_gen_zipf(_p(out), first, n, seed, _p(table), domain, perm_seed, threads)
    return out


def perm(rank: int, domain: int, seed: int) -> int:
    return lib().oracle_perm(rank, domain, seed)


def log_uniform(seed: int, w: int, lo: int, hi: int) -> int:
    return lib().oracle_log_uniform(seed, w, lo, hi)


def pair_hash(r: int, s: int) -> int:
    return lib().oracle_pair_hash(r, s)


# ---------------------------------------------------------------- restated reference joiners
def lazy_hj_count(left, right, distinct_keys, batch_size=0, threads=1) -> int:
    c = C.c_uint64()
    rc = lib().oracle_lazy_hj_count(_p(left), len(left), _p(right), len(right), distinct_keys,
                                    batch_size, threads, C.byref(c))
    if rc:
        raise ValueError("lazy CPU_HJ precondition violated (key >= distinct_keys or ragged batches)")
    return c.value


def lazy_smj_count(left, right, distinct_keys, threads=1) -> int:
    c = C.c_uint64()
    rc = lib().oracle_lazy_smj_count(_p(left), len(left), _p(right), len(right), distinct_keys,
                                     threads, C.byref(c))
    if rc:
        raise ValueError("lazy CPU_SMJ precondition violated (key >= distinct_keys)")
    return c.value


def lazy_nlj_count(left, right) -> int:
    return lib().oracle_lazy_nlj_count(_p(left), len(left), _p(right), len(right))


def eager_hj(left, right, batch_size, window_size, distinct_keys):
    nb = len(left) // batch_size
    bc = np.zeros(2 * nb, np.uint64)
    wc = np.zeros(nb * 2 + 2, np.uint64)
    nw = lib().oracle_eager_hj(_p(left), _p(right), nb, batch_size, window_size, distinct_keys,
                               _p(bc), _p(wc), len(wc))
    if nw < 0:
        raise ValueError("bad eager arguments")
    return bc, wc[:nw]


# ---------------------------------------------------------------- result restatement
def join(left, right, enumerate_pairs=True, pairs_capacity=None):
    """count, xor, prod and the sorted pair list of one window."""
    cap = 0 if not enumerate_pairs else (pairs_capacity if pairs_capacity is not None else 1 << 22)
    pairs = np.empty(max(cap, 1), PAIR_DTYPE)
    res = OracleResult()
    rc = lib().oracle_join(_p(left), len(left), _p(right), len(right), int(enumerate_pairs),
                           _p(pairs) if cap else None, cap, C.byref(res))
    if rc:
        raise MemoryError("oracle_join failed")
    return {"count": res.count, "xor": res.xor_checksum, "prod": res.prod_checksum,
            "pairs": pairs[:res.n_pairs] if enumerate_pairs else None}


def join_windows(left, right, descs, enumerate_pairs=False, pairs_total=0, threads=8):
    """Per-window (count, xor, prod) for descriptor tuples
    (left_offset, n_left, right_offset, n_right, pairs_offset, pairs_capacity)."""
    n = len(descs)
    arr = (WindowDesc * n)(*[WindowDesc(*d) for d in descs])
    res = (OracleResult * n)()
    pairs = np.empty(max(pairs_total, 1), PAIR_DTYPE) if pairs_total else None
    rc = lib().oracle_join_windows(_p(left), _p(right), C.cast(arr, C.c_void_p), n, int(enumerate_pairs),
                                   _p(pairs), C.cast(res, C.c_void_p), threads)
    if rc:
        raise MemoryError("oracle_join_windows failed")
    out = [{"count": r.count, "xor": r.xor_checksum, "prod": r.prod_checksum, "n_pairs": r.n_pairs} for r in res]
    return out, pairs


# ---------------------------------------------------------------- the reference's own joiners
def ref_lazy_hj_count(left, right, distinct_keys, batch_size, threads=1) -> int:
    c = C.c_uint64()
    if ref_lib().ref_lazy_hj_count(_p(left), len(left), _p(right), len(right), distinct_keys, batch_size,
                                   threads, C.byref(c)):
        raise ValueError("ragged batches")
    return c.value


def ref_lazy_smj_count(left, right, distinct_keys, batch_size, threads=1) -> int:
    c = C.c_uint64()
    if ref_lib().ref_lazy_smj_count(_p(left), len(left), _p(right), len(right), distinct_keys, batch_size,
                                    threads, C.byref(c)):
        raise ValueError("ragged batches")
    return c.value


def ref_lazy_nlj_count(left, right, batch_size) -> int:
    c = C.c_uint64()
    if ref_lib().ref_lazy_nlj_count(_p(left), len(left), _p(right), len(right), batch_size, C.byref(c)):
        raise ValueError("ragged batches")
    return c.value


def ref_eager_hj(left, right, batch_size, window_size, distinct_keys):
    nb = len(left) // batch_size
    bc = np.zeros(2 * nb, np.uint64)
    wc = np.zeros(nb * 2 + 2, np.uint64)
    nw = ref_lib().ref_eager_hj(_p(left), _p(right), nb, batch_size, window_size, distinct_keys,
                                _p(bc), _p(wc), len(wc))
    if nw < 0:
        raise ValueError("bad eager arguments")
    return bc, wc[:nw]
