"""Python binding of libsjbg.so, the GB300 stream-join library (C ABI in include/sjbg.h).

This is a thin ctypes layer: every call goes through the C ABI into the
library's CUDA kernels.  It never falls back to a CPU implementation; when the
library or a GPU is missing, calls raise ``SjbgError``.

Inputs are numpy structured arrays of ``TUPLE_DTYPE`` (host memory) or any
object exposing a device pointer via ``data_ptr()`` (e.g. a torch tensor on
the GPU, viewed as raw bytes) together with ``mem=MEM_DEVICE``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libsjbg.so")

TUPLE_DTYPE = np.dtype([("key", "<u4"), ("val", "<u4"), ("ts", "<u8")])
PAIR_DTYPE = np.dtype([("r", "<u4"), ("s", "<u4")])

# enumerations (values of the reference's enums, include/sjb/windowing/BaseWindowing.cuh)
ALG_NLJ, ALG_HJ, ALG_SMJ = 1, 2, 3
EAGER, LAZY = 0, 1
RESULT_NO_OUTPUT, RESULT_COUNT_KERNEL, RESULT_ESTIMATED_SELECTIVITY, RESULT_BITMAP, RESULT_ATOMIC = 0, 1, 2, 3, 4
PART_AUTO, PART_NONE, PART_RADIX, PART_LEARNED = 0, 1, 2, 3
MEM_HOST, MEM_DEVICE = 0, 1
F_XOR, F_PROFILE, F_AUTOTUNE, F_VERIFY, F_GRAPH, F_PERSISTENT = 0x1, 0x2, 0x4, 0x8, 0x10, 0x20
WR_XOR, WR_PAIRS_TRUNCATED, WR_FALLBACK, WR_RADIX_BY_COST = 0x1, 0x2, 0x4, 0x8

STATUS = {0: "OK", 1: "E_INVALID", 2: "E_NOMEM", 3: "E_CUDA", 4: "E_TIMEOUT", 5: "E_CAPACITY",
          6: "E_UNSUPPORTED", 7: "E_BUDGET", 8: "E_STATE", 9: "E_MISMATCH"}

EXPORTS = [
    "sjbg_create", "sjbg_destroy", "sjbg_last_error", "sjbg_set_stream", "sjbg_version",
    "sjbg_lazy_execute", "sjbg_lazy_execute_ring", "sjbg_lazy_execute_batch",
    "sjbg_eager_execute", "sjbg_eager_clear_states", "sjbg_eager_window_result", "sjbg_eager_end_of_stream",
    "sjbg_eager_post", "sjbg_eager_wait", "sjbg_eager_pk_status",
    "sjbg_eager_run", "sjbg_stream_open", "sjbg_stream_push", "sjbg_stream_poll", "sjbg_stream_close",
    "sjbg_ring_open", "sjbg_ring_push", "sjbg_ring_poll", "sjbg_ring_close",
    "sjbg_generate", "sjbg_kernel_stats", "sjbg_kernel_stats_reset", "sjbg_launch_count",
    "sjbg_lazy_hj_noalloc", "sjbg_zipf_table",
]


class SjbgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("algorithm", C.c_uint32), ("progressiveness", C.c_uint32), ("result_mode", C.c_uint32),
                ("partitioner", C.c_uint32), ("batch_size", C.c_uint64), ("max_tuples_per_window", C.c_uint64),
                ("window_size", C.c_uint64), ("num_distinct_keys", C.c_uint64), ("flags", C.c_uint32),
                ("radix_bits", C.c_uint32), ("learned_leaves", C.c_uint32), ("sample_rate", C.c_float),
                ("overflow_bound", C.c_float), ("device", C.c_int32), ("hbm_budget_bytes", C.c_uint64),
                ("idle_timeout_ms", C.c_uint32), ("reserved", C.c_uint32)]


class WindowResult(C.Structure):
    _fields_ = [("count", C.c_uint64), ("xor_checksum", C.c_uint64), ("prod_checksum", C.c_uint64),
                ("n_pairs", C.c_uint64), ("status", C.c_uint32), ("flags", C.c_uint32),
                ("partitioner_used", C.c_uint32), ("ms", C.c_float)]

    def as_dict(self):
        return {"count": self.count, "xor": self.xor_checksum if self.flags & WR_XOR else None,
                "prod": self.prod_checksum, "n_pairs": self.n_pairs, "status": self.status, "flags": self.flags,
                "partitioner_used": self.partitioner_used, "ms": self.ms}


def window_dicts(res) -> list:
    """The windows of a WindowResult array filled by sjbg_eager_run: entries
    past the stream's last window carry status E_INVALID and are dropped.  Only
    the windows themselves are converted (a per-entry loop over all 2n + 2
    slots costs milliseconds of host time per call)."""
    mw = len(res)
    words = np.frombuffer(res, dtype=np.uint32).reshape(mw, C.sizeof(WindowResult) // 4)
    absent = np.flatnonzero(words[:, WindowResult.status.offset // 4] == 1)
    n = int(absent[0]) if absent.size else mw
    return [res[i].as_dict() for i in range(n)]


class WindowDesc(C.Structure):
    _fields_ = [("left_offset", C.c_uint64), ("n_left", C.c_uint64), ("right_offset", C.c_uint64),
                ("n_right", C.c_uint64), ("pairs_offset", C.c_uint64), ("pairs_capacity", C.c_uint64)]


class StreamWindow(C.Structure):
    _fields_ = [("result", WindowResult), ("window_id", C.c_uint64), ("n_left", C.c_uint64),
                ("n_right", C.c_uint64)]

    def as_dict(self):
        d = self.result.as_dict()
        d.update(window_id=self.window_id, n_left=self.n_left, n_right=self.n_right)
        return d


class StreamStats(C.Structure):
    _fields_ = [("windows_closed", C.c_uint64), ("tuples_joined", C.c_uint64), ("windows_rejected", C.c_uint64),
                ("fallbacks", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("busy_ms", C.c_double)]


_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Load libsjbg.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise SjbgError(6, f"{path} is missing: build it with gpu-stream-join-benchmark_gb300/build.py")
        L = C.CDLL(path)
        vp, u64, u32, i32 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int
        L.sjbg_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
        L.sjbg_destroy.argtypes = [vp]
        L.sjbg_last_error.argtypes = [vp]
        L.sjbg_last_error.restype = C.c_char_p
        L.sjbg_set_stream.argtypes = [vp, vp]
        L.sjbg_lazy_execute.argtypes = [vp, vp, u64, vp, u64, u32, vp, u64, C.POINTER(WindowResult)]
        L.sjbg_lazy_execute_ring.argtypes = [vp, vp, vp, u64, vp, vp, u64, vp, u64, C.POINTER(WindowResult)]
        L.sjbg_lazy_execute_batch.argtypes = [vp, vp, vp, u32, vp, u32, vp, vp]
        L.sjbg_eager_execute.argtypes = [vp, vp, u64, i32, u32, C.POINTER(u64)]
        L.sjbg_eager_clear_states.argtypes = [vp]
        L.sjbg_eager_window_result.argtypes = [vp, vp, u64, C.POINTER(WindowResult)]
        L.sjbg_eager_end_of_stream.argtypes = [vp]
        L.sjbg_eager_post.argtypes = [vp, vp, u64, i32, u32, C.POINTER(u64)]
        L.sjbg_eager_wait.argtypes = [vp, u64, C.POINTER(u64)]
        L.sjbg_eager_pk_status.argtypes = [vp, C.POINTER(i32), C.POINTER(u64)]
        L.sjbg_eager_run.argtypes = [vp, vp, vp, u64, u32, vp, vp, u32]
        L.sjbg_stream_open.argtypes = [vp, u64]
        L.sjbg_stream_push.argtypes = [vp, vp, u64, i32, u32]
        L.sjbg_stream_poll.argtypes = [vp, vp, u32, C.POINTER(u32)]
        L.sjbg_stream_close.argtypes = [vp, C.POINTER(StreamStats)]
        L.sjbg_ring_open.argtypes = [vp, u64, u32]
        L.sjbg_ring_push.argtypes = [vp, vp, u64, i32, u32]
        L.sjbg_ring_poll.argtypes = [vp, vp, u32, C.POINTER(u32)]
        L.sjbg_ring_close.argtypes = [vp, C.POINTER(StreamStats)]
        L.sjbg_generate.argtypes = [vp, vp, u64, u64, u64, u64, vp, u64]
        L.sjbg_kernel_stats.argtypes = [vp, u32, C.c_char_p, C.c_size_t, C.POINTER(u64), C.POINTER(C.c_double)]
        L.sjbg_kernel_stats_reset.argtypes = [vp]
        L.sjbg_launch_count.argtypes = [vp]
        L.sjbg_launch_count.restype = u64
        L.sjbg_lazy_hj_noalloc.argtypes = [vp, u64, vp, u64, vp, vp]
        L.sjbg_zipf_table.argtypes = [vp, u64, C.c_double]
        _lib = L
    return _lib


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    if isinstance(a, int):
        return C.c_void_p(a)
    raise TypeError(f"cannot take a pointer of {type(a)}")


def _len(a, dtype=TUPLE_DTYPE) -> int:
    if isinstance(a, np.ndarray):
        return len(a)
    if hasattr(a, "numel") and hasattr(a, "element_size"):
        return a.numel() * a.element_size() // dtype.itemsize
    raise TypeError("length of a device buffer must be given explicitly")


def zipf_table(n: int, z: float) -> np.ndarray:
    """Zipf(z) CDF table over n ranks for sjbg_generate (host memory)."""
    t = np.empty(n, np.uint64)
    rc = load().sjbg_zipf_table(t.ctypes.data_as(C.c_void_p), n, z)
    if rc:
        raise SjbgError(rc, "bad Zipf table arguments")
    return t


def lazy_hj_noalloc(left_dev_ptr: int, n_left: int, right_dev_ptr: int, n_right: int, out_dev_ptr: int,
                    stream: int | None = None) -> None:
    """The allocation-free lazy hash join (device inputs, device result record)."""
    L = load()
    rc = L.sjbg_lazy_hj_noalloc(C.c_void_p(left_dev_ptr), n_left, C.c_void_p(right_dev_ptr), n_right,
                                C.c_void_p(out_dev_ptr), C.c_void_p(stream) if stream else None)
    if rc:
        raise SjbgError(rc, L.sjbg_last_error(None).decode())


class Joiner:
    """One executor handle (sjbg_create / sjbg_destroy)."""

    def __init__(self, algorithm=ALG_HJ, progressiveness=LAZY, result_mode=RESULT_NO_OUTPUT,
                 partitioner=PART_AUTO, batch_size=0, max_tuples_per_window=1 << 26, window_size=0,
                 num_distinct_keys=0, flags=0, radix_bits=0, learned_leaves=0, sample_rate=0.0,
                 overflow_bound=0.0, device=0, hbm_budget_bytes=0, idle_timeout_ms=0):
        self.lib = load()
        self.cfg = Config(algorithm, progressiveness, result_mode, partitioner, batch_size, max_tuples_per_window,
                          window_size, num_distinct_keys, flags, radix_bits, learned_leaves, sample_rate,
                          overflow_bound, device, hbm_budget_bytes, idle_timeout_ms, 0)
        h = C.c_void_p()
        rc = self.lib.sjbg_create(C.byref(self.cfg), C.byref(h))
        if rc:
            raise SjbgError(rc, self.lib.sjbg_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.sjbg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc:
            raise SjbgError(rc, self.lib.sjbg_last_error(self.h).decode())

    def set_stream(self, stream_handle: int | None):
        self._check(self.lib.sjbg_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None))

    # ---- lazy
    def lazy_execute(self, left, right, mem=MEM_HOST, n_left=None, n_right=None, pairs=None, pairs_capacity=0):
        res = WindowResult()
        nl = n_left if n_left is not None else _len(left)
        nr = n_right if n_right is not None else _len(right)
        if pairs is not None and not pairs_capacity:
            pairs_capacity = _len(pairs, PAIR_DTYPE)
        self._check(self.lib.sjbg_lazy_execute(self.h, _ptr(left), nl, _ptr(right), nr, mem, _ptr(pairs),
                                               pairs_capacity, C.byref(res)))
        return res.as_dict()

    def lazy_execute_ring(self, left_ring, left_offsets, right_ring, right_offsets, pairs=None):
        res = WindowResult()
        lo = np.ascontiguousarray(left_offsets, np.uint64)
        ro = np.ascontiguousarray(right_offsets, np.uint64)
        cap = len(pairs) if pairs is not None else 0
        self._check(self.lib.sjbg_lazy_execute_ring(self.h, _ptr(left_ring), _ptr(lo), len(lo), _ptr(right_ring),
                                                    _ptr(ro), len(ro), _ptr(pairs), cap, C.byref(res)))
        return res.as_dict()

    def lazy_execute_batch(self, left, right, windows, mem=MEM_HOST, pairs=None):
        """windows: list of (left_offset, n_left, right_offset, n_right[, pairs_offset, pairs_capacity])."""
        n = len(windows)
        descs = (WindowDesc * n)(*[WindowDesc(*(tuple(w) + (0, 0))[:6]) for w in windows])
        res = (WindowResult * n)()
        self._check(self.lib.sjbg_lazy_execute_batch(self.h, _ptr(left), _ptr(right), mem, C.cast(descs, C.c_void_p),
                                                     n, _ptr(pairs), C.cast(res, C.c_void_p)))
        return [r.as_dict() for r in res]

    def lazy_execute_batch_raw(self, left_ptr: int, right_ptr: int, descs, res, mem=MEM_DEVICE, pairs_ptr=None):
        """Pre-built ctypes descriptor/result arrays (no per-call Python allocation)."""
        self._check(self.lib.sjbg_lazy_execute_batch(self.h, C.c_void_p(left_ptr), C.c_void_p(right_ptr), mem,
                                                     C.cast(descs, C.c_void_p), len(descs),
                                                     C.c_void_p(pairs_ptr) if pairs_ptr else None,
                                                     C.cast(res, C.c_void_p)))

    # ---- eager
    def eager_execute(self, batch, is_left: bool, mem=MEM_HOST, n=None):
        c = C.c_uint64()
        self._check(self.lib.sjbg_eager_execute(self.h, _ptr(batch), n if n is not None else _len(batch),
                                                int(is_left), mem, C.byref(c)))
        return c.value

    def eager_clear_states(self):
        self._check(self.lib.sjbg_eager_clear_states(self.h))

    def eager_window_result(self, pairs=None):
        res = WindowResult()
        cap = len(pairs) if pairs is not None else 0
        self._check(self.lib.sjbg_eager_window_result(self.h, _ptr(pairs), cap, C.byref(res)))
        return res.as_dict()

    def eager_end_of_stream(self):
        self._check(self.lib.sjbg_eager_end_of_stream(self.h))

    def eager_post(self, batch, is_left: bool, mem=MEM_HOST, n=None) -> int:
        """Post a batch to the persistent kernel (F_PERSISTENT handles); returns its ticket."""
        t = C.c_uint64()
        self._check(self.lib.sjbg_eager_post(self.h, _ptr(batch), n if n is not None else _len(batch),
                                             int(is_left), mem, C.byref(t)))
        return t.value

    def eager_wait(self, ticket: int) -> int:
        """New matches of a posted batch."""
        c = C.c_uint64()
        self._check(self.lib.sjbg_eager_wait(self.h, ticket, C.byref(c)))
        return c.value

    def eager_pk_status(self):
        """(status code, running, launches) of the persistent kernel; status 4
        (E_TIMEOUT) once after the kernel's wait for the next batch ran out."""
        running, launches = C.c_int32(), C.c_uint64()
        rc = self.lib.sjbg_eager_pk_status(self.h, C.byref(running), C.byref(launches))
        if rc not in (0, 4):
            self._check(rc)
        return rc, bool(running.value), launches.value

    def eager_run(self, left, right, n_batches, mem=MEM_HOST, max_windows=None):
        bc = np.zeros(2 * n_batches, np.uint64)
        mw = max_windows if max_windows is not None else 2 * n_batches + 2
        res = (WindowResult * mw)()
        self._check(self.lib.sjbg_eager_run(self.h, _ptr(left), _ptr(right), n_batches, mem, _ptr(bc),
                                            C.cast(res, C.c_void_p), mw))
        return bc, window_dicts(res)

    # ---- streaming
    def stream_open(self, window_ns: int):
        self._check(self.lib.sjbg_stream_open(self.h, window_ns))

    def stream_push(self, batch, is_left: bool, mem=MEM_HOST, n=None):
        self._check(self.lib.sjbg_stream_push(self.h, _ptr(batch), n if n is not None else _len(batch),
                                              int(is_left), mem))

    def stream_poll(self, max_out=1024):
        """Closed windows in id order: result fields plus window_id, n_left, n_right."""
        res = (StreamWindow * max_out)()
        n = C.c_uint32()
        self._check(self.lib.sjbg_stream_poll(self.h, C.cast(res, C.c_void_p), max_out, C.byref(n)))
        return [res[i].as_dict() for i in range(n.value)]

    def stream_close(self):
        st = StreamStats()
        self._check(self.lib.sjbg_stream_close(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in StreamStats._fields_}

    # ---- device-resident ingest ring (count-based lazy windows)
    def ring_open(self, window_tuples: int, depth: int = 4):
        self._check(self.lib.sjbg_ring_open(self.h, window_tuples, depth))

    def ring_push(self, batch, is_left: bool, mem=MEM_HOST, n=None):
        self._check(self.lib.sjbg_ring_push(self.h, _ptr(batch), n if n is not None else _len(batch),
                                            int(is_left), mem))

    def ring_poll(self, max_out=1024):
        """Finished windows in window order: result fields plus window_id, n_left, n_right."""
        res = (StreamWindow * max_out)()
        n = C.c_uint32()
        self._check(self.lib.sjbg_ring_poll(self.h, C.cast(res, C.c_void_p), max_out, C.byref(n)))
        return [res[i].as_dict() for i in range(n.value)]

    def ring_close(self):
        st = StreamStats()
        self._check(self.lib.sjbg_ring_close(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in StreamStats._fields_}

    # ---- utilities
    def generate(self, dev_ptr: int, first: int, n: int, seed: int, domain: int, zipf_table_ptr: int | None = None,
                 perm_seed: int = 0):
        self._check(self.lib.sjbg_generate(self.h, C.c_void_p(dev_ptr), first, n, seed, domain,
                                           C.c_void_p(zipf_table_ptr) if zipf_table_ptr else None, perm_seed))

    def kernel_stats(self):
        out = {}
        i = 0
        name = C.create_string_buffer(128)
        while True:
            launches, ms = C.c_uint64(), C.c_double()
            if self.lib.sjbg_kernel_stats(self.h, i, name, 128, C.byref(launches), C.byref(ms)):
                break
            out[name.value.decode()] = (launches.value, ms.value)
            i += 1
        return out

    def kernel_stats_reset(self):
        self._check(self.lib.sjbg_kernel_stats_reset(self.h))

    def launch_count(self) -> int:
        return self.lib.sjbg_launch_count(self.h)
