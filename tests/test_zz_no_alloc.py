"""GPU test of the allocation-free entry point sjbg_lazy_hj_noalloc.

Some callers of this library cannot allocate device memory: their host
framework owns every device allocation through its own pool, or they run a
steady-state loop that must not allocate.  sjbg_lazy_hj_noalloc lets them join
a window with inputs and output in memory they already own; its scratch is a
fixed device array inside the library.  This test calls it through the C ABI,
several calls in a row, and checks every result bit for bit against the
regular entry point (sjbg_lazy_execute) and the oracle, and the uniform
windows also against the committed golden counts.  Later calls check that the
shared scratch is re-initialised between calls.  The file is collected last
and passes alone or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_fixture

pytestmark = pytest.mark.gpu


def _noalloc(lib, torch, left, right, out, stream=None):
    dl = torch.from_numpy(left.view(np.uint8)).cuda()
    dr = torch.from_numpy(right.view(np.uint8)).cuda()
    out.fill_(0xAB)   # the entry point must overwrite every field it reports
    lib.lazy_hj_noalloc(dl.data_ptr(), len(left), dr.data_ptr(), len(right), out.data_ptr(), stream)
    torch.cuda.synchronize()
    return lib.WindowResult.from_buffer_copy(out.cpu().numpy().tobytes())


def test_noalloc_matches_golden_oracle_and_regular_entry_point(lib, golden, oracle):
    torch = pytest.importorskip("torch")
    fx, meta = load_fixture("lazy_uniform_small"), golden["lazy_uniform_small"]
    W = meta["W"]
    big_l = oracle.gen_uniform(0, 1 << 20, 1, 1 << 20)
    big_r = oracle.gen_uniform(0, 1 << 20, 2, 1 << 20)
    golden_cases = [(fx["left"][w * W:(w + 1) * W], fx["right"][w * W:(w + 1) * W], meta["windows"][w])
                    for w in range(len(meta["windows"]))]
    cases = [(l, r, g) for l, r, g in golden_cases]
    cases += [(big_l, big_r, None),                        # the largest window the scratch holds
              (big_l[:0], big_r, None),                     # empty left side
              (big_l, big_r[:0], None),                     # empty right side
              (big_l[:1], big_r, None),                     # one bucket holds every right tuple
              (big_l, big_r[:1], None),
              (golden_cases[0][0], golden_cases[0][1], golden_cases[0][2])]   # again, after a large window
    out = torch.zeros(C.sizeof(lib.WindowResult), dtype=torch.uint8, device="cuda")
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, max_tuples_per_window=1 << 20) as j:
        for left, right, gold in cases:
            want = j.lazy_execute(left, right)
            got = _noalloc(lib, torch, left, right, out)
            assert (got.count, got.prod_checksum, got.status, got.n_pairs) == (want["count"], want["prod"], 0, 0)
            assert got.partitioner_used == lib.PART_RADIX
            if gold is not None:
                assert (got.count, got.prod_checksum) == (gold["count"], gold["prod"])
            o = oracle.join(left, right, enumerate_pairs=False)
            assert (got.count, got.prod_checksum) == (o["count"], o["prod"])
    assert golden_cases[0][2]["count"] > 0


def test_noalloc_on_a_side_stream(lib, golden):
    torch = pytest.importorskip("torch")
    fx, meta = load_fixture("lazy_uniform_small"), golden["lazy_uniform_small"]
    W = meta["W"]
    out = torch.zeros(C.sizeof(lib.WindowResult), dtype=torch.uint8, device="cuda")
    side = torch.cuda.Stream()
    for w in (1, 2):
        left, right = fx["left"][w * W:(w + 1) * W], fx["right"][w * W:(w + 1) * W]
        with torch.cuda.stream(side):
            got = _noalloc(lib, torch, left, right, out, stream=side.cuda_stream)
        assert (got.count, got.prod_checksum, got.status) == (meta["windows"][w]["count"],
                                                              meta["windows"][w]["prod"], 0)


def test_noalloc_rejects_oversized_windows(lib):
    L = lib.load()
    assert L.sjbg_lazy_hj_noalloc(C.c_void_p(16), (1 << 20) + 1, C.c_void_p(16), 1, C.c_void_p(16), None) == 5
    assert b"2^20" in L.sjbg_last_error(None)
    assert L.sjbg_lazy_hj_noalloc(None, 1, None, 1, None, None) == 1
