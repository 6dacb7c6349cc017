"""GPU test of the allocation-free entry point sjbg_lazy_hj_noalloc.

Some callers of this library cannot allocate device memory (their host
framework owns every allocation, or they must not allocate in a steady-state
loop).  sjbg_lazy_hj_noalloc lets them join a window with inputs and output in
memory they already own: its scratch is a fixed device array inside the
library.  This test calls it twice in a row through the C ABI and checks both
results against the regular entry point (sjbg_lazy_execute) bit for bit; the
second call also checks that the shared scratch is re-initialised between
calls.  It lives in its own file, collected last, and passes alone or after
the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_fixture

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point_twice(lib, golden, oracle):
    torch = pytest.importorskip("torch")
    fx, meta = load_fixture("lazy_uniform_small"), golden["lazy_uniform_small"]
    W = meta["W"]
    big_l = oracle.gen_uniform(0, 1 << 20, 1, 1 << 20)
    big_r = oracle.gen_uniform(0, 1 << 20, 2, 1 << 20)
    cases = [(fx["left"][:W], fx["right"][:W]), (big_l, big_r), (fx["left"][W:2 * W], fx["right"][W:2 * W])]
    out = torch.zeros(C.sizeof(lib.WindowResult), dtype=torch.uint8, device="cuda")
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, max_tuples_per_window=1 << 20) as j:
        for left, right in cases:
            want = j.lazy_execute(left, right)
            dl = torch.from_numpy(left.view(np.uint8)).cuda()
            dr = torch.from_numpy(right.view(np.uint8)).cuda()
            out.fill_(0xAB)   # the entry point must overwrite every field it reports
            lib.lazy_hj_noalloc(dl.data_ptr(), len(left), dr.data_ptr(), len(right), out.data_ptr())
            torch.cuda.synchronize()
            got = lib.WindowResult.from_buffer_copy(out.cpu().numpy().tobytes())
            assert (got.count, got.prod_checksum, got.status) == (want["count"], want["prod"], 0)
    assert cases[0][0].size and want["count"] > 0


def test_noalloc_rejects_oversized_windows(lib):
    L = lib.load()
    assert L.sjbg_lazy_hj_noalloc(C.c_void_p(16), (1 << 20) + 1, C.c_void_p(16), 1, C.c_void_p(16), None) == 5
    assert L.sjbg_lazy_hj_noalloc(None, 1, None, 1, None, None) == 1
