"""GPU tests of the device-resident ingest ring (sjbg_ring_*), the GB300 form
of the reference's lazy count-based windowing over a pinned host ring
(include/sjb/windowing/lazy/CountBased.cuh:45-101): batches land in HBM as
they are pushed, each full window is joined there, and every window's count
and checksums equal the oracle's join of that window's tuples."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def push_all(j, left, right, batch, mem=None, to_dev=None):
    """L0, R0, L1, R1, ... as the reference's source feeds them; returns polled results."""
    out = []
    n = len(left)
    for a in range(0, n, batch):
        for is_left, src in ((True, left), (False, right)):
            part = src[a:a + batch]
            if to_dev is not None:
                ptr, m = to_dev(is_left, a), len(part)
                j.ring_push(ptr, is_left, mem=mem, n=m)
            else:
                j.ring_push(part, is_left)
        out += j.ring_poll()
    return out


def expected(oracle, left, right, W, enumerate_pairs):
    return [oracle.join(left[k * W:(k + 1) * W], right[k * W:(k + 1) * W], enumerate_pairs=enumerate_pairs)
            for k in range(len(left) // W)]


@pytest.mark.parametrize("algo,batch", [("HJ", 4096), ("HJ", 3000), ("SMJ", 4096), ("NLJ", 4096)])
def test_ring_windows_match_oracle(lib, oracle, algo, batch):
    """16 windows of 65,536 tuples per stream, keys uniform in [0, 65,536),
    pushed from pageable host memory in batches of 4,096 (windows are whole
    batches) or 3,000 (batches straddle window boundaries)."""
    W, nw = 65536, 16
    left = oracle.gen_uniform(0, nw * W, 1, W)
    right = oracle.gen_uniform(0, nw * W, 2, W)
    a = {"HJ": lib.ALG_HJ, "SMJ": lib.ALG_SMJ, "NLJ": lib.ALG_NLJ}[algo]
    with lib.Joiner(a, lib.LAZY, flags=lib.F_XOR, max_tuples_per_window=W) as j:
        j.ring_open(W, 4)
        res = push_all(j, left, right, batch)
        st = j.ring_close()
        res += j.ring_poll()
    want = expected(oracle, left, right, W, True)
    assert [r["window_id"] for r in res] == list(range(nw))
    assert st["windows_closed"] == nw and st["tuples_joined"] == 2 * nw * W
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for r, w in zip(res, want):
        assert r["status"] == 0 and (r["n_left"], r["n_right"]) == (W, W)
        assert (r["count"], r["xor"], r["prod"]) == (w["count"], w["xor"], w["prod"])


def test_ring_pinned_and_device_batches(lib, oracle):
    """Pinned host batches are copied asynchronously (the ring reads them in
    place) and device batches device to device; both equal the oracle."""
    torch = pytest.importorskip("torch")
    W, nw, B = 1 << 18, 6, 1 << 14
    left = oracle.gen_uniform(0, nw * W, 5, 1 << 20)
    right = oracle.gen_uniform(0, nw * W, 6, 1 << 20)
    want = expected(oracle, left, right, W, False)
    hl = torch.from_numpy(left.view(np.uint8)).pin_memory()
    hr = torch.from_numpy(right.view(np.uint8)).pin_memory()
    dl, dr = hl.cuda(), hr.cuda()
    torch.cuda.synchronize()
    for mem, bufs in ((lib.MEM_HOST, (hl, hr)), (lib.MEM_DEVICE, (dl, dr))):
        with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, max_tuples_per_window=W) as j:
            j.ring_open(W, 3)
            res = push_all(j, left, right, B, mem=mem,
                           to_dev=lambda is_left, a: bufs[0 if is_left else 1].data_ptr() + 16 * a)
            j.ring_close()
            res += j.ring_poll()
        assert [(r["count"], r["prod"]) for r in res] == [(w["count"], w["prod"]) for w in want], mem


def test_ring_full_when_one_side_runs_ahead(lib, oracle):
    """With two slots, the left side cannot start a third window before the
    right side has completed the first: the push fails with the reference's
    message and changes nothing; after the right side catches up every window
    is joined correctly."""
    W = 8192
    left = oracle.gen_uniform(0, 3 * W, 7, 4096)
    right = oracle.gen_uniform(0, 3 * W, 8, 4096)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, max_tuples_per_window=W) as j:
        j.ring_open(W, 2)
        j.ring_push(left[:2 * W], True)
        with pytest.raises(lib.SjbgError) as e:
            j.ring_push(left[2 * W:], True)
        assert e.value.code == 5 and "Ring buffer is full" in str(e.value)
        j.ring_push(right[:W], False)          # window 0 completes and is joined
        j.ring_push(left[2 * W:], True)        # its slot is reused
        j.ring_push(right[W:], False)
        j.ring_close()
        res = j.ring_poll()
    want = expected(oracle, left, right, W, False)
    assert [(r["window_id"], r["count"], r["prod"]) for r in res] == \
        [(k, w["count"], w["prod"]) for k, w in enumerate(want)]


def test_ring_argument_checks(lib):
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, max_tuples_per_window=1024) as j:
        with pytest.raises(lib.SjbgError):
            j.ring_poll()                       # not open
        with pytest.raises(lib.SjbgError) as e:
            j.ring_open(4096, 2)                # larger than max_tuples_per_window
        assert e.value.code == 5
        with pytest.raises(lib.SjbgError):
            j.ring_open(1024, 1)                # a ring needs two slots
