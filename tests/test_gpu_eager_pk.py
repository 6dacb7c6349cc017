"""GPU tests of the persistent eager kernel (SJBG_F_PERSISTENT, the role of the
reference's usePK executor GPU_HJ_PK,
src/sjb/windowing/eager/executor/GPU/GPU_HJ_PK.cu:10-89): per-batch counts,
window totals, checksums and pairs equal the golden eager fixture (made by the
reference's own eager CPU_HJ), the oracle, and the per-batch path; batches
posted ahead of their results; device-resident batches; the kernel's bounded
wait for the next batch runs out, is reported as SJBG_E_TIMEOUT, and the
handle goes on with the same window state."""
import time

import numpy as np
import pytest

from helpers import load_fixture, make_tuples, sorted_pairs
from test_gpu_eager import ALGS, alg, expected_windows

pytestmark = pytest.mark.gpu


def feed(j, left, right, B, W, nb, pairs=None, ahead=0):
    """Drive the reference's eager close rule (eager/CountBased.cuh:36-72) over
    batches L0, R0, L1, R1, ...  ahead > 0 posts up to that many batches before
    reading their counts.  Returns (batch counts, [(window result, sorted pairs)])."""
    counts, wins, tot, pending = [], [], [0, 0], []

    def drain():
        while pending:
            counts.append(j.eager_wait(pending.pop(0)))

    def close():
        drain()
        r = j.eager_window_result(pairs)
        wins.append((r, sorted_pairs(pairs[:r["n_pairs"]]) if pairs is not None else None))

    for b in range(nb):
        for side, src in ((0, left), (1, right)):
            if tot[0] >= W or tot[1] >= W:
                close()
                j.eager_clear_states()
                tot = [0, 0]
            batch = src[b * B:(b + 1) * B]
            if ahead:
                pending.append(j.eager_post(batch, side == 0))
                if len(pending) >= ahead:
                    counts.append(j.eager_wait(pending.pop(0)))
            else:
                counts.append(j.eager_execute(batch, side == 0))
            tot[side] += B
    close()
    j.eager_end_of_stream()
    return counts, wins


@pytest.mark.parametrize("name", ALGS)
@pytest.mark.parametrize("ahead", [0, 16])
def test_persistent_matches_golden_and_oracle(lib, golden, oracle, name, ahead):
    fx, meta = load_fixture("eager_small"), golden["eager_small"]
    B, W, nb = meta["batch"], meta["W"], meta["n_batches"]
    want = expected_windows(oracle, fx["left"], fx["right"], B, W, nb)
    pairs = np.zeros(1 << 20, lib.PAIR_DTYPE)
    with lib.Joiner(alg(lib, name), lib.EAGER, lib.RESULT_ATOMIC, flags=lib.F_PERSISTENT, batch_size=B,
                    window_size=W, max_tuples_per_window=W) as j:
        counts, wins = feed(j, fx["left"], fx["right"], B, W, nb, pairs, ahead)
        rc, running, launches = j.eager_pk_status()
    assert counts == [int(x) for x in fx["batch_counts"]]
    assert [r["count"] for r, _ in wins] == meta["window_counts"]
    for (r, p), e in zip(wins, want):
        assert (r["count"], r["xor"], r["prod"]) == (e["count"], e["xor"], e["prod"])
        assert np.array_equal(p, sorted_pairs(e["pairs"]))
    assert rc == 0 and not running and launches >= 1


@pytest.mark.parametrize("name", ALGS)
def test_persistent_count_only_equals_per_batch_path(lib, oracle, name):
    """No pair enumeration (count and prod only), uneven last batches, empty
    batches, and keys that collide often: the persistent kernel and the
    per-batch kernels give the same counts and totals."""
    B, W, nb = 512, 3000, 20
    left = oracle.gen_uniform(0, nb * B, 11, 64)
    right = oracle.gen_uniform(0, nb * B, 12, 64)
    left["key"][::7] = 0xFFFFFFFF   # the tables' empty marker is an ordinary key
    res = {}
    for flags in (0, lib.F_PERSISTENT):
        with lib.Joiner(alg(lib, name), lib.EAGER, flags=flags, batch_size=B, window_size=W,
                        max_tuples_per_window=W) as j:
            counts, wins, tot = [], [], [0, 0]
            for b in range(nb):
                for side, src in ((0, left), (1, right)):
                    if tot[0] >= W or tot[1] >= W:
                        wins.append(j.eager_window_result())
                        j.eager_clear_states()
                        tot = [0, 0]
                    n = B if b % 5 else B // 3   # every fifth batch is short
                    counts.append(j.eager_execute(src[b * B:b * B + n], side == 0))
                    counts.append(j.eager_execute(src[:0], side == 0))   # an empty batch changes nothing
                    tot[side] += n
            wins.append(j.eager_window_result())
            j.eager_end_of_stream()
        res[flags] = (counts, [(w["count"], w["prod"]) for w in wins])
    assert res[0] == res[lib.F_PERSISTENT]
    assert sum(res[0][0]) > 0


@pytest.mark.parametrize("name,W,D,nb", [("SMJ", 1 << 20, 1 << 20, 300), ("NLJ", 65536, 65536, 40),
                                         ("HJ", 1 << 20, 1 << 20, 300)])
def test_persistent_config_shapes(lib, oracle, name, W, D, nb):
    """Batches of 4,096 at the eager workloads' window sizes: every batch count
    and window count equals the oracle's eager CPU_HJ restatement."""
    B = 4096
    left = oracle.gen_uniform(0, nb * B, 1, D)
    right = oracle.gen_uniform(0, nb * B, 2, D)
    want_bc, want_wc = oracle.eager_hj(left, right, B, W, D)
    with lib.Joiner(alg(lib, name), lib.EAGER, flags=lib.F_PERSISTENT, batch_size=B, window_size=W,
                    max_tuples_per_window=W) as j:
        counts, wins = feed(j, left, right, B, W, nb, None, ahead=32)
    assert counts == [int(x) for x in want_bc]
    assert [w["count"] for w, _ in wins] == [int(x) for x in want_wc]


def test_persistent_device_batches(lib, golden):
    torch = pytest.importorskip("torch")
    fx, meta = load_fixture("eager_small"), golden["eager_small"]
    B, W, nb = meta["batch"], meta["W"], meta["n_batches"]
    dl = torch.from_numpy(fx["left"].view(np.uint8)).cuda()
    dr = torch.from_numpy(fx["right"].view(np.uint8)).cuda()
    torch.cuda.synchronize()
    counts, tot = [], [0, 0]
    with lib.Joiner(lib.ALG_HJ, lib.EAGER, flags=lib.F_PERSISTENT, batch_size=B, window_size=W,
                    max_tuples_per_window=W) as j:
        for b in range(nb):
            for side, d in ((0, dl), (1, dr)):
                if tot[0] >= W or tot[1] >= W:
                    j.eager_clear_states()
                    tot = [0, 0]
                counts.append(j.eager_execute(d.data_ptr() + 16 * b * B, side == 0, mem=lib.MEM_DEVICE, n=B))
                tot[side] += B
        j.eager_end_of_stream()
    assert counts == [int(x) for x in fx["batch_counts"]]


@pytest.mark.parametrize("name", ALGS)
def test_persistent_idle_wait_runs_out_and_the_handle_goes_on(lib, golden, name):
    """The kernel waits at most idle_timeout_ms for the next batch.  Posting
    nothing makes that wait run out: the kernel stores the timeout bit in its
    status word and returns, sjbg_eager_pk_status reports SJBG_E_TIMEOUT once,
    and the next batch relaunches the kernel on the same window state."""
    fx, meta = load_fixture("eager_small"), golden["eager_small"]
    B, W = meta["batch"], meta["W"]
    want = [int(x) for x in fx["batch_counts"]]
    with lib.Joiner(alg(lib, name), lib.EAGER, flags=lib.F_PERSISTENT, batch_size=B, window_size=W,
                    max_tuples_per_window=W, idle_timeout_ms=100) as j:
        got = []
        for b in range(3):
            got.append(j.eager_execute(fx["left"][b * B:(b + 1) * B], True))
            got.append(j.eager_execute(fx["right"][b * B:(b + 1) * B], False))
        assert j.eager_pk_status()[1:] == (True, 1)
        time.sleep(0.5)   # five times the limit: the kernel has given up waiting
        rc, running, launches = j.eager_pk_status()
        assert (rc, running, launches) == (4, False, 1)
        assert b"ran out" in lib.load().sjbg_last_error(j.h)
        assert j.eager_pk_status() == (0, False, 1)   # reported once
        for b in range(3, 6):
            got.append(j.eager_execute(fx["left"][b * B:(b + 1) * B], True))
            got.append(j.eager_execute(fx["right"][b * B:(b + 1) * B], False))
        assert j.eager_pk_status() == (0, True, 2)
        j.eager_end_of_stream()
        assert j.eager_pk_status() == (0, False, 2)
    assert got == want[:12]


def test_persistent_errors(lib):
    with lib.Joiner(lib.ALG_HJ, lib.EAGER, batch_size=4, window_size=8, max_tuples_per_window=8) as j:
        with pytest.raises(lib.SjbgError) as e:
            j.eager_post(make_tuples([1, 2, 3, 4]), True)   # not a persistent handle
        assert e.value.code == 8
    with lib.Joiner(lib.ALG_HJ, lib.EAGER, flags=lib.F_PERSISTENT, batch_size=4, window_size=8,
                    max_tuples_per_window=8) as j:
        for _ in range(3):
            j.eager_execute(make_tuples([1, 2, 3, 4]), True)
        with pytest.raises(lib.SjbgError) as e:   # past window_size + batch_size
            j.eager_execute(make_tuples([1, 2, 3, 4]), True)
        assert e.value.code == 5
        with pytest.raises(lib.SjbgError) as e:   # larger than batch_size
            j.eager_execute(make_tuples([1, 2, 3, 4, 5]), False)
        assert e.value.code == 1
        with pytest.raises(lib.SjbgError) as e:
            j.eager_wait(99)
        assert e.value.code == 1
        assert j.eager_execute(make_tuples([3, 3, 9, 9]), False) == 6   # the handle still works
        j.eager_end_of_stream()
