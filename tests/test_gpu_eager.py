"""GPU parity tests of the eager joins (hash, nested-loop, sort-merge) against
the reference's eager CPU_HJ batch counts (golden fixture) and the oracle."""
import numpy as np
import pytest

from helpers import load_fixture, make_tuples, sorted_pairs

pytestmark = pytest.mark.gpu

ALGS = ["HJ", "NLJ", "SMJ"]


def alg(lib, name):
    return {"HJ": lib.ALG_HJ, "NLJ": lib.ALG_NLJ, "SMJ": lib.ALG_SMJ}[name]


def window_members(n_batches, B, W):
    """The reference's eager windows (include/sjb/windowing/eager/CountBased.cuh:36-72):
    batches arrive L0,R0,L1,R1,...; before each batch the window closes when either
    side already holds >= W tuples.  Returns per window ([left batches], [right batches])."""
    wins, cur, tot = [], ([], []), [0, 0]
    for b in range(n_batches):
        for side in (0, 1):
            if tot[0] >= W or tot[1] >= W:
                wins.append(cur)
                cur, tot = ([], []), [0, 0]
            cur[side].append(b)
            tot[side] += B
    wins.append(cur)
    return wins


def expected_windows(oracle, left, right, B, W, n_batches):
    out = []
    for lb, rb in window_members(n_batches, B, W):
        l = np.concatenate([left[b * B:(b + 1) * B] for b in lb]) if lb else left[:0]
        r = np.concatenate([right[b * B:(b + 1) * B] for b in rb]) if rb else right[:0]
        out.append(oracle.join(l, r, enumerate_pairs=True, pairs_capacity=1 << 24))
    return out


@pytest.mark.parametrize("name", ALGS)
def test_golden_eager_batch_counts(lib, golden, oracle, name):
    fx, meta = load_fixture("eager_small"), golden["eager_small"]
    B, W, nb = meta["batch"], meta["W"], meta["n_batches"]
    with lib.Joiner(alg(lib, name), lib.EAGER, flags=lib.F_XOR, batch_size=B, window_size=W,
                    max_tuples_per_window=W) as j:
        bc, wins = j.eager_run(fx["left"], fx["right"], nb)
    assert np.array_equal(bc, fx["batch_counts"])
    nw = len(meta["window_counts"])
    assert [w["count"] for w in wins[:nw]] == meta["window_counts"]
    want = expected_windows(oracle, fx["left"], fx["right"], B, W, nb)
    for w, e in zip(wins[:nw], want):
        assert (w["count"], w["xor"], w["prod"]) == (e["count"], e["xor"], e["prod"])


@pytest.mark.parametrize("name", ALGS)
def test_eager_execute_per_batch_with_pairs(lib, golden, oracle, name):
    """The drop-in per-batch call (BaseEagerExecutor::execute) driven with the
    reference's close rule; pairs of each window equal the oracle's."""
    fx, meta = load_fixture("eager_small"), golden["eager_small"]
    B, W, nb = meta["batch"], meta["W"], meta["n_batches"]
    want = expected_windows(oracle, fx["left"], fx["right"], B, W, nb)
    got_counts, got_wins = [], []
    pairs = np.zeros(1 << 20, lib.PAIR_DTYPE)
    with lib.Joiner(alg(lib, name), lib.EAGER, lib.RESULT_ATOMIC, batch_size=B, window_size=W,
                    max_tuples_per_window=W) as j:
        tot = [0, 0]
        for b in range(nb):
            for side, src in ((0, fx["left"]), (1, fx["right"])):
                if tot[0] >= W or tot[1] >= W:
                    r = j.eager_window_result(pairs)
                    got_wins.append((r, sorted_pairs(pairs[:r["n_pairs"]])))
                    j.eager_clear_states()
                    tot = [0, 0]
                got_counts.append(j.eager_execute(src[b * B:(b + 1) * B], side == 0))
                tot[side] += B
        r = j.eager_window_result(pairs)
        got_wins.append((r, sorted_pairs(pairs[:r["n_pairs"]])))
        j.eager_end_of_stream()
    assert got_counts == [int(x) for x in fx["batch_counts"]]
    for (r, p), e in zip(got_wins, want):
        assert (r["count"], r["xor"], r["prod"]) == (e["count"], e["xor"], e["prod"])
        assert np.array_equal(p, sorted_pairs(e["pairs"]))


@pytest.mark.parametrize("name,W,D,nb", [("SMJ", 1 << 20, 1 << 20, 300), ("NLJ", 65536, 65536, 40),
                                         ("HJ", 1 << 20, 1 << 20, 300)])
def test_eager_config_shapes(lib, oracle, name, W, D, nb):
    """Batches of 4,096: sort-merge over windows of 2^20 (keys in [0, 2^20)),
    nested-loop over windows of 65,536 (keys in [0, 2^16))."""
    B = 4096
    left = oracle.gen_uniform(0, nb * B, 1, D)
    right = oracle.gen_uniform(0, nb * B, 2, D)
    want_bc, want_wc = oracle.eager_hj(left, right, B, W, D)
    with lib.Joiner(alg(lib, name), lib.EAGER, flags=lib.F_XOR, batch_size=B, window_size=W,
                    max_tuples_per_window=W) as j:
        bc, wins = j.eager_run(left, right, nb)
    assert np.array_equal(bc, want_bc)
    assert [w["count"] for w in wins[:len(want_wc)]] == [int(x) for x in want_wc]
    want = expected_windows(oracle, left, right, B, W, nb)
    for w, e in zip(wins, want):
        assert (w["xor"], w["prod"]) == (e["xor"], e["prod"])


@pytest.mark.parametrize("W,D,nb", [(1 << 20, 1 << 20, 300), (1 << 14, 64, 24), (1 << 14, 3, 12), (5000, 1 << 12, 9),
                                    (1 << 16, 1 << 30, 33)])
def test_eager_sort_merge_totals_from_batch_count_pass(lib, oracle, W, D, nb):
    """Sort-merge without pair enumeration takes each window's count and prod
    from the pass that forms the batch counts.  Cases: nearly distinct keys;
    key groups of ~500 tuples and of ~11,000 tuples, which span sort tiles of
    4,096 (the part of a group before a tile is found by binary search and
    summed from both ends of its tile); a window of 5,000 with batches of
    4,096, so that windows open alternately with a left and a right batch;
    keys that are all distinct."""
    B = 4096
    left = oracle.gen_uniform(0, nb * B, 5, D)
    right = oracle.gen_uniform(0, nb * B, 6, D)
    want_bc, want_wc = oracle.eager_hj(left, right, B, W, min(D, 1 << 22))
    with lib.Joiner(lib.ALG_SMJ, lib.EAGER, batch_size=B, window_size=W, max_tuples_per_window=W) as j:
        bc, wins = j.eager_run(left, right, nb)
    assert np.array_equal(bc, want_bc)
    members = window_members(nb, B, W)
    assert len(wins) == len(members) == len(want_wc)
    for w, (lb, rb), wc in zip(wins, members, want_wc):
        l = np.concatenate([left[b * B:(b + 1) * B] for b in lb]) if lb else left[:0]
        r = np.concatenate([right[b * B:(b + 1) * B] for b in rb]) if rb else right[:0]
        e = oracle.join(l, r, enumerate_pairs=False)
        assert (w["count"], w["prod"]) == (e["count"], e["prod"]) and w["count"] == int(wc)
        assert w["xor"] is None and w["n_pairs"] == 0


def test_eager_errors(lib):
    with lib.Joiner(lib.ALG_HJ, lib.LAZY) as j:
        with pytest.raises(lib.SjbgError) as e:
            j.eager_execute(make_tuples([1, 2]), True)
        assert e.value.code == 8
    with lib.Joiner(lib.ALG_HJ, lib.EAGER, batch_size=4, window_size=8, max_tuples_per_window=8) as j:
        for _ in range(3):
            j.eager_execute(make_tuples([1, 2, 3, 4]), True)
        with pytest.raises(lib.SjbgError) as e:
            j.eager_execute(make_tuples([1, 2, 3, 4]), True)
        assert e.value.code == 5
