"""GPU parity tests of the lazy nested-loop join against the oracle and the
golden fixtures made by the reference's CPU_NLJ."""
import numpy as np
import pytest

from helpers import load_fixture, make_tuples, sorted_pairs

pytestmark = pytest.mark.gpu


def test_golden_nlj_windows_with_pairs(lib, golden):
    fx, meta = load_fixture("nlj_small"), golden["nlj_small"]
    W = meta["W"]
    pairs = np.zeros(2 * W * 4, lib.PAIR_DTYPE)
    with lib.Joiner(lib.ALG_NLJ, lib.LAZY, lib.RESULT_ATOMIC, max_tuples_per_window=W) as j:
        res = j.lazy_execute_batch(fx["left"], fx["right"], [(w * W, W, w * W, W, w * W * 4, W * 4) for w in range(2)],
                                   pairs=pairs)
    for w, (r, win) in enumerate(zip(res, meta["windows"])):
        assert r["count"] == win["ref_nlj"] == win["count"]
        assert (r["xor"], r["prod"]) == (win["xor"], win["prod"])
    assert np.array_equal(sorted_pairs(pairs[:res[0]["n_pairs"]]), sorted_pairs(fx["pairs_w0"]))


def test_nlj_window_65536(lib, oracle):
    """One window of the 65,536-tuple nested-loop shape (keys in [0, 2^16))."""
    W = 65536
    left = oracle.gen_uniform(0, W, 1, W)
    right = oracle.gen_uniform(0, W, 2, W)
    want = oracle.join(left, right)
    pairs = np.zeros(want["count"] + 16, lib.PAIR_DTYPE)
    with lib.Joiner(lib.ALG_NLJ, lib.LAZY, lib.RESULT_ATOMIC, max_tuples_per_window=W) as j:
        got = j.lazy_execute(left, right, pairs=pairs)
    assert (got["count"], got["xor"], got["prod"]) == (want["count"], want["xor"], want["prod"])
    assert np.array_equal(sorted_pairs(pairs[:got["n_pairs"]]), sorted_pairs(want["pairs"]))


def test_nlj_edge_cases(lib, oracle):
    cases = [([], []), ([1], []), ([5], [5]), ([7] * 3000, [7] * 2100), ([0xFFFFFFFF, 1, 1], [1, 0xFFFFFFFF]),
             (list(range(2049)), list(range(1000, 20000)))]
    with lib.Joiner(lib.ALG_NLJ, lib.LAZY, flags=lib.F_XOR, max_tuples_per_window=1 << 16) as j:
        for kl, kr in cases:
            l, r = make_tuples(kl), make_tuples(kr, first=len(kl))
            want = oracle.join(l, r, enumerate_pairs=True, pairs_capacity=1 << 24)
            got = j.lazy_execute(l, r)
            assert (got["count"], got["xor"], got["prod"]) == (want["count"], want["xor"], want["prod"]), (kl[:3], kr[:3])
