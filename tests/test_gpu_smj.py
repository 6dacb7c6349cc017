"""GPU parity tests of the lazy sort-merge join (radix sort + merge path)
against the oracle and the golden fixtures made by the reference's CPU_SMJ."""
import numpy as np
import pytest

from helpers import load_fixture, make_tuples, sorted_pairs

pytestmark = pytest.mark.gpu


def test_golden_uniform_windows_with_pairs(lib, golden):
    fx, meta = load_fixture("lazy_uniform_small"), golden["lazy_uniform_small"]
    W = meta["W"]
    n = len(meta["windows"])
    pairs = np.zeros(n * W * 4, lib.PAIR_DTYPE)
    with lib.Joiner(lib.ALG_SMJ, lib.LAZY, lib.RESULT_ATOMIC, max_tuples_per_window=W) as j:
        res = j.lazy_execute_batch(fx["left"], fx["right"], [(w * W, W, w * W, W, w * W * 4, W * 4) for w in range(n)],
                                   pairs=pairs)
    for w, (r, win) in enumerate(zip(res, meta["windows"])):
        assert r["count"] == win["ref_smj"] == win["count"]
        assert (r["xor"], r["prod"]) == (win["xor"], win["prod"])
        if f"pairs_w{w}" in fx:
            got = pairs[w * W * 4: w * W * 4 + r["n_pairs"]]
            assert np.array_equal(sorted_pairs(got), sorted_pairs(fx[f"pairs_w{w}"]))


@pytest.mark.parametrize("z", [0.5, 1.0, 1.5])
def test_golden_zipf_counts(lib, golden, z):
    tag = f"zipf_small_z{str(z).replace('.', 'p')}"
    fx, meta = load_fixture(tag), golden[tag]
    W = meta["W"]
    with lib.Joiner(lib.ALG_SMJ, lib.LAZY, max_tuples_per_window=W) as j:
        res = j.lazy_execute_batch(fx["left"], fx["right"], [(w * W, W, w * W, W) for w in range(2)])
    for r, win in zip(res, meta["windows"]):
        assert (r["count"], r["prod"]) == (win["ref_smj"], win["prod"])


def test_smj_window_2p20(lib, oracle):
    """One window of the 2^20-tuple sort-merge shape, keys in [0, 2^20): every pair."""
    W = 1 << 20
    left = oracle.gen_uniform(0, W, 1, W)
    right = oracle.gen_uniform(0, W, 2, W)
    want = oracle.join(left, right)
    pairs = np.zeros(want["count"] + 64, lib.PAIR_DTYPE)
    with lib.Joiner(lib.ALG_SMJ, lib.LAZY, lib.RESULT_ATOMIC, max_tuples_per_window=W) as j:
        got = j.lazy_execute(left, right, pairs=pairs)
    assert (got["count"], got["xor"], got["prod"]) == (want["count"], want["xor"], want["prod"])
    assert np.array_equal(sorted_pairs(pairs[:got["n_pairs"]]), sorted_pairs(want["pairs"]))


def test_golden_batched_uneven_windows(lib, golden):
    fx, meta = load_fixture("batched_small"), golden["batched_small"]
    descs, off = [], 0
    for n in meta["sizes"]:
        descs.append((off, n, off, n))
        off += n
    with lib.Joiner(lib.ALG_SMJ, lib.LAZY, flags=lib.F_XOR, max_tuples_per_window=1 << 12) as j:
        res = j.lazy_execute_batch(fx["left"], fx["right"], descs)
    for r, win in zip(res, meta["windows"]):
        assert (r["count"], r["xor"], r["prod"]) == (win["count"], win["xor"], win["prod"])


def test_smj_edge_cases(lib, oracle):
    cases = [([], []), ([1], []), ([], [2]), ([5], [5]),
             ([7] * 9000, [7] * 5000),                                   # one key group spanning many tiles
             ([7] * 9000, [6] * 10 + [7] * 3 + [8] * 9000),              # right elements after a long left run
             ([0xFFFFFFFF, 1, 0xFFFFFFFF], [0xFFFFFFFF, 0]),
             (list(range(0, 20000, 2)), list(range(0, 20000, 3))),
             ([1 << 31] * 10 + [3] * 4097, [3] * 4097 + [1 << 31] * 7)]
    with lib.Joiner(lib.ALG_SMJ, lib.LAZY, flags=lib.F_XOR, max_tuples_per_window=1 << 16) as j:
        for kl, kr in cases:
            l, r = make_tuples(kl), make_tuples(kr, first=len(kl))
            want = oracle.join(l, r, enumerate_pairs=True, pairs_capacity=1 << 26)
            got = j.lazy_execute(l, r)
            assert (got["count"], got["xor"], got["prod"]) == (want["count"], want["xor"], want["prod"]), (kl[:3], kr[:3])
