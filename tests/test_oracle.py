"""CPU tests of the oracle: pinned against the golden fixtures made by the
reference's own CPU joiners, known-answer windows, and (where the reference
sources are present, see SJB_REF_SRC in oracle/Makefile) a live cross-check of
restatement vs reference."""
import numpy as np
import pytest

from helpers import load_fixture, make_tuples, sorted_pairs



# ------------------------------------------------------------------ generator pins
def test_generator_pins(oracle, golden):
    g = golden["generator"]
    assert [int(k) for k in oracle.gen_uniform(10 ** 9, 8, 1, 65536)["key"]] == g["uniform_seed1_dom65536_at1e9"]
    assert [oracle.perm(k, 1 << 24, 3) for k in range(8)] == g["perm_2p24_seed3"]
    assert [oracle.perm(k, 1000, 7) for k in range(8)] == g["perm_1000_seed7"]
    assert [oracle.log_uniform(4, w, 1 << 10, 1 << 20) for w in range(8)] == g["log_uniform_seed4"]
    assert [oracle.pair_hash(1, 2), oracle.pair_hash(0xFFFFFFFF, 0)] == g["pair_hash"]


@pytest.mark.parametrize("name,W,dk", [("lazy_uniform_small", 4096, 4096), ("nlj_small", 2048, 2048)])
def test_generator_reproduces_uniform_fixtures(oracle, name, W, dk):
    fx = load_fixture(name)
    n = len(fx["left_keys"])
    assert np.array_equal(oracle.gen_uniform(0, n, 1, dk)["key"], fx["left_keys"])
    assert np.array_equal(oracle.gen_uniform(0, n, 2, dk)["key"], fx["right_keys"])


@pytest.mark.parametrize("z", [0.5, 1.0, 1.5])
def test_generator_reproduces_zipf_fixtures(oracle, golden, z):
    tag = f"zipf_small_z{str(z).replace('.', 'p')}"
    fx = load_fixture(tag)
    D = 1 << 16
    T = oracle.zipf_table(D, z)
    assert int(np.bitwise_xor.reduce(T)) == golden[tag]["table_xor"]
    n = len(fx["left_keys"])
    assert np.array_equal(oracle.gen_zipf(0, n, 1, T, D, 3)["key"], fx["left_keys"])
    assert np.array_equal(oracle.gen_zipf(0, n, 2, T, D, 3)["key"], fx["right_keys"])


def test_perm_is_bijection(oracle):
    for D in (1, 2, 3, 1000, 4096, 65537):
        v = [oracle.perm(k, D, 9) for k in range(D)]
        assert sorted(v) == list(range(D))


# ------------------------------------------------------------------ restatement vs reference outputs
def test_lazy_hj_smj_counts_match_reference(oracle, golden):
    fx, meta = load_fixture("lazy_uniform_small"), golden["lazy_uniform_small"]
    W, dk, B = meta["W"], meta["distinct_keys"], meta["batch"]
    for w, win in enumerate(meta["windows"]):
        l, r = fx["left"][w * W:(w + 1) * W], fx["right"][w * W:(w + 1) * W]
        assert oracle.lazy_hj_count(l, r, dk, B, threads=3) == win["ref_hj"]
        assert oracle.lazy_smj_count(l, r, dk, threads=3) == win["ref_smj"]
        j = oracle.join(l, r)
        assert (j["count"], j["xor"], j["prod"]) == (win["count"], win["xor"], win["prod"])
        if f"pairs_w{w}" in fx:
            assert np.array_equal(sorted_pairs(j["pairs"]), sorted_pairs(fx[f"pairs_w{w}"]))


def test_nlj_counts_match_reference(oracle, golden):
    fx, meta = load_fixture("nlj_small"), golden["nlj_small"]
    W = meta["W"]
    for w, win in enumerate(meta["windows"]):
        l, r = fx["left"][w * W:(w + 1) * W], fx["right"][w * W:(w + 1) * W]
        assert oracle.lazy_nlj_count(l, r) == win["ref_nlj"] == win["count"]


@pytest.mark.parametrize("z", [0.5, 1.0, 1.5])
def test_zipf_smj_counts_match_reference(oracle, golden, z):
    tag = f"zipf_small_z{str(z).replace('.', 'p')}"
    fx, meta = load_fixture(tag), golden[tag]
    W, D = meta["W"], meta["distinct_keys"]
    for w, win in enumerate(meta["windows"]):
        l, r = fx["left"][w * W:(w + 1) * W], fx["right"][w * W:(w + 1) * W]
        assert oracle.lazy_smj_count(l, r, D, threads=2) == win["ref_smj"] == win["count"]
        j = oracle.join(l, r, enumerate_pairs=False)
        assert j["prod"] == win["prod"]


def test_eager_counts_match_reference(oracle, golden):
    fx, meta = load_fixture("eager_small"), golden["eager_small"]
    bc, wc = oracle.eager_hj(fx["left"], fx["right"], meta["batch"], meta["W"], meta["distinct_keys"])
    assert np.array_equal(bc, fx["batch_counts"])
    assert [int(x) for x in wc] == meta["window_counts"]


def test_batched_windows_match_reference(oracle, golden):
    fx, meta = load_fixture("batched_small"), golden["batched_small"]
    descs, off = [], 0
    for n in meta["sizes"]:
        descs.append((off, n, off, n, 0, 0))
        off += n
    res, _ = oracle.join_windows(fx["left"], fx["right"], descs, enumerate_pairs=True)
    for r, win in zip(res, meta["windows"]):
        assert (r["count"], r["xor"], r["prod"]) == (win["count"], win["xor"], win["prod"])
        assert win["ref_hj"] == win["count"]


# ------------------------------------------------------------------ known answers
def test_kat_all_equal_keys(oracle):
    l, r = make_tuples([7] * 300), make_tuples([7] * 200, first=1000)
    j = oracle.join(l, r)
    assert j["count"] == 300 * 200 == len(j["pairs"])
    assert oracle.lazy_nlj_count(l, r) == 60000
    assert oracle.lazy_smj_count(l, r, 8) == 60000


def test_kat_disjoint_and_empty(oracle):
    l, r = make_tuples(range(0, 100)), make_tuples(range(100, 200))
    assert oracle.join(l, r)["count"] == 0
    e = make_tuples([])
    assert oracle.join(e, r)["count"] == 0 and oracle.join(l, e)["count"] == 0
    assert oracle.join(e, e)["prod"] == 0


def test_kat_permutation(oracle):
    W = 5000
    rng = np.random.default_rng(5)
    l, r = make_tuples(rng.permutation(W)), make_tuples(rng.permutation(W))
    j = oracle.join(l, r)
    assert j["count"] == W
    assert oracle.lazy_hj_count(l, r, W) == W


def test_kat_single_hot_key(oracle):
    keys_l = [3] * 50 + list(range(10, 60))
    keys_r = [3] * 40 + list(range(100, 140))
    j = oracle.join(make_tuples(keys_l), make_tuples(keys_r))
    assert j["count"] == 50 * 40


def test_kat_max_key(oracle):
    l, r = make_tuples([0xFFFFFFFF, 0, 0xFFFFFFFF]), make_tuples([0xFFFFFFFF, 5])
    j = oracle.join(l, r)
    assert j["count"] == 2
    assert sorted_pairs(j["pairs"]).tolist() == [(0 << 32) | 0, (2 << 32) | 0]


def test_prod_checksum_is_pair_sum(oracle):
    rng = np.random.default_rng(11)
    l, r = make_tuples(rng.integers(0, 30, 400)), make_tuples(rng.integers(0, 30, 300), first=77)
    j = oracle.join(l, r)
    s = 0
    for p in j["pairs"]:
        s = (s + oracle.lib().oracle_fr(int(p["r"])) * oracle.lib().oracle_gs(int(p["s"]))) % (1 << 64)
    assert s == j["prod"]
    x = 0
    for p in j["pairs"]:
        x ^= oracle.pair_hash(int(p["r"]), int(p["s"]))
    assert x == j["xor"]


def test_lazy_hj_precondition(oracle):
    with pytest.raises(ValueError):
        oracle.lazy_hj_count(make_tuples([5, 9]), make_tuples([1, 2]), 8)


# ------------------------------------------------------------------ live cross-check with the reference
def test_restatement_equals_reference_live(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("the reference's CPU joiners are not built here (no reference sources)")
    rng = np.random.default_rng(3)
    for dk, n, B in ((64, 1024, 128), (1000, 4096, 512), (1 << 12, 8192, 1024)):
        l = make_tuples(rng.integers(0, dk, n))
        r = make_tuples(rng.integers(0, dk, n), first=n)
        want = oracle.join(l, r, enumerate_pairs=False)["count"]
        assert oracle.ref_lazy_hj_count(l, r, dk, B, 2) == want == oracle.lazy_hj_count(l, r, dk, B, 2)
        assert oracle.ref_lazy_smj_count(l, r, dk, B, 2) == want == oracle.lazy_smj_count(l, r, dk, 2)
        assert oracle.ref_lazy_nlj_count(l[:512], r[:512], 128) == oracle.lazy_nlj_count(l[:512], r[:512])
        bc, wc = oracle.ref_eager_hj(l, r, B, 4 * B, dk)
        bc2, wc2 = oracle.eager_hj(l, r, B, 4 * B, dk)
        assert np.array_equal(bc, bc2) and np.array_equal(wc, wc2)


def test_eager_windows_follow_close_rule(oracle):
    """Eager windows close when either side reached W before an incoming batch
    (include/sjb/windowing/eager/CountBased.cuh:38-46), so with the L,R batch
    order the right side's last batch of a window opens the next window."""
    B, W, dk = 4, 16, 8
    l = oracle.gen_uniform(0, 8 * B, 1, dk)
    r = oracle.gen_uniform(0, 8 * B, 2, dk)
    bc, wc = oracle.eager_hj(l, r, B, W, dk)
    # window 0 = L0..L3 with R0..R2
    j0 = oracle.join(l[:16], r[:12], enumerate_pairs=False)["count"]
    assert wc[0] == j0
    assert int(bc.sum()) == int(wc.sum())
