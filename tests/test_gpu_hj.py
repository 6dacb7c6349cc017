"""GPU parity tests of the lazy hash join (through the C ABI) against the
oracle and the golden fixtures made by the reference's CPU joiners."""
import numpy as np
import pytest

from helpers import load_fixture, make_tuples, sorted_pairs

pytestmark = pytest.mark.gpu


def windows_of(n_windows, W):
    return [(w * W, W, w * W, W, w * W * 4, W * 4) for w in range(n_windows)]


@pytest.mark.parametrize("part", ["radix", "learned"])
def test_golden_uniform_windows_with_pairs(lib, golden, part):
    fx, meta = load_fixture("lazy_uniform_small"), golden["lazy_uniform_small"]
    W = meta["W"]
    nwin = len(meta["windows"])
    pairs = np.zeros(nwin * W * 4, lib.PAIR_DTYPE)
    p = lib.PART_RADIX if part == "radix" else lib.PART_LEARNED
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, lib.RESULT_ATOMIC, partitioner=p, max_tuples_per_window=W) as j:
        res = j.lazy_execute_batch(fx["left"], fx["right"], windows_of(nwin, W), pairs=pairs)
    for w, (r, win) in enumerate(zip(res, meta["windows"])):
        assert r["count"] == win["count"] == win["ref_hj"]
        assert r["xor"] == win["xor"] and r["prod"] == win["prod"]
        got = pairs[w * W * 4: w * W * 4 + r["n_pairs"]]
        if f"pairs_w{w}" in fx:
            assert np.array_equal(sorted_pairs(got), sorted_pairs(fx[f"pairs_w{w}"]))


def test_config_uniform_16x65536(lib, oracle):
    """The 16 x 65,536 uniform workload: count, xor and prod per window."""
    W, n = 65536, 16
    left = oracle.gen_uniform(0, n * W, 1, 65536)
    right = oracle.gen_uniform(0, n * W, 2, 65536)
    descs = [(w * W, W, w * W, W, 0, 0) for w in range(n)]
    want, _ = oracle.join_windows(left, right, descs, enumerate_pairs=True)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, lib.RESULT_NO_OUTPUT, flags=lib.F_XOR, max_tuples_per_window=W) as j:
        got = j.lazy_execute_batch(left, right, descs)
    for g, w in zip(got, want):
        assert (g["count"], g["xor"], g["prod"]) == (w["count"], w["xor"], w["prod"])
    # the reference's own count for one window (restated CPU_HJ)
    assert got[0]["count"] == oracle.lazy_hj_count(left[:W], right[:W], 65536, 8192, 4)


@pytest.mark.parametrize("z", [0.5, 1.0, 1.5])
@pytest.mark.parametrize("part", ["radix", "learned"])
def test_golden_zipf_counts(lib, golden, z, part):
    tag = f"zipf_small_z{str(z).replace('.', 'p')}"
    fx, meta = load_fixture(tag), golden[tag]
    W = meta["W"]
    p = lib.PART_RADIX if part == "radix" else lib.PART_LEARNED
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=p, max_tuples_per_window=W) as j:
        res = j.lazy_execute_batch(fx["left"], fx["right"], [(w * W, W, w * W, W) for w in range(2)])
    for r, win in zip(res, meta["windows"]):
        assert r["count"] == win["count"] == win["ref_smj"]
        assert r["prod"] == win["prod"]


def test_golden_batched_uneven_windows(lib, golden):
    fx, meta = load_fixture("batched_small"), golden["batched_small"]
    descs, off = [], 0
    for n in meta["sizes"]:
        descs.append((off, n, off, n))
        off += n
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, flags=lib.F_XOR, max_tuples_per_window=1 << 12) as j:
        res = j.lazy_execute_batch(fx["left"], fx["right"], descs)
    for r, win in zip(res, meta["windows"]):
        assert (r["count"], r["xor"], r["prod"]) == (win["count"], win["xor"], win["prod"])


PARTS = {"radix": "PART_RADIX", "learned": "PART_LEARNED", "hbm_table": "PART_NONE"}


@pytest.mark.parametrize("part", ["radix", "learned", "hbm_table"])
def test_edge_cases(lib, oracle, part):
    p = getattr(lib, PARTS[part])
    cases = [
        ([], []), ([1, 2, 3], []), ([], [4]), ([5], [5]),
        ([7] * 3000, [7] * 2000),                                  # one hot key
        ([0xFFFFFFFF, 0, 0xFFFFFFFF, 9], [0xFFFFFFFF, 9, 9]),      # the all-ones key
        (list(range(10000)), list(range(5000, 15000))),            # half overlap
        ([3] * 5000 + list(range(100, 9000)), [3] * 3000 + list(range(50, 7000))),  # hot key + tail
    ]
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, lib.RESULT_ATOMIC, partitioner=p, max_tuples_per_window=1 << 16) as j:
        for kl, kr in cases:
            l, r = make_tuples(kl), make_tuples(kr, first=len(kl))
            want = oracle.join(l, r, enumerate_pairs=True, pairs_capacity=1 << 24)
            pairs = np.zeros(max(want["count"], 1), lib.PAIR_DTYPE)
            got = j.lazy_execute(l, r, pairs=pairs)
            assert got["count"] == want["count"], (kl[:5], kr[:5])
            assert got["xor"] == want["xor"] and got["prod"] == want["prod"]
            assert np.array_equal(sorted_pairs(pairs[:got["n_pairs"]]), sorted_pairs(want["pairs"]))


@pytest.mark.parametrize("part", ["radix", "learned", "hbm_table"])
def test_edge_cases_count_mode(lib, oracle, part):
    """The same edge cases through the count-only kernels (no pairs, no xor):
    the HBM table's all-ones key lives in its extra slot, a hot key is
    installed once and then added to, and a warp's equal keys are combined."""
    p = getattr(lib, PARTS[part])
    cases = [
        ([], []), ([1, 2, 3], []), ([], [4]), ([5], [5]),
        ([7] * 3000, [7] * 2000),
        ([0xFFFFFFFF, 0, 0xFFFFFFFF, 9], [0xFFFFFFFF, 9, 9]),
        ([0xFFFFFFFF] * 700 + [0] * 300, [0] * 5 + [0xFFFFFFFF] * 11),
        (list(range(10000)), list(range(5000, 15000))),
        ([3] * 5000 + list(range(100, 9000)), [3] * 3000 + list(range(50, 7000))),
    ]
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, lib.RESULT_NO_OUTPUT, partitioner=p, max_tuples_per_window=1 << 16) as j:
        for kl, kr in cases:
            l, r = make_tuples(kl), make_tuples(kr, first=len(kl))
            want = oracle.join(l, r, enumerate_pairs=False)
            got = j.lazy_execute(l, r)
            assert (got["count"], got["prod"]) == (want["count"], want["prod"]), (kl[:5], kr[:5])


def test_skewed_count_mode_overflow_passes(lib, oracle):
    """Buckets with more distinct keys than a shared table holds are joined in several passes."""
    n = 1 << 18
    rng = np.random.default_rng(1)
    l = make_tuples(rng.integers(0, 1 << 30, n))
    r = make_tuples(np.concatenate([l["key"][: n // 2], rng.integers(0, 1 << 30, n // 2)]), first=n)
    want = oracle.join(l, r, enumerate_pairs=False)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, radix_bits=2, max_tuples_per_window=n) as j:
        got = j.lazy_execute(l, r)
    assert (got["count"], got["prod"]) == (want["count"], want["prod"])


def test_pairs_truncation_and_count_kernel(lib, oracle):
    l, r = make_tuples([1] * 100), make_tuples([1] * 100)
    small = np.zeros(50, lib.PAIR_DTYPE)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, lib.RESULT_ATOMIC, max_tuples_per_window=1024) as j:
        got = j.lazy_execute(l, r, pairs=small)
    assert got["count"] == 10000 and got["n_pairs"] == 50 and got["flags"] & lib.WR_PAIRS_TRUNCATED
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, lib.RESULT_COUNT_KERNEL, max_tuples_per_window=1024) as j:
        with pytest.raises(lib.SjbgError) as e:
            j.lazy_execute(l, r, pairs=small)
        assert e.value.code == 5


def test_capacity_is_enforced(lib):
    l = make_tuples(range(100))
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, max_tuples_per_window=64) as j:
        with pytest.raises(lib.SjbgError) as e:
            j.lazy_execute(l, l)
        assert e.value.code == 5


def test_device_inputs_and_ring_api(lib, oracle):
    torch = pytest.importorskip("torch")
    W = 1 << 14
    left = oracle.gen_uniform(0, W, 1, W)
    right = oracle.gen_uniform(0, W, 2, W)
    want = oracle.join(left, right, enumerate_pairs=False)
    dl = torch.from_numpy(left.view(np.uint8)).cuda()
    dr = torch.from_numpy(right.view(np.uint8)).cuda()
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, max_tuples_per_window=W, batch_size=1024) as j:
        got = j.lazy_execute(dl, dr, mem=lib.MEM_DEVICE, n_left=W, n_right=W)
        assert (got["count"], got["prod"]) == (want["count"], want["prod"])
        # reference-style ring: batches of 1024 at scattered ring offsets
        ring_l = np.zeros(4 * W, lib.TUPLE_DTYPE)
        ring_r = np.zeros(4 * W, lib.TUPLE_DTYPE)
        offs = [(3 * i + 1) * 1024 for i in range(W // 1024)]
        for i, o in enumerate(offs):
            ring_l[o:o + 1024] = left[i * 1024:(i + 1) * 1024]
            ring_r[o:o + 1024] = right[i * 1024:(i + 1) * 1024]
        got2 = j.lazy_execute_ring(ring_l, offs, ring_r, offs)
        assert (got2["count"], got2["prod"]) == (want["count"], want["prod"])


def test_device_generator_matches_host(lib, oracle):
    torch = pytest.importorskip("torch")
    n, D = 100000, 1 << 16
    buf = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    T = oracle.zipf_table(D, 1.2)
    dT = torch.from_numpy(T.view(np.int64)).cuda()
    with lib.Joiner(lib.ALG_HJ, lib.LAZY) as j:
        j.generate(buf.data_ptr(), 12345, n, 1, D)
        got = buf.cpu().numpy().view(lib.TUPLE_DTYPE)
        assert np.array_equal(got, oracle.gen_uniform(12345, n, 1, D))
        j.generate(buf.data_ptr(), 7, n, 2, D, dT.data_ptr(), 3)
        got = buf.cpu().numpy().view(lib.TUPLE_DTYPE)
        assert np.array_equal(got, oracle.gen_zipf(7, n, 2, T, D, 3))


def test_profile_counts_kernels(lib, oracle):
    W = 4096
    left = oracle.gen_uniform(0, W, 1, W)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, flags=lib.F_PROFILE,
                    max_tuples_per_window=W) as j:
        j.lazy_execute(left, left)
        st = j.kernel_stats()
        assert {"part_hist", "part_scan", "bucket_join_count"} <= set(st)
        assert "part_scatter" in st or "part_fine" in st
        assert all(v[0] >= 1 and v[1] > 0 for v in st.values())
        assert j.launch_count() >= 4


@pytest.mark.parametrize("z", [0.8, 1.0])
def test_learned_keeps_its_model_when_many_keys_are_hot(lib, oracle, z):
    """Zipf over a wide domain has thousands of frequently sampled keys: the
    heaviest must still become heavy keys, so the model does not fall back,
    and the result equals radix partitioning and the oracle."""
    D, W = 1 << 26, 1 << 22
    table = oracle.zipf_table(D, z)
    left = oracle.gen_zipf(0, W, 1, table, D, 3)
    right = oracle.gen_zipf(0, W, 2, table, D, 3)
    want = oracle.join(left, right, enumerate_pairs=False)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=W) as j:
        got = j.lazy_execute(left, right)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, max_tuples_per_window=W) as j:
        rad = j.lazy_execute(left, right)
    assert got["partitioner_used"] == lib.PART_LEARNED and not (got["flags"] & lib.WR_FALLBACK)
    assert (got["count"], got["prod"]) == (want["count"], want["prod"]) == (rad["count"], rad["prod"])


@pytest.mark.parametrize("z", [1.5, 1.0, 0.5])
def test_config_skewed_8x2p24_full_size(lib, oracle, z):
    """The skewed workload at its full size: 8 windows of 2^24 tuples per stream,
    keys Zipf(z) over [0, 2^24) with ranks permuted (seed 3), R seed 1, S seed 2.
    In every window, learned partitioning, radix partitioning at 2^10, and the
    learned pipeline with a one-leaf model (light tuples bucketed by one line
    over their key range, i.e. radix by key range behind the same heavy-key
    set and compaction) all equal the oracle's count and prod."""
    D, W, nw = 1 << 24, 1 << 24, 8
    table = oracle.zipf_table(D, z)
    left = oracle.gen_zipf(0, nw * W, 1, table, D, 3, threads=16)
    right = oracle.gen_zipf(0, nw * W, 2, table, D, 3, threads=16)
    descs = [(w * W, W, w * W, W, 0, 0) for w in range(nw)]
    want, _ = oracle.join_windows(left, right, descs, enumerate_pairs=False, threads=16)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=W) as j:
        got = j.lazy_execute_batch(left, right, descs)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, radix_bits=10,
                    max_tuples_per_window=W) as j:
        rad = j.lazy_execute_batch(left, right, descs)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, learned_leaves=1,
                    max_tuples_per_window=W) as j:
        one = j.lazy_execute_batch(left, right, descs)
    for i, (g, r, o, w) in enumerate(zip(got, rad, one, want)):
        assert (g["count"], g["prod"]) == (w["count"], w["prod"]) == (r["count"], r["prod"]) == \
            (o["count"], o["prod"]), i
    if z == 1.5:
        assert all(g["partitioner_used"] == lib.PART_LEARNED for g in got)


def test_learned_keeps_its_model_on_streaming_keys(lib, oracle):
    """The streaming workload's keys: Zipf z = 1.2 over 2^26 with ranks permuted
    (seed 3).  The heavy set must place the heaviest keys, so that none is left
    in a light partition it would overflow, and the model does not fall back to
    radix partitioning; the result equals the oracle."""
    D, W = 1 << 26, 1 << 23
    table = oracle.zipf_table(D, 1.2)
    left = oracle.gen_zipf(0, W, 1, table, D, 3, threads=16)
    right = oracle.gen_zipf(0, W, 2, table, D, 3, threads=16)
    want = oracle.join(left, right, enumerate_pairs=False)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=W) as j:
        got = j.lazy_execute(left, right)
    assert got["partitioner_used"] == lib.PART_LEARNED and not (got["flags"] & lib.WR_FALLBACK)
    assert (got["count"], got["prod"]) == (want["count"], want["prod"])


def test_learned_keeps_radix_when_it_is_cheaper(lib, oracle):
    """Zipf z = 0.5 over 2^24 keys: heavy keys hold well under a tenth of the
    sample and radix buckets it evenly, so the learned partitioner keeps radix
    partitioning (flagged, not a fallback) and the result equals the oracle."""
    D, W = 1 << 24, 1 << 22
    table = oracle.zipf_table(D, 0.5)
    left = oracle.gen_zipf(0, W, 1, table, D, 3)
    right = oracle.gen_zipf(0, W, 2, table, D, 3)
    want = oracle.join(left, right, enumerate_pairs=False)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=W) as j:
        got = j.lazy_execute(left, right)
    assert got["partitioner_used"] == lib.PART_RADIX
    assert got["flags"] & lib.WR_RADIX_BY_COST and not (got["flags"] & lib.WR_FALLBACK)
    assert (got["count"], got["prod"]) == (want["count"], want["prod"])


def test_learned_heavy_keys_sharing_a_set_bucket(lib, oracle):
    """The heavy-key set has 2,048 buckets of two slots (bucket = top 11 bits of
    key * 0x9E3779B97F4A7C15).  Four heavy keys of one bucket: the two heaviest
    take its slots, the other two find it full and stay light, and are joined
    through the partitions; the result still equals the oracle and radix."""
    C, M = 0x9E3779B97F4A7C15, (1 << 64) - 1
    by_bucket = {}
    for k in range(1, 1 << 20):
        group = by_bucket.setdefault(((k * C) & M) >> 53, [])
        group.append(k)
        if len(group) == 4:
            break
    hot = group                                           # four keys of one bucket
    mult = [300_000, 250_000, 6_000, 5_000]               # heaviest first
    rng = np.random.default_rng(11)
    sides = []
    for side in range(2):
        keys = np.concatenate([np.full(m, k, np.uint32) for k, m in zip(hot, mult)] +
                              [rng.integers(1 << 24, (1 << 24) + (1 << 22), 1_000_000, dtype=np.uint32)])
        rng.shuffle(keys)
        sides.append(make_tuples(keys, first=side << 28))
    left, right = sides
    want = oracle.join(left, right, enumerate_pairs=False)
    n = len(left)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=n) as j:
        got = j.lazy_execute(left, right)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, max_tuples_per_window=n) as j:
        rad = j.lazy_execute(left, right)
    assert got["partitioner_used"] == lib.PART_LEARNED and not (got["flags"] & lib.WR_FALLBACK)
    assert (got["count"], got["prod"]) == (want["count"], want["prod"]) == (rad["count"], rad["prod"])


def test_learned_batch_mixes_every_kind_of_window(lib, oracle):
    """One call whose windows take every route of the later passes, which visit
    only the tiles and buckets listed for them: a compacted z = 1.5 window, a
    uniform 2^23 window (two-level: coarse runs, then the fine pass), a z = 1.0
    window, a tiny window and one with an empty side.  Each equals the oracle
    and radix partitioning."""
    D = 1 << 24
    t15, t10 = oracle.zipf_table(D, 1.5), oracle.zipf_table(D, 1.0)
    spec = [("z15", 1 << 20, 1 << 20), ("uni", 1 << 23, 1 << 23), ("z10", 1 << 21, 1 << 21),
            ("uni", 1000, 900), ("uni", 5000, 0)]
    lefts, rights, descs, lo, ro = [], [], [], 0, 0
    for kind, nl, nr in spec:
        if kind == "uni":
            l, r = oracle.gen_uniform(lo, nl, 1, D), oracle.gen_uniform(ro, nr, 2, D)
        else:
            tab = t15 if kind == "z15" else t10
            l, r = oracle.gen_zipf(lo, nl, 1, tab, D, 3), oracle.gen_zipf(ro, nr, 2, tab, D, 3)
        lefts.append(l)
        rights.append(r)
        descs.append((lo, nl, ro, nr, 0, 0))
        lo += nl
        ro += nr
    left, right = np.concatenate(lefts), np.concatenate(rights)
    want, _ = oracle.join_windows(left, right, descs, enumerate_pairs=False)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=1 << 23) as j:
        got = j.lazy_execute_batch(left, right, descs)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_RADIX, max_tuples_per_window=1 << 23) as j:
        rad = j.lazy_execute_batch(left, right, descs)
    for g, r, w in zip(got, rad, want):
        assert (g["count"], g["prod"]) == (w["count"], w["prod"]) == (r["count"], r["prod"])


def test_learned_compacts_light_tuples_of_heavy_windows(lib, oracle):
    """At z = 1.5 most tuples carry a heavy key: the counting pass compacts the
    light ones and only those are partitioned; several windows of different
    sizes in one call, each equal to the oracle."""
    D = 1 << 24
    table = oracle.zipf_table(D, 1.5)
    sizes = [1 << 20, 3 << 18, 1 << 16, 5000]
    lefts, rights, descs, off = [], [], [], 0
    for n in sizes:
        lefts.append(oracle.gen_zipf(off, n, 1, table, D, 3))
        rights.append(oracle.gen_zipf(off, n, 2, table, D, 3))
        descs.append((off, n, off, n, 0, 0))
        off += n
    left, right = np.concatenate(lefts), np.concatenate(rights)
    want, _ = oracle.join_windows(left, right, descs, enumerate_pairs=False)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=1 << 20) as j:
        got = j.lazy_execute_batch(left, right, descs)
    for g, w in zip(got, want):
        assert (g["count"], g["prod"]) == (w["count"], w["prod"])
    assert got[0]["partitioner_used"] == lib.PART_LEARNED


@pytest.mark.parametrize("enum", [False, True])
def test_hbm_table_join_matches_oracle(lib, oracle, enum):
    """The unpartitioned join (one open-addressing table per window in HBM):
    uneven windows (including empty and single-tuple sides), uniform and Zipf
    keys; counts, checksums and, when enumerating, the pairs."""
    D = 1 << 16
    table = oracle.zipf_table(D, 1.2)
    sizes = [1 << 16, 70000, 1, 0, 4097]
    lefts, rights, descs, off = [], [], [], 0
    for i, n in enumerate(sizes):
        m = n + 3   # right sides are 3 tuples longer; left sides use the first n
        if i % 2:
            lefts.append(oracle.gen_zipf(off, m, 1, table, D, 3))
            rights.append(oracle.gen_zipf(off, m, 2, table, D, 3))
        else:
            lefts.append(oracle.gen_uniform(off, m, 1, D))
            rights.append(oracle.gen_uniform(off, m, 2, D))
        descs.append((off, n, off, m))
        off += m
    left, right = np.concatenate(lefts), np.concatenate(rights)
    want = [oracle.join(left[d[0]:d[0] + d[1]], right[d[2]:d[2] + d[3]], enumerate_pairs=enum,
                        pairs_capacity=1 << 22) for d in descs]
    # pairs are written and compared for the windows with at most 2^22 of them
    caps = [int(w["count"]) if w["count"] <= (1 << 22) else 0 for w in want]
    pdescs = [d + (sum(caps[:i]), caps[i] if enum else 0) for i, d in enumerate(descs)]
    pairs = np.zeros(max(sum(caps), 1), lib.PAIR_DTYPE) if enum else None
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, lib.RESULT_ATOMIC if enum else lib.RESULT_NO_OUTPUT,
                    partitioner=lib.PART_NONE, flags=lib.F_XOR if enum else 0, max_tuples_per_window=1 << 17) as j:
        got = j.lazy_execute_batch(left, right, pdescs, pairs=pairs)
    for i, (g, w) in enumerate(zip(got, want)):
        assert (g["count"], g["prod"]) == (w["count"], w["prod"]), i
        assert g["partitioner_used"] == lib.PART_NONE
        if enum:
            assert g["xor"] == w["xor"], i
        if enum and caps[i]:
            got_pairs = pairs[pdescs[i][4]:pdescs[i][4] + g["n_pairs"]]
            assert np.array_equal(sorted_pairs(got_pairs), sorted_pairs(w["pairs"])), i


def test_auto_partitioner_by_window_size(lib, oracle):
    """SJBG_PART_AUTO: windows whose tables stay in L2 get one HBM table per
    window, larger windows radix partitioning; both equal the oracle."""
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, max_tuples_per_window=1 << 20) as j:
        for W, part in ((1 << 14, lib.PART_NONE), (1 << 20, lib.PART_RADIX)):
            left = oracle.gen_uniform(0, W, 1, W)
            right = oracle.gen_uniform(0, W, 2, W)
            want = oracle.join(left, right, enumerate_pairs=False)
            got = j.lazy_execute(left, right)
            assert got["partitioner_used"] == part
            assert (got["count"], got["prod"]) == (want["count"], want["prod"])
