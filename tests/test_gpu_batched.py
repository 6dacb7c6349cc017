"""GPU tests of batched uneven windows: many windows of log-uniform sizes in
one call, with the autotuner, CUDA-graph capture and replay, and the hash and
sort-merge joins checked against the oracle window by window."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def uneven_windows(oracle, n_windows, lo, hi, seed=4):
    sizes = [oracle.log_uniform(seed, w, lo, hi) for w in range(n_windows)]
    lefts, rights, descs, off = [], [], [], 0
    for w, n in enumerate(sizes):
        lefts.append(oracle.gen_uniform(off, n, 1, 4 * n))
        rights.append(oracle.gen_uniform(off, n, 2, 4 * n))
        descs.append((off, n, off, n, 0, 0))
        off += n
    return np.concatenate(lefts), np.concatenate(rights), descs


@pytest.mark.parametrize("algo", ["HJ", "SMJ"])
def test_batched_graph_replay_matches_oracle(lib, oracle, tmp_path, algo):
    torch = pytest.importorskip("torch")
    os.environ["SJBG_TUNE_CACHE"] = str(tmp_path / "tune.json")
    left, right, descs = uneven_windows(oracle, 256, 1 << 10, 1 << 17)
    want, _ = oracle.join_windows(left, right, descs, enumerate_pairs=True)
    dl = torch.from_numpy(left.view(np.uint8)).cuda()
    dr = torch.from_numpy(right.view(np.uint8)).cuda()
    a = lib.ALG_HJ if algo == "HJ" else lib.ALG_SMJ
    flags = lib.F_XOR | lib.F_GRAPH | (lib.F_AUTOTUNE if algo == "HJ" else 0)
    with lib.Joiner(a, lib.LAZY, flags=flags, max_tuples_per_window=1 << 17) as j:
        first = j.lazy_execute_batch(dl, dr, descs, mem=lib.MEM_DEVICE)     # tunes, runs, captures
        again = j.lazy_execute_batch(dl, dr, descs, mem=lib.MEM_DEVICE)     # replays the graph
    for g1, g2, w in zip(first, again, want):
        assert (g1["count"], g1["xor"], g1["prod"]) == (w["count"], w["xor"], w["prod"])
        assert (g2["count"], g2["xor"], g2["prod"]) == (w["count"], w["xor"], w["prod"])
    if algo == "HJ":
        text = (tmp_path / "tune.json").read_text()
        assert '"bucket_target"' in text and '"persistent"' in text


def test_learned_graph_replay_reruns_every_kernel(lib, oracle):
    """Learned partitioning under graph replay (the bench's throughput arms):
    every replay re-samples and re-fits on the device and equals the first run
    and the oracle; each replay counts its kernels again."""
    torch = pytest.importorskip("torch")
    D, W = 1 << 24, 1 << 20
    table = oracle.zipf_table(D, 1.5)
    left = np.concatenate([oracle.gen_zipf(w * W, W, 1, table, D, 3) for w in range(3)])
    right = np.concatenate([oracle.gen_zipf(w * W, W, 2, table, D, 3) for w in range(3)])
    descs = [(w * W, W, w * W, W, 0, 0) for w in range(3)]
    want, _ = oracle.join_windows(left, right, descs, enumerate_pairs=False)
    dl = torch.from_numpy(left.view(np.uint8)).cuda()
    dr = torch.from_numpy(right.view(np.uint8)).cuda()
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, flags=lib.F_GRAPH,
                    max_tuples_per_window=W) as j:
        runs, counts = [], []
        for _ in range(3):   # run + capture, then two replays
            runs.append(j.lazy_execute_batch(dl, dr, descs, mem=lib.MEM_DEVICE))
            counts.append(j.launch_count())
    for run in runs:
        for g, w in zip(run, want):
            assert (g["count"], g["prod"]) == (w["count"], w["prod"])
            assert g["partitioner_used"] == lib.PART_LEARNED
    per_replay = counts[2] - counts[1]
    assert per_replay >= 10 and counts[1] - counts[0] == per_replay


@pytest.fixture(scope="module")
def batched_1024(lib, oracle):
    """The 1,024-window shape (sizes log-uniform in [2^10, 2^20] per stream,
    seed 4; keys in [0, 4W)), generated on the device, and the oracle's count,
    xor checksum and prod of every window (about W/4 pairs per window, all
    enumerated)."""
    torch = pytest.importorskip("torch")
    sizes = [oracle.log_uniform(4, w, 1 << 10, 1 << 20) for w in range(1024)]
    total = sum(sizes)
    dl = torch.empty(total * 16, dtype=torch.uint8, device="cuda")
    dr = torch.empty(total * 16, dtype=torch.uint8, device="cuda")
    descs, off = [], 0
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, max_tuples_per_window=1 << 20) as g:
        for n in sizes:
            g.generate(dl.data_ptr() + 16 * off, off, n, 1, 4 * n)
            g.generate(dr.data_ptr() + 16 * off, off, n, 2, 4 * n)
            descs.append((off, n, off, n, 0, 0))
            off += n
    torch.cuda.synchronize()
    hl = dl.cpu().numpy().view(lib.TUPLE_DTYPE)
    hr = dr.cpu().numpy().view(lib.TUPLE_DTYPE)
    want, _ = oracle.join_windows(hl, hr, descs, enumerate_pairs=True, threads=os.cpu_count() or 8)
    return dl, dr, descs, want


@pytest.mark.parametrize("algo", ["HJ", "SMJ"])
def test_batched_1024_windows_match_oracle(lib, batched_1024, algo):
    """Every one of the 1,024 windows, first run and CUDA-graph replay: count,
    xor checksum (every pair enumerated) and prod equal the oracle's."""
    dl, dr, descs, want = batched_1024
    a = lib.ALG_HJ if algo == "HJ" else lib.ALG_SMJ
    with lib.Joiner(a, lib.LAZY, flags=lib.F_XOR | lib.F_GRAPH, max_tuples_per_window=1 << 20) as j:
        first = j.lazy_execute_batch(dl, dr, descs, mem=lib.MEM_DEVICE)
        again = j.lazy_execute_batch(dl, dr, descs, mem=lib.MEM_DEVICE)
    exp = [(w["count"], w["xor"], w["prod"]) for w in want]
    assert [(g["count"], g["xor"], g["prod"]) for g in first] == exp
    assert [(g["count"], g["xor"], g["prod"]) for g in again] == exp
    assert all(g["status"] == 0 for g in first)
    assert sum(w["count"] for w in want) > 1024 * 256   # about W/4 pairs per window


def test_batched_1024_windows_count_only_paths(lib, batched_1024):
    """Without pair enumeration (count and prod only) the automatic hash join,
    radix partitioning, learned partitioning and the sort-merge join all equal
    the oracle on every window."""
    dl, dr, descs, want = batched_1024
    exp = [(w["count"], w["prod"]) for w in want]
    for a, part in ((lib.ALG_HJ, lib.PART_AUTO), (lib.ALG_HJ, lib.PART_RADIX), (lib.ALG_HJ, lib.PART_LEARNED),
                    (lib.ALG_SMJ, lib.PART_AUTO)):
        with lib.Joiner(a, lib.LAZY, partitioner=part, max_tuples_per_window=1 << 20) as j:
            got = j.lazy_execute_batch(dl, dr, descs, mem=lib.MEM_DEVICE)
        assert [(g["count"], g["prod"]) for g in got] == exp, (a, part)
