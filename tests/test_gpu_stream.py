"""GPU tests of the event-time streaming loop: Poisson batches of two streams,
tumbling event-time windows, Zipf keys with a drifting exponent, learned
partitioning refitted per window; every window's result equals the oracle's
join of that window's tuples."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def poisson_stream(oracle, seed, n_batches, batch, mean_gap_ns, domain, z_of_time, perm_seed=3):
    """Tuples of one stream: batch k arrives at a Poisson time; its tuples share that ts."""
    rng = np.random.default_rng(seed)
    times = np.cumsum(rng.exponential(mean_gap_ns, n_batches)).astype(np.uint64)
    out = np.empty(n_batches * batch, oracle.TUPLE_DTYPE)
    tables = {}
    for k in range(n_batches):
        z = z_of_time(int(times[k]))
        if z not in tables:
            tables[z] = oracle.zipf_table(domain, z)
        t = oracle.gen_zipf(k * batch, batch, seed, tables[z], domain, perm_seed)
        t["ts"] = times[k]
        out[k * batch:(k + 1) * batch] = t
    return out


def interleave_pushes(left, right, chunk):
    """Push order by event time, chunk tuples at a time per side."""
    i = j = 0
    while i < len(left) or j < len(right):
        if j >= len(right) or (i < len(left) and left[i]["ts"] <= right[j]["ts"]):
            yield True, left[i:i + chunk]
            i += chunk
        else:
            yield False, right[j:j + chunk]
            j += chunk


def test_stream_windows_match_oracle(lib, oracle):
    W_NS = 1_000_000                     # 1 ms windows
    drift = lambda t: 0.8 if t < 8 * W_NS else (1.2 if t < 16 * W_NS else 1.5)
    left = poisson_stream(oracle, 1, 600, 256, 40_000.0, 1 << 16, drift)
    right = poisson_stream(oracle, 2, 600, 256, 40_000.0, 1 << 16, drift)
    results = []
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=1 << 22) as j:
        j.stream_open(W_NS)
        for is_left, chunk in interleave_pushes(left, right, 1000):
            j.stream_push(chunk, is_left)
            results += j.stream_poll()
        stats = j.stream_close()
        results += j.stream_poll()
    by_id = {r["window_id"]: r for r in results}
    wl, wr = left["ts"] // W_NS, right["ts"] // W_NS
    ids = sorted(set(wl.tolist()) | set(wr.tolist()))
    assert stats["windows_closed"] == len(ids) and stats["windows_rejected"] == 0
    assert stats["tuples_joined"] == len(left) + len(right)
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    for wid in ids:
        want = oracle.join(left[wl == wid], right[wr == wid], enumerate_pairs=False)
        got = by_id[wid]
        assert got["status"] == 0
        assert (got["count"], got["prod"]) == (want["count"], want["prod"]), wid


def test_stream_budget_rejects_windows(lib, oracle):
    W_NS = 1_000_000
    left = poisson_stream(oracle, 1, 200, 256, 40_000.0, 1 << 16, lambda t: 1.0)
    right = poisson_stream(oracle, 2, 200, 256, 40_000.0, 1 << 16, lambda t: 1.0)
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, max_tuples_per_window=1 << 22, hbm_budget_bytes=1 << 20) as j:
        j.stream_open(W_NS)
        for is_left, chunk in interleave_pushes(left, right, 1000):
            j.stream_push(chunk, is_left)
        stats = j.stream_close()
        res = j.stream_poll(4096)
    # a 1 MiB budget cannot hold the 1M-tuple minimum buffer of any window
    assert stats["windows_rejected"] == stats["windows_closed"] > 0
    assert all(r["status"] == 7 for r in res)


def test_stream_requires_ordered_event_time(lib):
    t = np.zeros(4, lib.TUPLE_DTYPE)
    t["ts"] = [5, 6, 7, 8]
    with lib.Joiner(lib.ALG_HJ, lib.LAZY) as j:
        j.stream_open(1000)
        j.stream_push(t, True)
        back = t.copy()
        back["ts"] = [1, 2, 3, 4]
        with pytest.raises(lib.SjbgError):
            j.stream_push(back, True)


def test_stream_full_scale_windows_match_oracle(lib, oracle):
    """The streaming workload at full scale: two streams at 1 G tuples/s
    together (Poisson batches of 4,096 per stream), 100 ms event-time windows
    (about 10^8 tuples each), keys Zipf over [0, 2^26) ranked through the
    seeded permutation, the exponent stepping 0.8 -> 1.2 -> 1.5 (two windows
    each here; the workload steps every 10 s), learned partitioning refitted
    on every window, 120 GB budget.  Generated on the device, pushed in event
    time order, copied back; every window's count and prod equal the
    oracle's join of that window's tuples."""
    import os

    torch = pytest.importorskip("torch")
    D, B, W_NS, n_win = 1 << 26, 4096, 100_000_000, 6
    zs = [0.8, 0.8, 1.2, 1.2, 1.5, 1.5]
    gap_ns = B / 0.5e9 * 1e9          # 0.5 G tuples/s per stream
    rng = np.random.default_rng(17)
    tables = {z: torch.from_numpy(lib.zipf_table(D, z).view(np.int64)).cuda() for z in set(zs)}
    bufs, times = [], []
    with lib.Joiner(lib.ALG_HJ, lib.LAZY, partitioner=lib.PART_LEARNED, max_tuples_per_window=1 << 30,
                    hbm_budget_bytes=120 << 30) as j:
        for side in (0, 1):
            t = np.cumsum(rng.exponential(gap_ns, int(1.1 * n_win * W_NS / gap_ns)))
            t = t[t < n_win * W_NS].astype(np.int64)
            buf = torch.empty(len(t) * B * 16, dtype=torch.uint8, device="cuda")
            wid = t // W_NS
            for k in range(n_win):   # each window's batches, with that window's exponent
                a, b = int(np.searchsorted(wid, k)), int(np.searchsorted(wid, k + 1))
                j.generate(buf.data_ptr() + 16 * a * B, a * B, (b - a) * B, 1 + side, D,
                           tables[zs[k]].data_ptr(), 3)
            buf.view(torch.int64).view(-1, 2)[:, 1] = torch.from_numpy(t).cuda().repeat_interleave(B)
            bufs.append(buf)
            times.append(t)
        torch.cuda.synchronize()
        j.stream_open(W_NS)
        results, nxt, step = [], [0, 0], 256   # 256 batches (1 Mi tuples) per push
        while nxt[0] < len(times[0]) or nxt[1] < len(times[1]):
            side = 0 if nxt[1] >= len(times[1]) or (nxt[0] < len(times[0]) and
                                                    times[0][nxt[0]] <= times[1][nxt[1]]) else 1
            a = int(nxt[side])
            b = int(min(a + step, len(times[side])))
            j.stream_push(bufs[side].data_ptr() + 16 * a * B, side == 0, mem=lib.MEM_DEVICE, n=(b - a) * B)
            nxt[side] = b
            results += j.stream_poll()
        stats = j.stream_close()
        results += j.stream_poll()
    assert stats["windows_closed"] == n_win and stats["windows_rejected"] == 0
    hl = bufs[0].cpu().numpy().view(lib.TUPLE_DTYPE)
    hr = bufs[1].cpu().numpy().view(lib.TUPLE_DTYPE)
    del bufs
    descs = []
    for k in range(n_win):
        la, lb = np.searchsorted(times[0] // W_NS, [k, k + 1]) * B
        ra, rb = np.searchsorted(times[1] // W_NS, [k, k + 1]) * B
        descs.append((int(la), int(lb - la), int(ra), int(rb - ra), 0, 0))
    want, _ = oracle.join_windows(hl, hr, descs, enumerate_pairs=False, threads=min(n_win, os.cpu_count() or 1))
    by_id = {r["window_id"]: r for r in results}
    for k in range(n_win):
        got = by_id[k]
        assert got["status"] == 0
        assert (got["n_left"], got["n_right"]) == (descs[k][1], descs[k][3])
        assert (got["count"], got["prod"]) == (want[k]["count"], want[k]["prod"]), k
        assert descs[k][1] + descs[k][3] > 9 * 10 ** 7   # about 10^8 tuples per window
