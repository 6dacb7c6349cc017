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
