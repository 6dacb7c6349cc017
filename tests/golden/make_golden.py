"""Generate the golden fixtures under tests/golden/ (run where the reference
sources are mounted; needs only the CPU).

Counts come from the reference's OWN CPU joiners (lazy CPU_HJ, CPU_SMJ,
CPU_NLJ and eager CPU_HJ, compiled from their sources by ``make -C oracle ref``
against the oracle's TBB-API shim).  Checksums and sorted pair lists, which no
reference code produces, come from the oracle's result restatement and are
cross-checked here against the reference counts.  Input keys are stored too
(val = ts = tuple index, so keys determine the tuples), so a test can also
confirm that the generator reproduces them bit for bit on another machine.

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle_py as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def check(a, b, what):
    if a != b:
        raise SystemExit(f"reference and restatement disagree on {what}: {a} != {b}")


def lazy_windows(name, left, right, W, dk, batch, algos, pairs_for=(0,)):
    nwin = len(left) // W
    rec = {"W": W, "distinct_keys": dk, "batch": batch, "windows": []}
    pairs = {}
    for w in range(nwin):
        l, r = left[w * W:(w + 1) * W], right[w * W:(w + 1) * W]
        j = O.join(l, r, enumerate_pairs=True)
        win = {"count": int(j["count"]), "xor": int(j["xor"]), "prod": int(j["prod"])}
        if "hj" in algos:
            win["ref_hj"] = O.ref_lazy_hj_count(l, r, dk, batch, 4)
            check(win["ref_hj"], win["count"], f"{name} w{w} CPU_HJ")
        if "smj" in algos:
            win["ref_smj"] = O.ref_lazy_smj_count(l, r, dk, batch, 4)
            check(win["ref_smj"], win["count"], f"{name} w{w} CPU_SMJ")
        if "nlj" in algos:
            win["ref_nlj"] = O.ref_lazy_nlj_count(l, r, batch)
            check(win["ref_nlj"], win["count"], f"{name} w{w} CPU_NLJ")
        rec["windows"].append(win)
        if w in pairs_for:
            pairs[f"pairs_w{w}"] = np.stack([j["pairs"]["r"], j["pairs"]["s"]], axis=1).astype(np.uint32)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), left_keys=left["key"], right_keys=right["key"], **pairs)
    return rec


def main():
    if O.ref_lib() is None:
        raise SystemExit("the reference sources are needed to make the fixtures")
    meta = {}

    # 1. lazy hash join, the shape of the 16 x 65,536 uniform workload reduced to 4 x 4,096.
    W, dk = 4096, 4096
    L = O.gen_uniform(0, 4 * W, 1, dk)
    R = O.gen_uniform(0, 4 * W, 2, dk)
    meta["lazy_uniform_small"] = lazy_windows("lazy_uniform_small", L, R, W, dk, 1024, ("hj", "smj"), (0, 1))

    # 2. nested-loop shape: 2 windows x 2,048, keys in [0, 2,048).
    W, dk = 2048, 2048
    L = O.gen_uniform(0, 2 * W, 1, dk)
    R = O.gen_uniform(0, 2 * W, 2, dk)
    meta["nlj_small"] = lazy_windows("nlj_small", L, R, W, dk, 512, ("nlj", "hj"), (0,))

    # 3. skewed shape: Zipf z in {0.5, 1.0, 1.5} over [0, 2^16), 2 windows x 2^15, permutation seed 3.
    D, W = 1 << 16, 1 << 15
    for z in (0.5, 1.0, 1.5):
        T = O.zipf_table(D, z)
        L = O.gen_zipf(0, 2 * W, 1, T, D, 3)
        R = O.gen_zipf(0, 2 * W, 2, T, D, 3)
        tag = f"zipf_small_z{str(z).replace('.', 'p')}"
        meta[tag] = lazy_windows(tag, L, R, W, D, 4096, ("smj",), ())
        meta[tag]["z"] = z
        meta[tag]["table_xor"] = int(np.bitwise_xor.reduce(T))

    # 4. eager shape: batches of 256, window 2,048, keys in [0, 1,024), 24 batches per side.
    B, W, dk, nb = 256, 2048, 1024, 24
    L = O.gen_uniform(0, nb * B, 1, dk)
    R = O.gen_uniform(0, nb * B, 2, dk)
    bc, wc = O.ref_eager_hj(L, R, B, W, dk)
    bc2, wc2 = O.eager_hj(L, R, B, W, dk)
    check(bc.tolist(), bc2.tolist(), "eager batch counts")
    np.savez_compressed(os.path.join(OUT, "eager_small.npz"), left_keys=L["key"], right_keys=R["key"],
                        batch_counts=bc, window_counts=wc)
    meta["eager_small"] = {"batch": B, "W": W, "distinct_keys": dk, "n_batches": nb,
                           "window_counts": [int(x) for x in wc]}

    # 5. batched uneven windows: 24 windows, sizes log-uniform in [2^6, 2^12] (seed 4), keys in [0, 4W).
    sizes = [O.log_uniform(4, w, 1 << 6, 1 << 12) for w in range(24)]
    lefts, rights, descs, off = [], [], [], 0
    for w, n in enumerate(sizes):
        lefts.append(O.gen_uniform(off, n, 1, 4 * n))
        rights.append(O.gen_uniform(off, n, 2, 4 * n))
        descs.append((off, n, off, n, 0, 0))
        off += n
    L, R = np.concatenate(lefts), np.concatenate(rights)
    res, _ = O.join_windows(L, R, descs, enumerate_pairs=True)
    wins = []
    for w, (d, r) in enumerate(zip(descs, res)):
        l, rr = L[d[0]:d[0] + d[1]], R[d[2]:d[2] + d[3]]
        ref = O.ref_lazy_hj_count(l, rr, 4 * d[1], d[1], 1)
        check(ref, r["count"], f"batched w{w}")
        wins.append({"n": d[1], "count": r["count"], "xor": r["xor"], "prod": r["prod"], "ref_hj": ref})
    np.savez_compressed(os.path.join(OUT, "batched_small.npz"), left_keys=L["key"], right_keys=R["key"])
    meta["batched_small"] = {"sizes": sizes, "windows": wins}

    # 6. generator pins: first tuples of each stream kind at a large index offset.
    meta["generator"] = {
        "uniform_seed1_dom65536_at1e9": [int(x) for x in O.gen_uniform(10 ** 9, 8, 1, 65536)["key"]],
        "perm_2p24_seed3": [O.perm(k, 1 << 24, 3) for k in range(8)],
        "perm_1000_seed7": [O.perm(k, 1000, 7) for k in range(8)],
        "log_uniform_seed4": [O.log_uniform(4, w, 1 << 10, 1 << 20) for w in range(8)],
        "pair_hash": [O.pair_hash(1, 2), O.pair_hash(0xFFFFFFFF, 0)],
    }

    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
