"""GPU tests of the C++ host harness end to end: runExperiment generates both
streams, feeds them batch by batch through the reference's windowing
(lazy ring buffer / eager close rule) into the GPU joiners, and its match count,
product checksum and per-batch progress equal the oracle's on the same
streams."""
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 18            # tuples per stream
W = 1 << 16            # windowSizesMB: [1]
B = 1 << 13            # batchSizeKB: [128]
DISTINCT = 1000


def run(harness, tmp_path, alg, prog, result="NoOutput", theta="0.0", distinct=DISTINCT, power="No", extra=""):
    y = tmp_path / "exp.yaml"
    y.write_text(
        f'algTypes: [ "{alg}" ]\ndeviceTypes: [ "GPU" ]\nprogressivenessModes: [ "{prog}" ]\n'
        f"distinctKeys: [ {distinct} ]\nzipfThetas: [ {theta} ]\nresultMaterializationMethod: [ \"{result}\" ]\n"
        f'windowSizesMB: [ 1 ]\nbatchSizeKB: [ 128 ]\nmeasuredMetric: "cumulativePercentage"\n'
        f'measurePowerUsage: "{power}"\nrepeat: 1\nparStrats: [ "INTRA" ]\ndataSize: {N}\n'
        + (extra if "sourceThreads" in extra else extra + "sourceThreads: 1\n"))
    r = subprocess.run([harness, str(y), str(tmp_path / "out.csv")], capture_output=True, text=True,
                       cwd=tmp_path, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    run.last = r
    m = re.search(r"Match Count: (\d+)", r.stdout)
    p = re.search(r"Prod checksum: (\d+)", r.stdout)
    w = re.search(r"Windows: (\d+)", r.stdout)
    run.window_pairs = int(re.search(r"Window pairs: (\d+)", r.stdout).group(1))
    rows = (tmp_path / "progressiveness.csv").read_text().strip().splitlines()[1:]
    progress = [int(row.split(",")[4]) for row in rows]
    return int(m.group(1)), int(p.group(1)), int(w.group(1)), progress


def streams(oracle, theta=0.0, distinct=DISTINCT):
    """The harness's streams: seeds 123 / 456, val = key, STEADY timestamps."""
    out = []
    for seed in (123, 456):
        if theta > 0:
            t = oracle.gen_zipf(0, N, seed, oracle.zipf_table(distinct, float(np.float32(theta))), distinct, 3)
        else:
            t = oracle.gen_uniform(0, N, seed, distinct)
        t["val"] = t["key"]
        t["ts"] = np.floor(np.arange(N) / np.floor(N / 1000)).astype(np.uint64)
        out.append(t)
    return out


@pytest.mark.parametrize("alg,result", [("HJ", "NoOutput"), ("HJ", "Atomic"), ("SMJ", "NoOutput"),
                                        ("NLJ", "CountKernel")])
def test_lazy_harness_matches_oracle(harness, oracle, tmp_path, alg, result):
    left, right = streams(oracle)
    count, prod, windows, progress = run(harness, tmp_path, alg, "LAZY", result)
    want_c = want_p = 0
    cum = []
    for k in range(N // W):
        r = oracle.join(left[k * W:(k + 1) * W], right[k * W:(k + 1) * W], enumerate_pairs=False)
        want_c += r["count"]
        want_p = (want_p + r["prod"]) % (1 << 64)
        cum.append(want_c)
    assert windows == N // W
    assert (count, prod) == (want_c, want_p)
    assert progress == cum


@pytest.mark.parametrize("alg", ["HJ", "SMJ"])
def test_lazy_harness_device_ring_matches_oracle(harness, oracle, tmp_path, alg):
    """deviceRing: "Yes" replaces the pinned host ring with the device-resident
    ring: batches land in HBM as they arrive and each window is joined there.
    Same windows, counts, checksum and per-window progress as the oracle."""
    left, right = streams(oracle)
    count, prod, windows, progress = run(harness, tmp_path, alg, "LAZY", extra='deviceRing: "Yes"\n')
    want = [oracle.join(left[k * W:(k + 1) * W], right[k * W:(k + 1) * W], enumerate_pairs=False)
            for k in range(N // W)]
    assert windows == N // W
    assert count == sum(r["count"] for r in want)
    assert prod == sum(r["prod"] for r in want) % (1 << 64)
    assert progress == np.cumsum([r["count"] for r in want]).tolist()
    assert "lazy_gpu_" + alg.lower() + "_nm_ring" in run.last.stdout


def test_lazy_harness_zipf(harness, oracle, tmp_path):
    left, right = streams(oracle, theta=0.9, distinct=1 << 16)
    count, prod, _, _ = run(harness, tmp_path, "HJ", "LAZY", theta="0.9", distinct=1 << 16)
    want = [oracle.join(left[k * W:(k + 1) * W], right[k * W:(k + 1) * W], enumerate_pairs=False)
            for k in range(N // W)]
    assert count == sum(r["count"] for r in want)
    assert prod == sum(r["prod"] for r in want) % (1 << 64)


@pytest.mark.parametrize("alg,pk", [("HJ", "No"), ("NLJ", "No"), ("HJ", "Yes"), ("NLJ", "Yes"), ("SMJ", "Yes")])
def test_eager_harness_matches_oracle(harness, oracle, tmp_path, alg, pk):
    """usePK: "Yes" runs the eager joiner as one persistent kernel."""
    left, right = streams(oracle)
    count, _, windows, progress = run(harness, tmp_path, alg, "EAGER", extra=f'usePK: "{pk}"\n')
    bc, wc = oracle.eager_hj(left, right, B, W, DISTINCT)
    assert count == int(bc.sum())
    assert progress == np.cumsum(bc).tolist()          # one progress record per batch, arrival order
    assert windows == len(wc) - 1                      # closes counted; the last window stays open


@pytest.mark.parametrize("pk", ["No", "Yes"])
def test_eager_harness_eight_source_threads(harness, tmp_path, pk):
    """Eight source threads deliver batches concurrently.  The order differs
    from run to run, but each batch is executed and counted in the window it
    joined: the sum of the batch counts equals the sum of the windows' own
    totals, and every tuple is accounted for."""
    count, _, windows, progress = run(harness, tmp_path, "HJ", "EAGER",
                                      extra=f'usePK: "{pk}"\nsourceThreads: 8\n')
    assert count == run.window_pairs > 0
    assert len(progress) == 2 * N // B and progress[-1] == count
    assert windows >= N // W - 1


def test_power_samples_written(harness, tmp_path):
    """measurePowerUsage: "Yes" samples the GPU's power while the experiment
    runs and appends epoch-ms,watts lines to power_data.txt, as the
    reference's power agent does."""
    run(harness, tmp_path, "HJ", "LAZY", power="Yes")
    if "NVML unavailable" in run.last.stderr:
        pytest.skip("NVML is not available on this machine")
    lines = (tmp_path / "power_data.txt").read_text().strip().splitlines()
    assert lines
    ms, watts = lines[0].split(",")
    assert int(ms) > 0 and 0.0 < float(watts) < 5000.0
