"""CPU tests of the C++ host harness (runExperiment): the YAML reader accepts
the reference's experiment files, the configuration cross product and the
WindowingFactory's algorithm names match the reference's, and bad files fail
with the reference's messages.  Nothing here launches a kernel."""
import subprocess

import pytest

BASE = {
    "algTypes": '[ "HJ" ] # "NLJ" | "HJ" | "SMJ"',
    "deviceTypes": '[ "GPU" ]',
    "progressivenessModes": '[ "LAZY" ]',
    "distinctKeys": "[ 1000 ]",
    "zipfThetas": "[ 0.0 ]",
    "resultMaterializationMethod": '[ "NoOutput" ]',
    "windowSizesMB": "[ 1 ]",
    "batchSizeKB": "[ 128 ]",
    "measuredMetric": '"Throughput"  # or "cumulativePercentage"',
    "measurePowerUsage": '"No"',
    "repeat": "5 # runs per configuration",
    "parStrats": '[ "INTRA" ]',
}


def write_yaml(tmp_path, **over):
    d = dict(BASE, **over)
    text = "# experiment file\n" + "".join(f"{k}: {v}\n" for k, v in d.items() if v is not None)
    p = tmp_path / "exp.yaml"
    p.write_text(text)
    return p


def listing(harness, path):
    r = subprocess.run([harness, str(path), "/dev/null", "--list"], capture_output=True, text=True, timeout=60)
    return r.returncode, r.stdout.strip().splitlines()[1:], r.stderr


def test_cross_product_and_names(harness, tmp_path):
    p = write_yaml(tmp_path, algTypes='[ "NLJ", "HJ", "SMJ" ]', progressivenessModes='[ "LAZY", "EAGER" ]',
                   windowSizesMB="[ 1, 2, 4 ]", zipfThetas="[ 0.0, 0.5 ]")
    rc, rows, err = listing(harness, p)
    assert rc == 0, err
    assert len(rows) == 3 * 2 * 3 * 2
    names = [r.split(",")[0] for r in rows]
    assert names[0] == "lazy_gpu_nlj_nm"
    assert set(names) == {f"{m}_gpu_{a}_nm" for m in ("lazy", "eager") for a in ("nlj", "hj", "smj")}
    # windowSizesMB and batchSizeKB are MiB / KiB of 16-byte tuples
    assert {int(r.split(",")[1]) for r in rows} == {65536, 131072, 262144}
    assert {int(r.split(",")[2]) for r in rows} == {8192}


@pytest.mark.parametrize("mode,suffix", [("NoOutput", "nm"), ("CountKernel", "ck"), ("EstimatedSelectivity", "es"),
                                         ("Atomic", "at")])
def test_result_mode_suffixes(harness, tmp_path, mode, suffix):
    rc, rows, err = listing(harness, write_yaml(tmp_path, resultMaterializationMethod=f'[ "{mode}" ]'))
    assert rc == 0, err
    assert rows[0].split(",")[0] == f"lazy_gpu_hj_{suffix}"


def test_bitmap_only_for_nested_loop(harness, tmp_path):
    rc, rows, _ = listing(harness, write_yaml(tmp_path, algTypes='[ "NLJ", "HJ" ]',
                                              resultMaterializationMethod='[ "Bitmap" ]'))
    assert rc == 0
    assert [r.split(",")[0] for r in rows] == ["lazy_gpu_nlj_bm", "Not Implemented"]


def test_cpu_device_is_not_provided(harness, tmp_path):
    rc, rows, _ = listing(harness, write_yaml(tmp_path, deviceTypes='[ "CPU", "GPU" ]'))
    assert rc == 0
    assert [r.split(",")[0] for r in rows] == ["Not Implemented", "lazy_gpu_hj_nm"]


def test_parallelization_strategy_sets_joiner_threads(harness, tmp_path):
    import os

    rc, rows, _ = listing(harness, write_yaml(tmp_path, parStrats='[ "INTRA", "INTER", "HYBRID" ]'))
    assert rc == 0
    joiners = [int(r.split(",")[5]) for r in rows]
    assert joiners == [1, os.cpu_count(), 4]


def test_optional_keys(harness, tmp_path):
    rc, rows, _ = listing(harness, write_yaml(tmp_path, dataSize="262144", sourceThreads="1"))
    assert rc == 0 and int(rows[0].split(",")[6]) == 262144
    rc, rows, _ = listing(harness, write_yaml(tmp_path))
    assert int(rows[0].split(",")[6]) == 2560 * 65536     # the reference's default stream length


@pytest.mark.parametrize("key,value,msg", [
    ("algTypes", '[ "XJ" ]', "Unknown algorithm type: XJ"),
    ("deviceTypes", '[ "TPU" ]', "Unknown device type: TPU"),
    ("parStrats", '[ "BOTH" ]', "Unknown parallelization strategy: BOTH"),
    ("measurePowerUsage", '"Maybe"', "Unknown parameter for measure power: Maybe"),
    ("measuredMetric", '"Latency"', "Unknown measured metrics: Latency"),
    ("repeat", None, "missing key repeat"),
])
def test_bad_files_fail(harness, tmp_path, key, value, msg):
    p = write_yaml(tmp_path, **{key: value})
    rc, _, err = listing(harness, p)
    assert rc == 2 and msg in err


def test_usage_message(harness):
    r = subprocess.run([harness], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "runExperiment <path_to_yaml_config> <outputFileName>" in r.stdout


def test_device_ring_key(harness, tmp_path):
    rc, _, err = listing(harness, write_yaml(tmp_path, deviceRing='"Maybe"'))
    assert rc == 2 and "Unknown parameter for deviceRing: Maybe" in err
    rc, rows, _ = listing(harness, write_yaml(tmp_path, deviceRing='"Yes"'))
    assert rc == 0 and rows


def test_use_pk_key(harness, tmp_path):
    rc, rows, _ = listing(harness, write_yaml(tmp_path, usePK='"Yes"', progressivenessModes='[ "EAGER" ]'))
    assert rc == 0 and rows[0].split(",")[0] == "eager_gpu_hj_pk_nm"
    rc, _, err = listing(harness, write_yaml(tmp_path, usePK='"Sometimes"'))
    assert rc == 2 and "Unknown parameter for usePK: Sometimes" in err


@pytest.fixture(scope="module")
def host_units(tmp_path_factory):
    """tests/host_units.cpp linked with the host windowing (CPU stand-in executors)."""
    import os
    import shutil

    import build as b

    b.build_lib()
    exe = str(tmp_path_factory.mktemp("units") / "host_units")
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(b.nvcc())))
    here = os.path.dirname(os.path.abspath(__file__))
    cmd = [shutil.which("g++") or "g++", "-O1", "-std=c++17", "-I", os.path.join(b.ROOT, "include"), "-I", b.HOST,
           "-I", os.path.join(cuda, "include"), os.path.join(here, "host_units.cpp"),
           os.path.join(b.HOST, "sjb_host.cpp"), "-o", exe, "-L", b.LIBDIR, "-lsjbg", "-Wl,-rpath," + b.LIBDIR,
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64"),
           "-lpthread", "-ldl"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _units(exe, mode):
    r = subprocess.run([exe, mode], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return dict(line.split("=", 1) for line in r.stdout.strip().splitlines())


def test_lazy_ring_buffer_full_is_an_error_and_the_windowing_goes_on(host_units):
    """With every batch slot held by a window being joined, the next batch
    fails with the reference's message instead of exiting the process; once
    the join returns the next window goes through."""
    out = _units(host_units, "ring")
    assert out["ring_full_thrown"] == "1" and out["message"] == "Ring buffer is full"
    assert out["windows"] == "2" and int(out["match_count"]) == 2 * (2 * 1000 + 2)


def test_eager_close_rule_under_eight_source_threads(host_units):
    """Eight source threads: the executor is never entered twice at once, and
    every batch's matches are counted into the window it joined."""
    out = _units(host_units, "eager")
    assert out["overlap"] == "0"
    assert out["match_count"] == out["window_total"] and int(out["match_count"]) > 0
    assert out["windows_closed"] == out["sink_windows"] and int(out["windows_closed"]) > 30
