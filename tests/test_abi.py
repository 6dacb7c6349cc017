"""CPU tests of the C-ABI boundary: the library builds, loads and exports
every entry point include/sjbg.h declares; the Python structures match the C
layouts; host-side argument checks fail loudly without touching a GPU."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sjbg.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^SJBG_API [^(]*?\b(sjbg_\w+)\(", text, flags=re.M)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for s in ("sjbg_create", "sjbg_destroy", "sjbg_lazy_execute", "sjbg_lazy_execute_batch", "sjbg_eager_execute",
              "sjbg_eager_clear_states", "sjbg_stream_open", "sjbg_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = set(re.findall(r" T (sjbg_\w+)", out.stdout))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    assert sorted(lib.EXPORTS) == declared_symbols()
    L = lib.load()
    for s in declared_symbols():
        assert hasattr(L, s)


def test_struct_layouts_match_header(lib):
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "sjbg.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(sjbg_tuple), sizeof(sjbg_pair), sizeof(sjbg_config),
         sizeof(sjbg_window_result), sizeof(sjbg_window_desc), sizeof(sjbg_stream_stats),
         offsetof(sjbg_config, hbm_budget_bytes), sizeof(sjbg_stream_window),
         offsetof(sjbg_stream_window, window_id));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [16, 8, C.sizeof(lib.Config), C.sizeof(lib.WindowResult), C.sizeof(lib.WindowDesc),
                     C.sizeof(lib.StreamStats), lib.Config.hbm_budget_bytes.offset, C.sizeof(lib.StreamWindow),
                     lib.StreamWindow.window_id.offset]
    assert lib.TUPLE_DTYPE.itemsize == 16 and lib.PAIR_DTYPE.itemsize == 8


def test_create_validates_before_touching_a_device(lib):
    bad = [dict(algorithm=7), dict(progressiveness=5), dict(result_mode=9), dict(partitioner=9),
           dict(radix_bits=20), dict(max_tuples_per_window=0),
           dict(progressiveness=lib.EAGER, batch_size=0, window_size=16)]
    for kw in bad:
        with pytest.raises(lib.SjbgError) as e:
            lib.Joiner(**kw)
        assert e.value.code == 1 or e.value.code == 6, kw


def test_null_handle_calls_return_invalid(lib):
    L = lib.load()
    assert L.sjbg_destroy(None) == 1
    assert L.sjbg_lazy_execute(None, None, 0, None, 0, 0, None, 0, None) == 1
    assert L.sjbg_kernel_stats_reset(None) == 1
    assert L.sjbg_launch_count(None) == 0
    assert L.sjbg_version() == 1


def test_eager_run_results_stop_at_the_first_absent_window():
    """sjbg_eager_run fills one result per window and status E_INVALID after the
    last one; the binding returns exactly the windows (no kernel runs here)."""
    import sjbg

    res = (sjbg.WindowResult * 8)()
    for i in range(8):
        res[i].count = 100 + i
        res[i].prod_checksum = 7 * i
        res[i].flags = sjbg.WR_XOR if i == 1 else 0
        res[i].xor_checksum = 99
        res[i].status = 0 if i < 3 else 1
    wins = sjbg.window_dicts(res)
    assert [w["count"] for w in wins] == [100, 101, 102]
    assert [w["prod"] for w in wins] == [0, 7, 14]
    assert [w["xor"] for w in wins] == [None, 99, None]
    for i in range(8):
        res[i].status = 0
    assert len(sjbg.window_dicts(res)) == 8
    res[0].status = 1
    assert sjbg.window_dicts(res) == []
