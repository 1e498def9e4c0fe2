"""The C ABI library loads, exports every entry point include/rj.h declares,
and its struct layouts agree with the binding (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

import rasterjoin as rj

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rj.h")


def declared_functions():
    src = open(HEADER).read()
    return re.findall(r"RJ_API\s+[\w\s\*]+?\b(rj_\w+)\s*\(", src)


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("rj_create", "rj_destroy", "rj_load_points", "rj_set_polygons", "rj_execute", "rj_last_error",
              "rj_get_timings", "rj_format_time_stats", "rj_query_init", "rj_attach_points_device"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(rj.LIB_PATH)
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", rj.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (rj_\w+)", out))
    assert set(declared_functions()) <= exported
    # nothing but the C ABI is exported under the rj_ prefix
    assert exported <= set(declared_functions())


def test_struct_layouts_match_binding(tmp_path):
    probe = tmp_path / "probe.c"
    probe.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "rj.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(rj_constraint), sizeof(rj_query), sizeof(rj_result),
         sizeof(rj_config), sizeof(rj_column), sizeof(rj_timings), offsetof(rj_query, flags),
         sizeof(rj_batch_stats), sizeof(rj_server_config), sizeof(rj_request_info),
         offsetof(rj_batch_stats, kernel_launches));
  return 0;
}
''')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(probe), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert vals[0] == 16 == C.sizeof(rj.QueryConstraint)       # QueryConstraint, main.cpp:376
    assert vals[1] == C.sizeof(rj.Query)
    assert vals[2] == C.sizeof(rj.Result)
    assert vals[3] == C.sizeof(rj.Config)
    assert vals[4] == C.sizeof(rj.Column)
    assert vals[5] == C.sizeof(rj.Timings)
    assert vals[6] == rj.Query.flags.offset
    assert vals[7] == C.sizeof(rj.BatchStats)
    assert vals[8] == C.sizeof(rj.ServerConfig)
    assert vals[9] == C.sizeof(rj.RequestInfo)
    assert vals[10] == rj.BatchStats.kernel_launches.offset


def test_query_defaults(built):
    q = rj.default_query()
    # reference defaults: accuracy 100 m (main.cpp:268), grid 256 (main.cpp:299), tile 8192
    assert q.accuracy_m == 100.0 and q.grid_res == 256 and q.max_fbo_size == 8192
    assert q.function_type == rj.RasterJoinFn and q.aggregation == rj.Count and q.time_attrib == -1


def test_enum_values_match_reference():
    assert (rj.RasterJoinFn, rj.IndexJoinFn, rj.HybridJoinFn, rj.RasterJoinBoundFn) == (0, 1, 2, 3)
    assert (rj.Count, rj.Avg, rj.Sum) == (0, 1, 2)
    assert (rj.EQ, rj.LT, rj.LTE, rj.GT, rj.GTE) == (0, 1, 2, 3, 4)
    assert (rj.Location, rj.Uint, rj.Int, rj.Float) == (0, 1, 2, 3)


def test_create_without_gpu_returns_status(built):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = rj.load_library()
    h = C.c_void_p()
    rc = lib.rj_create(C.byref(rj.Config(0, 0, None)), C.byref(h))
    assert rc == -5 and not h.value
    # calls on a null context are rejected, not crashing
    assert lib.rj_execute(None, None, None) == -1
    assert lib.rj_set_polygons(None, None, None, 0, None) == -1
    assert lib.rj_execute_batch(None, 0, None, None, None, None, 0, None) == -1
    assert lib.rj_build_time_index(None, 0, 0) == -1
    assert lib.rj_submit(None, None, None, None, None) == -1
    assert lib.rj_poll(None, 0, 0, None) == -1
    with pytest.raises(rj.RJError):
        rj.GLHandler()


def header_constants(prefixes):
    """Integer #defines of include/rj.h whose names start with one of prefixes."""
    out = {}
    for name, val in re.findall(r"^#define\s+(RJ_\w+)\s+(-?(?:0x[0-9A-Fa-f]+|\d+))u?\b", open(HEADER).read(), re.M):
        if name.startswith(prefixes):
            out[name] = int(val, 0)
    return out


def test_binding_constants_match_header():
    """Every flag, tuning knob and batch flag of the header has the binding's
    constant of the same name and value, and the status names agree."""
    consts = header_constants(("RJ_FLAG_", "RJ_TUNE_", "RJ_BATCH_"))
    assert len(consts) >= 20
    for name, val in consts.items():
        assert getattr(rj, name[3:]) == val, name
    status = header_constants(("RJ_OK", "RJ_E_", "RJ_PENDING"))
    assert status and all(rj.STATUS[v] == name for name, v in status.items())
