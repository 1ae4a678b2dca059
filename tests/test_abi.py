"""CPU tests of the C ABI library: it builds for sm_103a, loads, and exports
every function include/letkf_gpu.h declares; argument validation that needs
no device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "letkf_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:int|void|const char\*)\s+\**(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for n in ("lg_create", "lg_set_grid", "lg_set_obs", "lg_run", "lg_run_device",
              "lg_core_batch", "letkf_core_", "lg_destroy", "lg_get_stats", "lg_get_tuning",
              "lg_set_tuning", "lg_autotune"):
        assert n in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_null_arguments(built_lib):
    import letkf_gb300 as lg
    L = lg.load_library()
    assert L.lg_status_string(0) == b"LG_OK"
    assert L.lg_status_string(-4) == b"LG_ERR_NAN"
    assert L.lg_create(None, None) == -1
    cfg = lg.preset("tiny2d").to_c()
    cfg.cube_n = 2
    cfg.overlap = 2
    h = C.c_void_p()
    assert L.lg_create(C.byref(h), C.byref(cfg)) == -1  # overlap >= cube_n: no step
    cfg = lg.preset("tiny2d").to_c()
    cfg.ens = 1
    assert L.lg_create(C.byref(h), C.byref(cfg)) == -1
    assert L.lg_letkf_core(1, 0, None, None, None, None, None, None, 1.0) == -1
    assert L.lg_get_tuning(None, None) == -1
    assert L.lg_set_tuning(None, None) == -1
    assert L.lg_autotune(None, None, None, None, None, None, None) == -1
    assert L.lg_get_timeline(None, None, 0, None) == -1


def test_python_mirror_struct_layout_matches_header(built_lib, tmp_path):
    """Compile the header with gcc and compare sizes and field offsets with the
    ctypes mirror used by the Python host code."""
    import subprocess

    import letkf_gb300 as lg
    structs = {"lg_config": lg.LgConfig, "lg_obs_type": lg.LgObsType,
               "lg_obs_soa": lg.LgObsSoa, "lg_stats": lg.LgStats, "lg_tuning": lg.LgTuning}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "letkf_gpu.h"',
             "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.split() for line in subprocess.check_output([str(exe)], text=True).splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


def test_context_creation_fails_loudly_without_a_gpu(built_lib):
    """No host fallback: without a CUDA device, creating a context is an
    error (LG_ERR_CUDA), not a silent CPU path."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import letkf_gb300 as lg
    with pytest.raises(RuntimeError, match="LG_ERR_CUDA"):
        lg.Letkf(lg.preset("tiny2d"))
