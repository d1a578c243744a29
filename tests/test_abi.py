"""The C-ABI library loads and exports every entry point include/gi.h declares
(no compute calls here)."""
import ctypes as C
import re

import pytest


def test_header_entry_points_exported(pkg):
    names = pkg.header_functions()
    assert len(names) >= 15
    lib = pkg.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(pkg):
    lib = pkg.lib()
    for s in range(8):
        assert lib.gi_status_string(s)
    assert lib.gi_status_string(0) == b"ok"


def test_null_arguments_rejected(pkg):
    lib = pkg.lib()
    assert lib.gi_create(None, 0, 0) == pkg.GI_ERR_ARG
    assert lib.gi_destroy(None) == pkg.GI_OK
    assert lib.gi_set_symmetry(None, 1) == pkg.GI_ERR_ARG
    # streamed dipole and the split GEMM probe check their arguments before any CUDA call
    assert lib.gi_set_dipole_streamed(None, 10, None, 0, 0) == pkg.GI_ERR_ARG
    assert lib.gi_dipole_panel_rows(None) == 0
    assert lib.gi_probe_split_gemm(0, 0, 0, 4, 64, None, None, None) == pkg.GI_ERR_ARG
    assert lib.gi_probe_split_gemm(0, 0, 4, 4, -1, None, None, None) == pkg.GI_ERR_ARG


def test_struct_layouts_match_header(pkg, tmp_path):
    """Field offsets of the ctypes mirrors equal the C compiler's for gi.h."""
    import os
    import subprocess
    import numpy as np
    structs = {"gi_params": pkg.gi_params, "gi_stats": pkg.gi_stats,
               "gi_serve_config": pkg.gi_serve_config, "gi_job_info": pkg.gi_job_info,
               "gi_serve_stats": pkg.gi_serve_stats, "gi_line_text": pkg.gi_line_text}
    dtypes = {"gi_line": pkg.LINE_DTYPE, "gi_level": pkg.LEVEL_DTYPE,
              "gi_line_compact": pkg.LINE_COMPACT_DTYPE}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gi.h"', "int main(void){"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    for name, dt in dtypes.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f in dt.names:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    inc = os.path.dirname(pkg.HEADER)
    subprocess.check_call(["gcc", "-I", inc, str(src), "-o", str(exe)])
    got = dict(l.split() for l in subprocess.check_output([str(exe)]).decode().splitlines())
    for name, cls in structs.items():
        assert int(got[name]) == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(got[f"{name}.{f}"]) == getattr(cls, f).offset, (name, f)
    for name, dt in dtypes.items():
        assert int(got[name]) == dt.itemsize, name
        for f in dt.names:
            assert int(got[f"{name}.{f}"]) == dt.fields[f][1], (name, f)


def test_create_without_gpu_fails_cleanly(pkg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.GiError):
        pkg.Engine(0)
