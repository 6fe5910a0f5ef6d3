"""The C ABI library builds for sm_103a and exports every symbol the header
declares.  CPU only: no compute calls."""
import ctypes
import subprocess

import pytest


def test_library_builds_and_exports_all_declared_symbols():
    from letkf_gb300 import _build
    from letkf_gb300.lib import declared_symbols

    path = _build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    declared = declared_symbols()
    assert len(declared) >= 10
    missing = [s for s in declared if s not in exported]
    assert not missing, f"declared but not exported: {missing}"
    lib = ctypes.CDLL(path)
    for s in declared:
        getattr(lib, s)


def test_status_strings_and_version():
    from letkf_gb300 import lib as L

    lib = L.lib()
    assert b"sm_103a" in lib.letkf_version()
    for code in range(8):
        assert lib.letkf_status_string(code)


def test_no_gpu_is_an_error_not_a_fallback():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np

    from letkf_gb300.core import letkf_core
    from letkf_gb300.lib import LETKF_ERR_NOGPU, LetkfError

    with pytest.raises(LetkfError) as e:
        letkf_core(4, 2, 2, np.ones((2, 4)), np.ones(2), np.ones(2), np.zeros(2), 1.0)
    assert e.value.status == LETKF_ERR_NOGPU


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the server structs have the C layout (a probe
    compiled by gcc against include/letkf_gpu.h prints sizes and offsets)."""
    import os
    import shutil

    from letkf_gb300 import serve
    from letkf_gb300.lib import HEADER

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not available")
    structs = {"letkf_server_desc": serve.ServerDesc, "letkf_job_desc": serve.JobDesc,
               "letkf_job_result": serve.JobResult, "letkf_server_stats": serve.ServerStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "letkf_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_server_without_gpu_is_an_error():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from letkf_gb300.lib import LETKF_ERR_NOGPU, LetkfError
    from letkf_gb300.serve import Server

    with pytest.raises(LetkfError) as e:
        Server(nslots=2)
    assert e.value.status == LETKF_ERR_NOGPU


def test_new_entry_points_check_arguments_before_the_device():
    """letkf_sweep_run_host, letkf_sweep_deferred and letkf_search_l96_adaptive
    reject invalid arguments with LETKF_ERR_ARG before any device call (so the
    check holds on a machine without a GPU)."""
    import ctypes as C

    from letkf_gb300 import lib as L
    from letkf_gb300.sweep import _L

    lib = _L()
    assert lib.letkf_sweep_run_host(None, None, None, 4, None) == L.LETKF_ERR_ARG
    n = C.c_int(7)
    assert lib.letkf_sweep_deferred(None, C.byref(n)) == L.LETKF_ERR_ARG
    raw = L.lib()
    ad = raw.letkf_search_l96_adaptive
    for msw in (-1, 3):
        assert ad(40, 1, 40, None, 0, None, 0, 3.0, 2.0, 1.0, msw, 1.0, 1.0, 20, None, None, None, None, None, None,
                  None, None) == L.LETKF_ERR_ARG
    # adaptive modes need the perturbations
    cell = (C.c_int * 4)(1, 2, 3, 4)
    pix = (C.c_int * 2)(1, 2)
    assert ad(8, 1, 4, cell, 2, pix, 0, 3.0, 2.0, 1.0, 1, 1.0, 1.0, 20, None, None, None, None, None, None, None,
              None) == L.LETKF_ERR_ARG
    # slot out of range
    assert ad(8, 1, 4, cell, 2, pix, 1, 3.0, 2.0, 1.0, 0, 1.0, 1.0, 20, None, None, None, None, None, None, None,
              None) == L.LETKF_ERR_ARG


def test_scale_obsope_checks_arguments_before_the_device():
    """letkf_scale_obsope refuses khalo < 2 (the reference's level search can
    reach two halo levels above the top), short variable strides and missing
    observation arrays with LETKF_ERR_ARG, before any device call."""
    from letkf_gb300 import lib as L

    f = L.lib().letkf_scale_obsope
    plane3, plane2 = 36 * 30 * 24, 36 * 30
    args = lambda kh, var3, nobs: (36, 30, 24 - 2 * kh, kh, 4, None, 0, var3, None, 0, plane2, nobs, None, None, None,
                                   None, None, 0, 100.0, None, None, None, None)
    assert f(*args(1, plane3, 0)) == L.LETKF_ERR_ARG
    assert f(*args(2, plane3, 0)) == L.LETKF_ERR_ARG        # NULL fields
    import ctypes as C

    buf = (C.c_double * 1)()
    a = list(args(2, plane3 - 1, 0))
    a[5] = a[8] = C.cast(buf, C.c_void_p)
    assert f(*a) == L.LETKF_ERR_ARG                        # variable stride below one domain
    a = list(args(2, plane3, 5))
    a[5] = a[8] = C.cast(buf, C.c_void_p)
    assert f(*a) == L.LETKF_ERR_ARG                        # observations missing
