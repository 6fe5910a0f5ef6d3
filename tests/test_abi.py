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
    for code in range(7):
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
