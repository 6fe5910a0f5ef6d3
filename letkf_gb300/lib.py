"""ctypes binding of libletkf_gpu.so (the C ABI in include/letkf_gpu.h).

The library is the product path: if it is missing or no CUDA device is
present, the calls fail loudly.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import _build

LETKF_OK = 0
LETKF_ERR_ARG = 1
LETKF_ERR_EIG = 2
LETKF_ERR_CUDA = 3
LETKF_ERR_CAPACITY = 4
LETKF_ERR_NOGPU = 5
LETKF_ERR_TIMEOUT = 6
LETKF_MAX_NE = 128
LETKF_LARGEK_MAX_NE = 1024
LETKF_MAX_NOBS_PER_GRID_LIMIT = 256

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "letkf_gpu.h")


class LetkfError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__(f"{what}: letkf status {status} ({status_string(status)})")


_lib = None

_vp = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_d = C.c_double
_pd = C.POINTER(C.c_double)

_SIGS = {
    "letkf_version": (C.c_char_p, []),
    "letkf_status_string": (C.c_char_p, [_i]),
    "letkf_launch_count": (_i64, []),
    "letkf_device_sync": (_i, []),
    "letkf_core_c": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _d]),
    "letkf_core_batch_f64": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _d, _vp, _vp]),
    "letkf_core_batch_mixed": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _d, _vp, _vp]),
    "letkf_update_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "letkf_search_scale": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp,
                                _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_search_scale_limited": (_i, [_i, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i,
                                        _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_sort_obs_latlon": (_i, [_i, _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_search_gfs": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp,
                              _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_search_speedy": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp,
                                 _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_exclusive_scan": (_i, [_i, _vp, _vp, _vp]),
    "letkf_exclusive_scan_static": (_i, [_i, _vp, _vp, _vp]),
    "letkf_gather_rows": (_i, [_i, _i64, _vp, _vp, _vp, _i, _vp, _vp, _vp]),
    "letkf_search_l96": (_i, [_i, _i, _vp, _i, _vp, _d, _d, _d, _d, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_search_l96_4d": (_i, [_i, _i, _i, _vp, _i, _vp, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_search_l96_adaptive": (_i, [_i, _i, _i, _vp, _i, _vp, _i, _d, _d, _d, _i, _d, _d, _i, _vp, _vp, _vp, _vp,
                                       _vp, _vp, _vp, _vp]),
    "letkf_l96_obs_cell": (_i, [_i, _i, _vp, _vp, _vp]),
    "letkf_obs_departure": (_i, [_i, _i, _vp, _vp, _vp, _d, _vp, _vp, _vp, _vp, _vp]),
    "letkf_core_batch_largek": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _d, _vp, _vp]),
    "letkf_update_mixed": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "letkf_core_batch_largek_indexed": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _d, _vp,
                                             _vp]),
    "letkf_update_bf16": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_obs_analysis": (_i, [_i, _i, _vp, _vp, _vp, _d, _vp, _d, _vp, _vp, _vp]),
    "letkf_efso": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_grd_decode": (_i, [_i64, _i, _i, _vp, _i, _i, _i, _i, _vp, _i64, _i64, _vp]),
    "letkf_grd_encode": (_i, [_i64, _i, _i, _vp, _i, _i64, _i64, _i, _i, _i, _vp, _vp]),
    "letkf_ens_mean_spread": (_i, [_i64, _i, _i, _vp, _i64, _i64, _vp, _vp, _vp]),
    "letkf_speedy_obsope": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _i, _vp, _vp, _vp, _vp,
                                 _vp, _vp, _vp, _vp, _vp]),
    "letkf_scale_obsope": (_i, [_i, _i, _i, _i, _i, _vp, _i64, _i64, _vp, _i64, _i64, _i, _vp, _vp, _vp, _vp, _vp,
                                _i, _d, _vp, _vp, _vp, _vp]),
    "letkf_update_relax_f64": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "letkf_relax_beta": (_i, [_i, _i, _vp, _vp, _vp, _i, _i, _d, _d, _d, _d, _i, _i, _i, _i, _vp, _vp]),
}


def declared_symbols():
    """Function names declared in include/letkf_gpu.h."""
    with open(HEADER) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(letkf_[a-z0-9_]+)\s*\(", txt)))


def lib(build: bool = True):
    """Load libletkf_gpu.so (building it in-tree first if needed)."""
    global _lib
    if _lib is None:
        path = _build.build() if build else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(f"libletkf_gpu.so is missing at {path}; run __graft_entry__.build()")
        L = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(s):
    try:
        return lib().letkf_status_string(int(s)).decode()
    except Exception:  # pragma: no cover - only while the library cannot load
        return "?"


def check(status, what="letkf"):
    if status != LETKF_OK:
        raise LetkfError(status, what)
    return status


def launch_count():
    return int(lib().letkf_launch_count())
