"""CPU-side checks of the C ABI: the library builds, loads, exports every entry point that
include/hpdex_gb300.h declares, and refuses to compute without a GPU (no CPU fallback)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "hpdex_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hpdex_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from hpdex_gb300 import _lib
    L = _lib.lib()
    names = declared_functions()
    assert len(names) >= 13
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.EXPORTS, f"{n} has no ctypes signature"


def test_options_default_matches_reference_binding():
    from hpdex_gb300 import _lib
    o = _lib.MwuOptions()
    _lib.lib().hpdex_mwu_options_default(ctypes.byref(o))
    # module.cpp:215-227 defaults; the C default of fast_norm is 0 (the precise path), the
    # Python binding passes the reference's fast_norm=True explicitly
    assert (o.ref_sorted, o.tar_sorted, o.tie_correction, o.use_continuity) == (0, 0, 1, 0)
    assert (o.zero_handling, o.alternative, o.method) == (0, 2, 2)


def test_no_device_fails_loudly():
    from hpdex_gb300 import _lib
    from hpdex_gb300.backend.bin import kernel
    if _lib.device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(_lib.HpdexError, match="no CUDA device"):
        kernel.mannwhitneyu(np.ones(4, np.float32), np.arange(4), np.array([0, 4]),
                            np.zeros(4, np.int32), 1)


def test_unsupported_dtype_message():
    from hpdex_gb300.backend.bin import kernel
    with pytest.raises(RuntimeError, match="Unsupported dtype for data"):
        kernel.mannwhitneyu(np.ones(4, np.float16), np.arange(4), np.array([0, 4]),
                            np.zeros(4, np.int32), 1)
