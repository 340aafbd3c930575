"""The C-ABI library loads and exports every entry point include/tt_cuda.h
declares (no compute calls: this file also runs without a GPU)."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared():
    txt = (ROOT / "include" / "tt_cuda.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tt_cuda_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared()
    for must in ["tt_cuda_fillsinks", "tt_cuda_fillsinks_hybrid", "tt_cuda_identifyflats",
                 "tt_cuda_gwdt_computecosts", "tt_cuda_gwdt", "tt_cuda_flow_routing_d8_carve",
                 "tt_cuda_flow_accumulation", "tt_cuda_hillshade", "tt_cuda_hillshade_fused",
                 "tt_cuda_gradient_secondorder", "tt_cuda_reconstruct",
                 "tt_cuda_reconstruct_hybrid", "tt_cuda_flow_accumulation_backward",
                 "tt_cuda_hillshade_backward", "tt_cuda_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol():
    from libtopotoolbox_gb300 import _native

    lib = _native.lib()  # loads; no compute
    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(tt_cuda_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    for n in declared():
        assert hasattr(lib, n)
    # the Python binding covers the whole header
    assert set(declared()) == set(_native.SIGNATURES)


def test_status_strings():
    from libtopotoolbox_gb300 import _native

    lib = _native.lib()
    for code, text in _native.STATUS.items():
        assert lib.tt_cuda_status_string(code).decode() == text


def test_no_cpu_fallback_when_library_missing(tmp_path, monkeypatch):
    """Compute entry points raise when the native library is absent."""
    from libtopotoolbox_gb300 import _native

    monkeypatch.setattr(_native, "LIB_PATH", tmp_path / "missing.so")
    monkeypatch.setattr(_native, "_LIB", None)
    import numpy as np

    from libtopotoolbox_gb300 import api

    with pytest.raises(ImportError):
        api.fillsinks(np.zeros((4, 4), np.float32), np.ones((4, 4), np.uint8))


def test_deferral_without_a_device():
    """Deferred status on a host without a GPU: nothing to defer, and ending a
    deferral that never began is an argument error (no device call made)."""
    from libtopotoolbox_gb300 import _native

    lib = _native.lib()
    if lib.tt_cuda_has_gpu():
        pytest.skip("a GPU is present: tests/test_gpu_deferred.py covers deferral")
    assert lib.tt_cuda_defer_end() == 1
    assert lib.tt_cuda_defer_begin(None) == 6
    assert lib.tt_cuda_defer_end() == 1
