"""The C-ABI library builds, loads and exports every entry point declared in include/gfe.h
(no compute calls: runs without a GPU)."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    text = (ROOT / "include" / "gfe.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t)\s+(gfe_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    names = header_functions()
    for required in ("gfe_version", "gfe_last_error", "gfe_csr_structure", "gfe_laplace_assemble",
                     "gfe_cg_solve"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from iron_gb300 import build as gb
    from iron_gb300 import _lib
    lib_path = gb.build()
    L = _lib.load(lib_path)
    missing = [n for n in header_functions() if not hasattr(L, n)]
    assert not missing, missing
    # ctypes signatures cover the whole header
    assert set(header_functions()) <= set(_lib.SIGNATURES)
    assert L.gfe_version() >= 100


def test_error_text_roundtrip_without_gpu():
    """Argument validation happens before any device work; the message is retrievable."""
    from iron_gb300 import _lib
    L = _lib.load()
    rc = L.gfe_csr_structure(-1, 8, None, 10, None, None, 0, None, None)
    assert rc == -1
    assert "gfe_csr_structure" in _lib.last_error()
    with pytest.raises(_lib.GfeError) as ei:
        _lib.check(rc)
    assert ei.value.status == -1


def test_no_cpu_fallback_without_cuda():
    import torch
    from iron_gb300 import _lib
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    with pytest.raises(_lib.GfeError):
        _lib.require_cuda()
