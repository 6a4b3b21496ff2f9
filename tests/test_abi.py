"""The C-ABI library loads and exports every entry point include/knc.h declares."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    text = (ROOT / "include" / "knc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(knc_[a-z0-9_]+)\s*\(", text)
    # typedef'd function pointer types are not entry points
    return sorted(set(n for n in names if not n.endswith("_fn")))


def test_header_declares_entry_points():
    names = header_functions()
    assert "knc_advance" in names and "knc_create" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    import ctypes
    from knc import abi
    if not abi.LIB_PATH.exists():
        import build as b
        b.build()
    lib = ctypes.CDLL(str(abi.LIB_PATH))
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding declares a signature for each of them
    assert set(header_functions()) <= set(abi.SIGNATURES), set(header_functions()) - set(abi.SIGNATURES)


def test_no_cpu_fallback_without_library(tmp_path):
    from knc import abi
    with pytest.raises(FileNotFoundError):
        abi.load(tmp_path / "libknc_gpu.so")
