"""CPU checks of the drop-in boundary: the C-ABI library loads and exports every
entry point declared in include/iskra_gpu.h (no compute calls: no GPU here)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "iskra_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*\*?\s*(iskra_\w+)\s*\(", src)))


def test_header_declares_the_api():
    syms = declared_symbols()
    assert "iskra_ctx_create" in syms and "iskra_step" in syms and "iskra_mcc_perform" in syms
    assert len(syms) >= 35


def test_library_exports_every_declared_symbol():
    from iskra_gb300 import _lib
    lib = _lib.load()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"missing exports: {missing}"


def test_python_binding_covers_every_symbol():
    from iskra_gb300 import _lib
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) == bound


def test_library_links_no_oracle():
    """The product library must not reference the oracle."""
    from iskra_gb300 import _lib
    data = open(_lib.LIB_PATH, "rb").read()
    assert b"orc_" not in data and b"liboracle" not in data


def test_missing_device_fails_loudly():
    """Without a CUDA device, context creation returns an error code (no fallback)."""
    import pytest
    from iskra_gb300 import _lib
    from iskra_gb300.device import Context
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except Exception:
        pass
    with pytest.raises(_lib.IskraError):
        Context(8, 8, 1.0, 1.0)


def test_grid_struct_layout():
    from iskra_gb300 import _lib
    assert ctypes.sizeof(_lib.Grid) == 4 + 4 + 8 * 4 + 4 * 4
