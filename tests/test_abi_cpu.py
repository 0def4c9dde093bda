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


def elf_dynamic(path):
    """(DT_NEEDED libraries, dynamic symbols as (name, defined)) of a 64-bit
    little-endian ELF shared object, read from its section headers, .dynsym,
    .dynstr and .dynamic (the ELF-64 object file format)."""
    import struct
    data = open(path, "rb").read()
    assert data[:4] == b"\x7fELF" and data[4] == 2 and data[5] == 1, "64-bit little-endian ELF expected"
    shoff, = struct.unpack_from("<Q", data, 0x28)
    shentsize, shnum, shstrndx = struct.unpack_from("<HHH", data, 0x3A)
    secs = []
    for k in range(shnum):
        name, typ, _, _, off, size, link, _, _, entsize = struct.unpack_from("<IIQQQQIIQQ", data, shoff + k * shentsize)
        secs.append((name, typ, off, size, link, entsize))

    def cstr(off):
        return data[off:data.index(b"\0", off)].decode()

    SHT_DYNSYM, SHT_DYNAMIC = 11, 6
    syms, needed = [], []
    for name, typ, off, size, link, entsize in secs:
        strtab = secs[link][2]
        if typ == SHT_DYNSYM:
            for e in range(off, off + size, entsize):
                st_name, _, _, st_shndx = struct.unpack_from("<IBBH", data, e)
                if st_name:
                    syms.append((cstr(strtab + st_name), st_shndx != 0))
        elif typ == SHT_DYNAMIC:
            for e in range(off, off + size, 16):
                tag, val = struct.unpack_from("<qQ", data, e)
                if tag == 0:
                    break
                if tag == 1:  # DT_NEEDED
                    needed.append(cstr(strtab + val))
    return needed, syms


def test_library_links_no_oracle():
    """The product library neither needs the oracle's library nor imports or
    exports any oracle symbol (its dynamic section and symbol table)."""
    from iskra_gb300 import _lib
    needed, syms = elf_dynamic(_lib.LIB_PATH)
    assert needed, "no DT_NEEDED entries read"
    assert not [n for n in needed if "oracle" in n], needed
    assert not [s for s, _ in syms if s.startswith("orc_")]
    exported = {s for s, defined in syms if defined}
    assert set(declared_symbols()) <= exported


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
