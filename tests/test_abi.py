"""CPU checks of the C ABI: the library builds, loads without a GPU and
exports every entry point that include/*.h declares."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:GBX_API\s+)?(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gbx_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def built():
    from dtcf_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "gbx_transpose" in names and "gbx_local_contraction" in names and "gbx_execute" in names


def test_library_exports_every_declared_symbol(built):
    import ctypes
    lib = ctypes.CDLL(built)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built):
    from dtcf_gb300 import _lib
    missing = [n for n in declared_symbols() if n not in _lib.SIGNATURES]
    assert not missing, missing


def test_error_path_without_gpu(built):
    """Argument checks run on the host and report through gbx_last_error."""
    import ctypes
    from dtcf_gb300 import _lib
    lib = _lib.lib()
    perm = (ctypes.c_int * 2)(0, 0)
    widths = (ctypes.c_int * 2)(3, 4)
    rc = lib.gbx_transpose(None, None, perm, 2, widths, None)
    assert rc == -1
    assert b"permutation" in lib.gbx_last_error()
    assert lib.gbx_version().startswith(b"dtcf_gb300")
