"""The C-ABI library builds, loads without a GPU and exports every entry point
declared in include/ubs.h (no compute calls: this runs on CPU-only hosts)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(ubs_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "ubs_raster_fwd" in names and "ubs_isect_count" in names and len(names) >= 19


def test_library_exports_every_declared_symbol():
    from ubs import _lib
    lib = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    unbound = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not unbound, "no ctypes signature for %s" % unbound
    assert lib.ubs_abi_version() == 2


def test_workspace_queries_and_argument_checks():
    """Size queries and argument validation run on the host."""
    from ubs import _lib
    lib = _lib.lib()
    assert lib.ubs_raster_workspace_bytes(1000, 3) >= 1000 * 48
    assert lib.ubs_isect_sort_workspace_bytes(1, 1000, 8160, 5000) >= 5000 * 16
    # bad tile size is rejected before any device work
    rc = lib.ubs_raster_fwd(1, 10, 3, 0, *([None] * 7), 64, 64, 12, 6, 6, None, None, None, None,
                            None, None, 0, None)
    assert rc == -3 and "tile_size" in _lib.last_error()
    rc = lib.ubs_cond_fwd(10, 15, *([None] * 8), None)
    assert rc == -3


def test_product_path_has_no_cpu_fallback():
    """Calling a product operator without a CUDA tensor raises instead of
    computing on the CPU."""
    import torch
    from gsplat.cuda._wrapper import l_triangle_to_rotmat
    with pytest.raises((ValueError, RuntimeError, AssertionError)):
        l_triangle_to_rotmat(torch.zeros(4, 3))
