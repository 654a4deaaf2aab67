"""The C-ABI library builds, loads and exports every declared entry point
(no GPU needed)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "bsamg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bsamg_\w+)\s*\(", txt)))


def test_header_declares_the_interface():
    names = declared()
    for must in ("bsamg_init", "bsamg_hier_create", "bsamg_patch_add", "bsamg_commit",
                 "bsamg_put_field", "bsamg_get_field", "bsamg_multigrid_iterations",
                 "bsamg_time_step", "bsamg_strerror"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    import ctypes
    L = pkg.lib()
    for name in declared():
        assert hasattr(L, name), name
        assert isinstance(getattr(L, name), ctypes._CFuncPtr)


def test_status_strings(pkg):
    L = pkg.lib()
    assert L.bsamg_strerror(0) == b"ok"
    assert b"budget" in L.bsamg_strerror(-3)
