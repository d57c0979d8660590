"""The C-ABI library builds, loads without a GPU, and exports every entry
point that include/ads_gpu.h declares (no compute calls)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ads_gpu.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ads_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared()
    assert "ads_create" in names and "ads_step" in names and "ads_heat_adjoint" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(ads_mod):
    lib = ctypes.CDLL(ads_mod.lib_path())
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header(ads_mod):
    from ads_mpi_gb300.ads import ABI
    bound = {n for n, _, _ in ABI}
    assert set(declared()) <= bound


def test_status_strings(ads_mod):
    L = ads_mod.load()
    assert L.ads_status_string(0) == b"ok"
    assert L.ads_status_string(7) == b"unsupported configuration"
