"""The C-ABI library loads without a GPU and exports every entry point that
include/diver_gb300.h declares (no compute calls)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"DV_API\s+[\w\s\*]*?\b(dv_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "dv_masked_intersect" in names and "dv_ray_march" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol():
    from diver_gb300 import _native

    lib = _native.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_bindings_cover_header():
    from diver_gb300 import _native

    missing = [n for n in declared_symbols() if n not in _native.SIGNATURES]
    assert not missing, f"no ctypes signature for: {missing}"


def test_status_strings_and_version():
    from diver_gb300 import _native

    lib = _native.lib()
    assert lib.dv_version() >= 100
    assert lib.dv_status_string(0) == b"ok"
    assert lib.dv_status_string(1) == b"invalid argument"


def test_argument_errors_need_no_gpu():
    from diver_gb300 import _native

    lib = _native.lib()
    # negative sizes and NULL buffers are rejected before any CUDA call
    assert lib.dv_ray_voxel_count(-1, 0.0, 64.0, 1.0, None, None, None, None, None) == 1
    assert lib.dv_masked_count(8, 0.0, 64.0, 1.0, 1.0, None, None, None, None, None, None) == 1
    assert lib.dv_aabb_intersect(8, None, None, None, None, None, None, 100, None) == 1
    # empty batches are a no-op success
    assert lib.dv_ray_march(0, None, None, None, None, 64, None) == 0
