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
    assert lib.dv_masked_count(8, 0.0, 64.0, 1.0, 1.0, None, None, None, None, None, None, None) == 1
    assert lib.dv_aabb_intersect(8, None, None, None, None, None, None, 100, None) == 1
    # empty batches are a no-op success
    assert lib.dv_ray_march(0, None, None, None, None, 64, None) == 0


def test_argument_errors_of_the_later_entry_points_need_no_gpu():
    """Validation of the device-count, save-buffer, occupancy, implicit-stage,
    camera and real-time-frame entry points runs on the host first."""
    import ctypes as C

    from diver_gb300 import _native

    lib = _native.lib()
    fake = C.c_void_p(16)  # never dereferenced: every call below fails validation first
    # empty work is a no-op success
    assert lib.dv_occupancy_max(0, None, None, None, 64, 0, None, None) == 0
    assert lib.dv_corner_rows(None, None, 3, 0, 65, None, None) == 0
    assert lib.dv_integrate_table_fwd(None, 0, 32, None, None, None, 3, 0, None, None) == 0
    assert lib.dv_camera_rays(4, 4, 1.0, (C.c_float * 12)(), 0, 0, None, None, None) == 0
    assert lib.dv_realtime_frame(32, 0, None, None, None, 64, None, None, None, 65, None, None, None) == 0
    # invalid sizes / missing buffers
    assert lib.dv_occupancy_max(4, None, None, None, 64, 0, None, None) == 1
    assert lib.dv_occupancy_max(4, fake, fake, fake, 64, -1, fake, None) == 1
    assert lib.dv_corner_rows(fake, fake, 2, 10, 65, fake, None) == 1  # row stride below 3
    assert lib.dv_integrate_table_fwd(fake, 10, 30, fake, fake, fake, 3, 5, fake, None) == 1  # channels % 4
    assert lib.dv_camera_rays(4, 4, 1.0, (C.c_float * 12)(), 10, 10, fake, fake, None) == 1  # past the image
    assert lib.dv_realtime_frame(32, 8, fake, fake, fake, 100, fake, fake, fake, 101, fake, fake, None) == 1  # N % 64
    assert lib.dv_realtime_frame(48, 8, fake, fake, fake, 64, fake, fake, fake, 65, fake, fake, None) == 1  # width
    assert lib.dv_mark_corner_rows(None, 0, None, 33, 33, 33, None, None) == 0
    assert lib.dv_mark_corner_rows(fake, 10, None, 0, 33, 33, fake, None) == 1  # empty grid
    assert lib.dv_mark_corner_rows(fake, 10, None, 33, 33, 33, None, None) == 1  # no byte map
    assert lib.dv_clear_marked_rows(fake, 30, 33, 33, 33, fake, None) == 1  # channels % 4
    assert lib.dv_clear_marked_rows(C.c_void_p(20), 32, 33, 33, 33, fake, None) == 1  # grid not 16-byte aligned
    assert lib.dv_clear_marked_rows(None, 32, 33, 33, 33, fake, None) == 1
    assert lib.dv_decode_tc_save_bytes(32, 32, 128) == 128 * 2 * (32 + 4 * 32)
    assert lib.dv_decode_tc_save_bytes(33, 32, 128) == -1
    # a layer table whose shapes do not fit the blob is rejected
    layers = (C.c_int * 20)()
    assert lib.dv_decode_fwd_tc(32, 32, 1, fake, 16, fake, 4, layers, 5, fake, None, 65, 65, 65, fake, fake, 256,
                                None, fake, fake, fake, 16, None, None) == 1
