"""The voxel walks divide by a direction component through its correctly
rounded reciprocal (Markstein's theorem) instead of an IEEE division per
step.  This checks on the CPU that the two agree bit for bit over the domain
the walks use; the GPU traversal parity tests then check whole walks."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import pytest

SRC = Path(__file__).with_name("markstein_check.c")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    out = tmp_path_factory.mktemp("markstein") / "libmarkstein.so"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", str(SRC), "-o", str(out),
                    "-lm"], check=True)
    lib = ctypes.CDLL(str(out))
    lib.markstein_check.argtypes = [ctypes.c_longlong, ctypes.c_longlong]
    lib.markstein_check.restype = ctypes.c_longlong
    return lib


def test_reciprocal_division_matches_ieee(checker):
    assert checker.markstein_check(20_000_000, 1 << 21) == 0
