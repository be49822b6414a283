"""The solver's integer-only double-float conversions equal the FP64 routines bit for bit.

The fused solver keeps x and b as double-float pairs (hi + lo in two floats) and converts every
fluid cell between FP64 and that form with integer operations (GB300's FP64 pipe runs at a small
fraction of its FP32 rate).  tests/csrc/df_check.cu compares both directions against the plain FP64
conversions on hashed inputs, ties included; it is compiled here against the library's own header.
"""
import ctypes as C
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def df_lib(tmp_path_factory, cuda):
    from mlpcg_gb300 import _build
    out = tmp_path_factory.mktemp("df") / "df_check.so"
    cmd = [_build._nvcc(), *_build.ARCH_FLAGS, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
           "-I", str(ROOT / "mlpcg_gb300" / "csrc"), "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "csrc" / "df_check.cu"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(str(out))
    lib.df_check.argtypes = [C.c_ulonglong, C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    lib.df_check.restype = C.c_int
    return lib


@pytest.mark.parametrize("seed", [1, 0x5EED])
def test_conversions_bit_identical_to_fp64(df_lib, seed):
    bad = (C.c_ulonglong * 2)()
    assert df_lib.df_check(1 << 26, seed, bad) == 0
    assert (bad[0], bad[1]) == (0, 0), (bad[0], bad[1])
