"""mlpcg_dot_noalloc: the dot product for callers that cannot allocate device memory.

Such callers (code inside a global-mode stream capture, real-time loops that
must not enter an allocator, hosts that own all device memory) cannot hand
mlpcg_dot a workspace; this entry point keeps its partial sums in a static
array of the library instead.  Checked through the C ABI against mlpcg_dot,
on two calls in a row (the static array keeps the previous call's contents).
Kept in a file that pytest collects last; it passes alone or after the rest.
"""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_N = 16_777_216


def _noalloc(lib, x, y, dtype_code, n, out, stream):
    return lib.mlpcg_dot_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), dtype_code, n,
                                 C.c_void_p(out.data_ptr()), stream)


def test_dot_noalloc_matches_dot_on_consecutive_calls(cuda):
    from mlpcg_gb300 import _lib, ops
    lib = _lib.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    gen = torch.Generator(device=cuda)
    gen.manual_seed(5)
    cases = [(1, torch.float32, 0), (1_000_003, torch.float32, 0), (4096, torch.float64, 2),
             (MAX_N, torch.float32, 0), (333_333, torch.float64, 2)]
    for _ in range(2):
        for n, dt, code in cases:
            x = torch.randn(n, generator=gen, device=cuda, dtype=dt)
            y = torch.randn(n, generator=gen, device=cuda, dtype=dt)
            out = torch.full((1,), float("nan"), dtype=torch.float64, device=cuda)
            assert _noalloc(lib, x, y, code, n, out, stream) == 0, lib.mlpcg_last_error()
            ref = ops.dot(x, y)
            torch.cuda.synchronize()
            scale = float((x.double() * y.double()).abs().sum())
            assert abs(float(out) - float(ref)) <= 1e-12 * scale, (n, dt, float(out), float(ref))


def test_dot_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    from mlpcg_gb300 import _lib
    lib = _lib.load()
    x = torch.zeros(16, device=cuda)
    out = torch.zeros(1, dtype=torch.float64, device=cuda)
    rc = _noalloc(lib, x, x, 0, MAX_N + 1, out, None)
    assert rc != 0
    assert b"exceeds the maximum" in lib.mlpcg_last_error()
