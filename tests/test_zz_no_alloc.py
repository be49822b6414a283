"""mlpcg_dot_noalloc: the dot product for callers that cannot allocate device memory.

Some callers of this library never allocate on the GPU themselves: real-time
loops that must not enter an allocator (its latency is unbounded), and host
runtimes or plug-in hosts that own all device memory through their own arena
and hand a library only the buffers of its inputs and outputs.  They cannot
hand mlpcg_dot a workspace, so this entry point keeps its partial sums in a
static array of the library instead.

Checked through the C ABI against an FP64 reduction computed by torch on the
same inputs (not against mlpcg_dot, which runs the same kernels), for FP32,
FP64 and BF16 vectors, on two rounds of calls in a row (the static array keeps
the previous call's contents).  Kept in a file that pytest collects last; it
passes alone or after the rest.
"""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_N = 16_777_216
F32, BF16, F64 = 0, 1, 2


def _noalloc(lib, x, y, dtype_code, n, out, stream):
    return lib.mlpcg_dot_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), dtype_code, n,
                                 C.c_void_p(out.data_ptr()), stream)


def test_dot_noalloc_matches_fp64_reduction_on_consecutive_calls(cuda):
    from mlpcg_gb300 import _lib
    lib = _lib.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    gen = torch.Generator(device=cuda)
    gen.manual_seed(5)
    cases = [(1, torch.float32, F32), (1_000_003, torch.float32, F32), (4096, torch.float64, F64),
             (MAX_N, torch.float32, F32), (333_333, torch.float64, F64), (777_777, torch.bfloat16, BF16),
             (MAX_N, torch.bfloat16, BF16)]
    for _ in range(2):
        for n, dt, code in cases:
            x = torch.randn(n, generator=gen, device=cuda, dtype=torch.float32).to(dt)
            y = torch.randn(n, generator=gen, device=cuda, dtype=torch.float32).to(dt)
            out = torch.full((1,), float("nan"), dtype=torch.float64, device=cuda)
            assert _noalloc(lib, x, y, code, n, out, stream) == 0, lib.mlpcg_last_error()
            prod = x.double() * y.double()  # exact for FP32 and BF16 inputs
            ref = float(prod.sum())
            scale = float(prod.abs().sum())
            got = float(out)
            # both sides sum FP64 products in FP64, in different orders
            assert abs(got - ref) <= 1e-12 * scale, (n, dt, got, ref)


def test_dot_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    from mlpcg_gb300 import _lib
    lib = _lib.load()
    x = torch.zeros(16, device=cuda)
    out = torch.zeros(1, dtype=torch.float64, device=cuda)
    rc = _noalloc(lib, x, x, F32, MAX_N + 1, out, None)
    assert rc != 0
    assert b"exceeds the maximum" in lib.mlpcg_last_error()
