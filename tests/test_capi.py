"""The C-ABI library builds, loads without a GPU, exports every declared symbol and
rejects bad arguments before touching the device (CPU only)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(mlpcg_[a-z0-9_]+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    from mlpcg_gb300 import _lib
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    import subprocess
    from mlpcg_gb300 import _build
    declared = _declared()
    assert len(declared) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", str(_build.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (mlpcg_[a-z0-9_]+)", out))
    assert declared <= exported, sorted(declared - exported)
    # nothing but the ABI is exported
    assert exported == declared, sorted(exported - declared)
    for name in declared:
        getattr(lib, name)


def test_ctypes_prototypes_cover_header(lib):
    from mlpcg_gb300 import _lib
    assert set(_lib.exported_symbols()) == _declared()


def test_abi_version(lib):
    assert lib.mlpcg_abi_version() >= 1


def test_null_pointer_rejected_without_device(lib):
    from mlpcg_gb300._lib import MLPCGError, call
    with pytest.raises(MLPCGError, match="image must not be NULL"):
        call("mlpcg_stencil_gen", None, 0, 8, 8, 8, None, None, None, 0, 512, None)
    assert b"NULL" in lib.mlpcg_last_error()


def test_bad_shapes_rejected(lib):
    from mlpcg_gb300._lib import MLPCGError, call
    dummy = C.c_void_p(16)  # never dereferenced: validation fails first
    with pytest.raises(MLPCGError, match="grid sizes"):
        call("mlpcg_stencil_gen", dummy, 0, 0, 8, 8, dummy, dummy, dummy, 0, 512, None)
    with pytest.raises(MLPCGError, match="plane_stride"):
        call("mlpcg_stencil_gen", dummy, 0, 8, 8, 8, dummy, dummy, dummy, 0, 100, None)
    with pytest.raises(MLPCGError, match="even"):
        call("mlpcg_avg_pool2", dummy, dummy, 0, 1, 7, 8, 8, None)
    with pytest.raises(MLPCGError, match="workspace too small"):
        call("mlpcg_sm_block_3d_forward", dummy, 0, dummy, 0, dummy, dummy, dummy, 1, 8, 8, 8, 0,
             dummy, 16, None)


def test_workspace_queries(lib):
    from mlpcg_gb300._lib import query
    assert query("mlpcg_sm_block_3d_workspace", 8, 8, 8) >= 27 * 512 * 4
    assert query("mlpcg_sm_linear_3d_workspace", 8, 8, 8) > 0
    assert query("mlpcg_dot_workspace", 1 << 20) >= 8


def test_solver_bind_rejects_misaligned_vectors(lib):
    """Binding checks the caller's pointers before any kernel reads them (no device work)."""
    import ctypes as C2
    from mlpcg_gb300._lib import MLPCGError, call
    plan, solver = C2.c_void_p(), C2.c_void_p()
    call("mlpcg_precond_create", 16, 16, 16, 2, 1, 1, 0, 0, 1, C2.byref(plan))
    try:
        call("mlpcg_solver_create", 16, 16, 16, plan, 0, 10, C2.c_double(1e-6), 25, C2.byref(solver))
        try:
            nbytes = lib.mlpcg_solver_workspace(solver)
            ws = C2.c_void_p(1 << 20)   # 256-byte aligned, never dereferenced
            good = C2.c_void_p(1 << 21)
            with pytest.raises(MLPCGError, match="16-byte"):
                call("mlpcg_solver_bind", solver, ws, nbytes, good, C2.c_void_p((1 << 21) + 8), good)
            with pytest.raises(MLPCGError, match="4-byte"):
                call("mlpcg_solver_bind", solver, ws, nbytes, C2.c_void_p((1 << 21) + 1), good, good)
        finally:
            lib.mlpcg_solver_destroy(solver)
    finally:
        lib.mlpcg_precond_destroy(plan)


def test_precond_apply_rejects_misaligned_vectors(lib):
    """Both application entry points check r (16 bytes) and z (32 bytes) before the plan's state
    and before any kernel reads them (no device work)."""
    from mlpcg_gb300._lib import MLPCGError, call
    plan = C.c_void_p()
    call("mlpcg_precond_create", 16, 16, 16, 2, 1, 1, 0, 0, 1, C.byref(plan))
    try:
        good, st = C.c_void_p(1 << 21), C.c_void_p(0)
        for name, lead in (("mlpcg_precond_apply", ()), ("mlpcg_precond_apply_stages", (0, 0))):
            with pytest.raises(MLPCGError, match="16-byte"):
                call(name, plan, *lead, C.c_void_p((1 << 21) + 4), None, good, st)
            with pytest.raises(MLPCGError, match="32-byte"):
                call(name, plan, *lead, good, None, C.c_void_p((1 << 21) + 16), st)
            with pytest.raises(MLPCGError, match="not set up"):  # aligned: the next check fires
                call(name, plan, *lead, good, None, good, st)
    finally:
        lib.mlpcg_precond_destroy(plan)



def test_python_constructors_refuse_unknown_options():
    """Unknown solver methods, coefficient layouts and storage dtypes are refused up front with a
    ValueError naming the option (no device work)."""
    import torch
    from mlpcg_gb300.precond import PrecondPlan
    from mlpcg_gb300.solver import FusedSolver
    with pytest.raises(ValueError, match="method"):
        FusedSolver(None, torch.zeros((4, 4, 4), dtype=torch.uint8), method="cg")
    img = torch.zeros((3, 4, 4, 4))
    with pytest.raises(ValueError, match="layout"):
        PrecondPlan(None, img, layout="sparse")
    with pytest.raises(ValueError, match="storage"):
        PrecondPlan(None, img, storage=torch.float16)
