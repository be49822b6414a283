"""The host-side AMG comparator (oracle/amg.cpp) -- TEST AND BASELINE INFRASTRUCTURE ONLY.

The reference reports its network-preconditioned solves beside an AMGCL solve on the host
(``cg_tests.py:343-346`` calling ``pyamgcl.solve``, ``cxx_src/pyamgcl.cpp:9-16``,
``cxx_src/lib/AMGCLSolver.h:58-128``: smoothed-aggregation AMG with SPAI-0 relaxation inside an
FP64 CG, x0 = 0, tol = max(tol, atol / |b|), returning iterations, setup + solve time and the
residual).  AMGCL is an un-vendored submodule with no recoverable commit, so ``amg.cpp`` restates
the published methods (its header gives them and their parameters): a comparator whose iteration
counts are not pinned to AMGCL's.

``solve(A, b, ...)`` mirrors ``cg_tests.AMGCL``'s return (x, (iterations, seconds, residual)) plus a
dict of details; ``python -m oracle.amg --size N --seed S --spheres K`` solves a synthetic scene's
FP64 system and prints one JSON line (``bench.py`` runs it in a child process, so that the
comparator's time and memory stay out of the GPU measurement).  The library is compiled with g++
and OpenMP on first use, into ``oracle/_build/``.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "amg.cpp"
OUT_DIR = HERE / "_build"

_lib = None


def library_path() -> Path:
    return OUT_DIR / f"libmlpcg_amg_{platform.machine()}.so"


def _compile(out: Path) -> None:
    OUT_DIR.mkdir(exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=OUT_DIR, suffix=".so")
    os.close(fd)
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", str(SRC), "-o", tmp]
    try:
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        os.replace(tmp, out)
    except subprocess.CalledProcessError as e:
        Path(tmp).unlink(missing_ok=True)
        raise RuntimeError(f"building the AMG comparator failed: {' '.join(cmd)}\n{e.stderr}") from e


def load():
    """The compiled comparator (built when missing or older than its source)."""
    global _lib
    if _lib is not None:
        return _lib
    out = library_path()
    if not out.exists() or out.stat().st_mtime < SRC.stat().st_mtime:
        _compile(out)
    try:
        lib = C.CDLL(str(out))
    except OSError:  # a library built for another machine: rebuild once
        _compile(out)
        lib = C.CDLL(str(out))
    i64p, i32p, f64p = (np.ctypeslib.ndpointer(t, flags="C_CONTIGUOUS") for t in (np.int64, np.int32, np.float64))
    lib.amg_cg_solve.argtypes = [C.c_int64, i64p, i32p, f64p, f64p, f64p, C.c_double, C.c_double, C.c_int,
                                 C.c_int, f64p]
    lib.amg_cg_solve.restype = C.c_int
    lib.amg_apply.argtypes = [C.c_int64, i64p, i32p, f64p, f64p, f64p, C.POINTER(C.c_int)]
    lib.amg_apply.restype = C.c_int
    lib.amg_fluid_matrix.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.POINTER(C.c_int64),
                                     C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.amg_fluid_matrix.restype = C.c_int
    _lib = lib
    return lib


def _csr_arrays(A):
    A = A.tocsr()
    if A.shape[0] != A.shape[1]:
        raise ValueError("A must be square")
    return (A.shape[0], np.ascontiguousarray(A.indptr, dtype=np.int64),
            np.ascontiguousarray(A.indices, dtype=np.int32), np.ascontiguousarray(A.data, dtype=np.float64))


def solve(A, b, tol=1e-10, atol=1e-10, max_it=100, threads=0):
    """x, (iterations, setup + solve seconds, true relative residual), details -- the return of the
    reference's AMGCL shim (cg_tests.py:343-346) with the details added."""
    n, ptr, col, val = _csr_arrays(A)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if b.shape != (n,):
        raise ValueError("b must have one value per row of A")
    x = np.zeros(n)
    stats = np.zeros(8)
    rc = load().amg_cg_solve(n, ptr, col, val, b, x, float(tol), float(atol), int(max_it), int(threads), stats)
    if rc != 0:
        raise ValueError("amg_cg_solve: bad arguments")
    it, setup_s, solve_s, res, levels, opc, coarsest, used = stats
    details = {"iterations": int(it), "setup_s": setup_s, "solve_s": solve_s, "rel_res": res,
               "levels": int(levels), "operator_complexity": opc, "coarsest_unknowns": int(coarsest),
               "threads": int(used)}
    return x, (int(it), setup_s + solve_s, res), details


def apply_preconditioner(A, r):
    """z = B r, one V-cycle of the hierarchy of A, and the hierarchy's depth."""
    n, ptr, col, val = _csr_arrays(A)
    r = np.ascontiguousarray(r, dtype=np.float64)
    z = np.zeros(n)
    levels = C.c_int(0)
    if load().amg_apply(n, ptr, col, val, r, z, C.byref(levels)) != 0:
        raise ValueError("amg_apply: bad arguments")
    return z, levels.value


def assemble_csr(flags):
    """(A, fluid_cells): the FP64 matrix of ``oracle.laplacian.assemble`` (the same rows, columns
    and values) built by ``amg_fluid_matrix`` in two passes, directly in CSR form."""
    import scipy.sparse as sp
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    n1, n2, n3 = flags.shape
    lib = load()
    nf, nnz = C.c_int64(0), C.c_int64(0)
    fptr = flags.ctypes.data_as(C.c_void_p)
    if lib.amg_fluid_matrix(n1, n2, n3, fptr, C.byref(nf), C.byref(nnz), None, None, None, None) != 0:
        raise ValueError("amg_fluid_matrix: bad arguments")
    fluid = np.empty(nf.value, dtype=np.int64)
    ptr = np.empty(nf.value + 1, dtype=np.int64)
    col = np.empty(nnz.value, dtype=np.int32)
    val = np.empty(nnz.value)
    if lib.amg_fluid_matrix(n1, n2, n3, fptr, C.byref(nf), C.byref(nnz), fluid.ctypes.data_as(C.c_void_p),
                            ptr.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
                            val.ctypes.data_as(C.c_void_p)) != 0:
        raise ValueError("amg_fluid_matrix: inconsistent sizes")
    return sp.csr_matrix((val, col, ptr), shape=(nf.value, nf.value)), fluid


def main(argv=None):
    import argparse
    import json
    import sys
    import time
    sys.path.insert(0, str(HERE.parent))
    from mlpcg_gb300.scenes import make_scene
    ap = argparse.ArgumentParser(description="AMG-preconditioned CG on a synthetic scene (host cores)")
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--spheres", type=int, default=6)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--max-it", type=int, default=1000)
    ap.add_argument("--threads", type=int, default=0)
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    load()
    scene = make_scene(a.size, a.seed, a.spheres)
    A, fluid = assemble_csr(scene.flags)
    b = scene.rhs.ravel()[fluid]
    prep = time.perf_counter() - t0
    _, (it, secs, res), d = solve(A, b, tol=a.tol, atol=1e-20, max_it=a.max_it, threads=a.threads)
    print(json.dumps({"value": round(secs * 1e3, 1), "unit": "ms", "cores": d["threads"], "kind": "port",
                      "method": "smoothed-aggregation AMG (SPAI-0 relaxation, V-cycle) + FP64 CG, x0 = 0",
                      "iterations": it, "rel_res": res, "setup_ms": round(d["setup_s"] * 1e3, 1),
                      "solve_ms": round(d["solve_s"] * 1e3, 1), "levels": d["levels"],
                      "operator_complexity": round(d["operator_complexity"], 3),
                      "unknowns": int(b.size), "host_cpus": os.cpu_count(),
                      "matrix_assembly_s": round(prep, 2)}))


if __name__ == "__main__":
    main()
