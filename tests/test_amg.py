"""The host AMG comparator (oracle/amg.cpp: smoothed-aggregation AMG + SPAI-0 inside FP64 CG, the
method of the reference's AMGCL comparator, cxx_src/lib/AMGCLSolver.h:58-128) on CPU: its matrix
equals the oracle's, it solves to the tolerance asked, its V-cycle is symmetric positive definite
(so plain CG applies), and its iteration count stays flat as the grid grows."""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import amg
from oracle import laplacian as olap


def _scene(shape, seed, spheres=3):
    from mlpcg_gb300.scenes import make_scene
    return make_scene(shape, seed, spheres)


@pytest.mark.parametrize("shape,seed", [((16, 16, 16), 3), ((7, 13, 29), 1), ((40, 24, 33), 5), ((1, 5, 3), 2)])
def test_matrix_equals_the_oracle_assembly(shape, seed):
    flags = _scene(shape, seed).flags
    A0, f0 = olap.assemble(flags)
    A1, f1 = amg.assemble_csr(flags)
    assert np.array_equal(f0, f1)
    assert np.array_equal(A0.indptr, A1.indptr) and np.array_equal(A0.indices, A1.indices)
    assert np.array_equal(A0.data, A1.data)


def test_matrix_with_every_flag_value():
    """Random boundary / solid / fluid / air cells, including fluid cells with no fluid or air
    neighbour (a zero row)."""
    flags = np.random.default_rng(4).integers(0, 4, (11, 9, 14)).astype(np.uint8)
    A0, f0 = olap.assemble(flags)
    A1, f1 = amg.assemble_csr(flags)
    assert np.array_equal(f0, f1) and (A0 != A1).nnz == 0 and np.array_equal(A0.indices, A1.indices)


def test_solves_to_the_tolerance_and_matches_a_direct_solve():
    sc = _scene((32, 32, 32), 6)
    A, fluid = amg.assemble_csr(sc.flags)
    b = sc.rhs.ravel()[fluid]
    x, (it, secs, res), d = amg.solve(A, b, tol=1e-10, atol=1e-30, max_it=200)
    assert res < 1e-10 and res == pytest.approx(np.linalg.norm(b - A @ x) / np.linalg.norm(b), rel=1e-6)
    xd = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-7
    _, plain_it = olap.cg_fp64(A, b, tol=1e-10)
    assert it < plain_it / 4, (it, plain_it)
    assert d["levels"] >= 2 and 1.0 < d["operator_complexity"] < 2.5 and secs > 0


def test_vcycle_is_symmetric_positive_definite():
    sc = _scene((24, 20, 28), 9)
    A, _ = amg.assemble_csr(sc.flags)
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal(A.shape[0]), rng.standard_normal(A.shape[0])
    Bu, levels = amg.apply_preconditioner(A, u)
    Bv, _ = amg.apply_preconditioner(A, v)
    assert levels >= 2
    assert abs(Bu @ v - u @ Bv) <= 1e-12 * abs(Bu @ v)
    assert u @ Bu > 0 and v @ Bv > 0


def test_iterations_stay_flat_as_the_grid_grows():
    its = []
    for n in (16, 32, 48):
        sc = _scene(n, 3)
        A, fluid = amg.assemble_csr(sc.flags)
        _, (it, _, res), _ = amg.solve(A, sc.rhs.ravel()[fluid], tol=1e-8, atol=1e-30, max_it=200)
        assert res < 1e-8
        its.append(it)
    assert max(its) <= 16 and max(its) - min(its) <= 4, its


def test_stopping_rule_and_edge_cases():
    """tol = max(tol, atol / |b|) as the reference's shim sets it (AMGCLSolver.h:67); a zero rhs
    takes no iteration; a size mismatch is refused."""
    sc = _scene((16, 16, 16), 2)
    A, fluid = amg.assemble_csr(sc.flags)
    b = sc.rhs.ravel()[fluid]
    nb = np.linalg.norm(b)
    _, (it_tight, _, _), _ = amg.solve(A, b, tol=1e-10, atol=1e-30)
    _, (it_atol, _, res), _ = amg.solve(A, b, tol=1e-10, atol=1e-3 * nb)
    assert it_atol < it_tight and res < 1e-3
    x0, (it0, _, r0), _ = amg.solve(A, np.zeros_like(b))
    assert it0 == 0 and r0 == 0.0 and not x0.any()
    with pytest.raises(ValueError):
        amg.solve(A, b[:-1])


def test_repeats_bit_for_bit_with_the_same_thread_count():
    """Fixed-order reductions and a deterministic parallel transpose: the same solution bits on
    every run with a given thread count; one thread and four threads agree to the tolerance."""
    sc = _scene((32, 28, 36), 8)
    A, fluid = amg.assemble_csr(sc.flags)
    b = sc.rhs.ravel()[fluid]
    x4 = [amg.solve(A, b, tol=1e-9, atol=1e-30, threads=4)[0] for _ in range(3)]
    assert all(np.array_equal(x4[0], x) for x in x4[1:])
    x1 = amg.solve(A, b, tol=1e-9, atol=1e-30, threads=1)[0]
    amg.solve(A, b, threads=os.cpu_count() or 1)  # leave the process at its default thread count
    assert np.linalg.norm(x1 - x4[0]) / np.linalg.norm(x1) < 1e-7
