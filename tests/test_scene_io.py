"""Simulator scene files (flags, matrix, rhs) read and written like the reference's
lib/read_data.py / lib/write_data.py; pinned to files written by the reference's own
writers and to what its readers return for them (tests/golden/make_golden.py)."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

from mlpcg_gb300 import scene_io
from mlpcg_gb300.laplacian import csr_from_flags

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def ref():
    return dict(np.load(GOLDEN / "scene_files_8.npz"))


def test_read_reference_files(ref):
    d = GOLDEN / "scene_8"
    flags = scene_io.read_flags(d / "flags_1.bin")
    np.testing.assert_array_equal(flags, ref["flags"])
    A = scene_io.read_matrix(d / "A_1.bin")
    A.sort_indices()
    np.testing.assert_array_equal(A.indptr, ref["A_indptr"])
    np.testing.assert_array_equal(A.indices, ref["A_indices"])
    np.testing.assert_array_equal(A.data, ref["A_data"])
    rhs = scene_io.load_vector(d / "div_v_star_1.bin")
    np.testing.assert_array_equal(rhs, ref["rhs"])
    np.testing.assert_array_equal(scene_io.compressed_vec(rhs, flags), ref["rhs_fluid"])


def test_load_frame_matches_reference_compression(ref):
    flags, rhs, A = scene_io.load_frame(GOLDEN / "scene_8", 1, (8, 8, 8))
    assert flags.dtype == np.uint8 and flags.shape == (8, 8, 8)
    A.sort_indices()
    np.testing.assert_array_equal(A.indptr, ref["Ac_indptr"])
    np.testing.assert_array_equal(A.indices, ref["Ac_indices"])
    np.testing.assert_array_equal(A.data, ref["Ac_data"])
    np.testing.assert_array_equal(rhs, ref["rhs_fluid"])


def test_file_matrix_is_the_flags_operator(ref):
    """The compressed file matrix is the fluid block of this package's operator from the same flags."""
    flags = ref["flags"].reshape(8, 8, 8).astype(np.uint8)
    _, _, A = scene_io.load_frame(GOLDEN / "scene_8", 1, (8, 8, 8))
    ours, fluid = csr_from_flags(flags, device="cpu")
    ours = ours.to_dense().numpy()
    fluid = np.asarray(fluid.cpu() if hasattr(fluid, "cpu") else fluid)
    assert A.shape[0] >= ours.shape[0]
    # rows the reference keeps beyond the fluid cells are decoupled (its lap_with_bc quirk)
    keep = np.flatnonzero(np.asarray((A != 0).sum(axis=1)).ravel() > 0)
    Af = A.toarray()
    full = np.flatnonzero(scene_io.read_matrix(GOLDEN / "scene_8" / "A_1.bin").getnnz(1) > 0)
    pos = {c: i for i, c in enumerate(full)}
    rows = [pos[c] for c in fluid]
    np.testing.assert_allclose(Af[np.ix_(rows, rows)], ours, rtol=0, atol=0)
    assert len(keep) == A.shape[0]


def test_writers_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    flags = rng.integers(0, 4, size=5 * 6 * 7)
    scene_io.write_flags(tmp_path / "flags_3.bin", flags)
    np.testing.assert_array_equal(scene_io.read_flags(tmp_path / "flags_3.bin"), flags)
    v = rng.standard_normal(91)
    scene_io.write_vector(tmp_path / "v.bin", v)
    np.testing.assert_array_equal(scene_io.load_vector(tmp_path / "v.bin"), v)
    A = sp.random(40, 40, density=0.1, random_state=1, format="csr")
    scene_io.write_matrix(A, tmp_path / "A.bin")
    B = scene_io.read_matrix(tmp_path / "A.bin")
    assert (abs(A - B)).max() == 0 and B.shape == A.shape
    Bc = scene_io.read_matrix(tmp_path / "A.bin", sparse_type="csc")
    assert sp.isspmatrix_csc(Bc) and (abs(A - Bc)).max() == 0
    Bf = scene_io.read_matrix(tmp_path / "A.bin", sparse_type="coo")
    assert (abs(A - Bf.tocsr())).max() == 0


def test_expand_and_images():
    flags = np.array([[[0, 2, 3], [2, 1, 2]]])
    b = np.array([1.0, 2.0, 3.0])
    g = scene_io.expand_vec(b, flags)
    np.testing.assert_array_equal(g, [0, 1, 0, 2, 0, 3])
    np.testing.assert_array_equal(scene_io.compressed_vec(g, flags), b)
    img = scene_io.convert_to_binary_images(flags, 3)
    np.testing.assert_array_equal(img[0].ravel(), [0, 0, 1, 0, 0, 0])
    np.testing.assert_array_equal(img[1].ravel(), [0, 1, 0, 1, 0, 1])
    np.testing.assert_array_equal(img[2].ravel(), [0, 1, 1, 1, 0, 1])
    assert scene_io.convert_to_binary_images(flags, 1).shape == (1,) + flags.shape
    assert scene_io.convert_to_binary_images(flags, 2).shape == (2,) + flags.shape


@pytest.mark.gpu
def test_solve_file_scene_on_gpu(cuda):
    """A frame loaded from the simulator files solves with the fused solver; the FP64 residual
    against the file's own matrix meets the tolerance."""
    import torch
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    from mlpcg_gb300.solver import FusedSolver
    flags, rhs, A = scene_io.load_frame(GOLDEN / "scene_8", 1, (8, 8, 8))
    torch.manual_seed(0)
    model = SmallSMModelDn3D(2, 3, "trilinear").to(cuda)
    with torch.no_grad():
        for p in model.parameters():
            p.mul_(0.0)
        model.pre[0].bias[13] += 1.0
        model.c0[0].bias[0] += 1.0
    solver = FusedSolver(model, torch.as_tensor(flags, device=cuda), method="npcg", max_it=200, tol=1e-8,
                         storage=torch.float32)
    b_h = torch.from_numpy(rhs.copy()).pin_memory()
    x_h = torch.empty(rhs.size, dtype=torch.float64).pin_memory()
    solver.solve_host(torch.from_numpy(flags).pin_memory(), b_h, x_h)
    res = solver.result()
    torch.cuda.synchronize()
    assert res.status == "converged"
    full = scene_io.read_matrix(GOLDEN / "scene_8" / "A_1.bin")
    keep = np.flatnonzero(full.getnnz(1) > 0)
    fluid = np.flatnonzero(flags.ravel() == scene_io.FLUID)
    rows = np.searchsorted(keep, fluid)
    Af = A[rows][:, rows]
    x = x_h.numpy()
    assert np.linalg.norm(rhs - Af @ x) / np.linalg.norm(rhs) < 1e-7
