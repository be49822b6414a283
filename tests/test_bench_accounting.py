"""bench.py's byte and launch accounting on stand-in plans (CPU): the per-cell counts of one
fused iteration, derived by hand from the kernel sequence of each network, and the launch counters
running for every network kind."""
from types import SimpleNamespace

import pytest

import bench

N0 = 64 ** 3


def _plan(kind, levels=1, masked=False, swap=False, cluster=-1):
    return SimpleNamespace(levels=levels, kind=kind, spd=kind != 0, masked=masked, swap=swap, layout="classed",
                           level_info=lambda l: (0, True, False),
                           coarse_cluster=lambda: (cluster, 16 if cluster > 0 else 0))


def test_smallsm_iteration_bytes_dense():
    # level 0 with 54 B/cell of BF16 coefficient planes:
    #   pre 54 + r 4 + y 2 + pooled 0.25; prolongation pass coarse 0.25 + u 4;
    #   post 54 + u 4 + y 2 + z 4 + fluid mask 1; coarsest level: 54 + x 2 + out 2;
    #   npsd vectors 12 + 16 + 18 + 24
    got = bench.iteration_bytes(_plan(0), N0, [None, None], method="npsd")
    assert got == pytest.approx(N0 * (60.25 + 4.25 + 65 + 70) + N0 / 8 * 58)
    masked = bench.iteration_bytes(_plan(0, masked=True), N0, [None, None], method="npsd")
    assert masked - got == pytest.approx(2 * N0)       # the block mask, read by both level-0 blocks
    swapped = bench.iteration_bytes(_plan(0, swap=True), N0, [None, None], method="npsd")
    assert swapped == pytest.approx(got)                # y read by the pass instead of the block
    fused = bench.iteration_bytes(_plan(0), N0, [None, None], method="npsd", fused_dots=True)
    assert got - fused == pytest.approx(4 * N0)         # z . Ap in the post-block: z not read again


def test_spd_iteration_bytes_dense():
    # SmallSPDSMModelDn3D, npcg: pre 54 + 6.25; pass coarse 0.25 + y 2 + u 4; transposed block
    # 54 + u 4 + z 4 + mask 1; coarsest l and l_t 54 + 54 + 8; vectors 8 + 17 + 24
    got = bench.iteration_bytes(_plan(1), N0, [None, None], [None, None], method="npcg")
    assert got == pytest.approx(N0 * (60.25 + 6.25 + 63 + 49) + N0 / 8 * 116)
    # SPDSMModelDn3D: V pre 60.25, V pass 4.25, V post 54 + 4 + 2 + 4 (v0 FP32), V^T pre 54 + 4.25,
    # V^T pass 0.25 + 4 + 4, V^T post 54 + 4 + 5
    full = bench.iteration_bytes(_plan(2), N0, [None, None], [None, None], method="npcg")
    assert full == pytest.approx(N0 * (60.25 + 4.25 + 64 + 58.25 + 8.25 + 63 + 49) + N0 / 8 * 116)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_launch_counters_run(kind):
    p = _plan(kind, levels=5)
    assert bench.precond_launches(p) > 0 and bench.setup_launches(p) > 0
    mixed = [1000, 500, 100, 50, 10, 4]
    assert bench.iteration_bytes(p, 256 ** 3, mixed, mixed if kind else None) > 0


def test_launch_count_with_the_coarse_cluster():
    # SmallSMModelDn3D, 5 tiled levels: 5 pre-blocks, the coarsest block, the level-0 prolongation
    # pass + post-block and 4 post-blocks = 12 launches; with levels 3..5 in one cluster launch:
    # pre 0-2, the cluster, post 2, post 1, prolongation + post 0 = 8
    assert bench.precond_launches(_plan(0, levels=5)) == 12
    assert bench.precond_launches(_plan(0, levels=5, cluster=3)) == 8
