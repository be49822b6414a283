"""CPU oracle of the MLPCG hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy (FP64) and torch-CPU, the reference
algorithm of the neural-preconditioned CG Poisson solve of kai-lan/MLPCG:

* ``ops``       -- the three extension ops (sm_block_3d, sm_block_trans_3d,
                   sm_linear_3d), their gradients, avg-pool / trilinear transfer;
* ``model``     -- SmallSMModelDn3D.forward composed from those ops;
* ``laplacian`` -- the FP64 assembled 7-point mixed-boundary matrix and an
                   FP64 CG solved to 1e-12;
* ``cg``        -- the reference's npcg / npcg_flex / npsd iterations;
* ``cpu_path``  -- the reference's CPU path (torch-CPU Conv3d + unfold blocks,
                   torch-CPU CG), timed as the CPU baseline.
* ``amg``       -- the reference's host AMG comparator (smoothed-aggregation
                   AMG with SPAI-0 relaxation inside FP64 CG, as its AMGCL
                   shim configures it), restated in C++ (``amg.cpp``, built
                   with g++ / OpenMP) from the published methods: AMGCL is
                   an un-vendored submodule, so this comparator's iteration
                   counts are not pinned to AMGCL's.

Parity is pinned: ``tests/golden/make_golden.py`` imports the reference's own
Python modules (sm_model_3d_py.py, model.py, lib/discrete_laplacian.py,
cg_tests.py) and records their outputs as fixtures, and
``tests/test_oracle_golden.py`` checks this oracle against them.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU
baseline leg and its ``--impl reference`` arm) may import this package, and
only as the checker or the timed CPU baseline.  The product
(``mlpcg_gb300``) never imports it and has no CPU fallback.
"""
