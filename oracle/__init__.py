"""CPU oracle for the BETSE electrodiffusion step -- TEST INFRASTRUCTURE ONLY.

This package is a NumPy restatement of BETSE's per-timestep electrodiffusion
step (``betse/science/sim.py:1132-1390`` and the helpers it calls), written
with CSR segment sums instead of BETSE's dense ``M_sum_mems`` /
``M_divmap_mem2ecm`` matrices so that it scales past a few thousand cells.

It is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it. The CUDA path in ``betse_gb300`` never calls into it and has no CPU
fallback.

Parity is pinned: ``tests/test_oracle_golden.py`` checks this restatement
against fixtures produced by running BETSE's own ``Simulator`` on seeded
clusters (``tests/golden/make_golden.py``).
"""
from .step import (electroflux, pump_nakatp, step, run, init_vm,  # noqa: F401
                   init_fields, seg_sum, env_scatter, OracleState)
from .fields import (gradient, diff, divergence, integrator,  # noqa: F401
                     gaussian_filter, make_laplacian_inverse, hh_decomp)
