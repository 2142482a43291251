"""oracle -- TEST INFRASTRUCTURE ONLY: the CPU parity oracle of pyop2_gb300.

A sequential CPU restatement of PyOP2's par_loop backend, sparsity builder
and Mat insertion (see oracle/op2.py and oracle/sparsity.c for the reference
file:line each part follows).  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg use it -- as the checker or the timed CPU
baseline, never as part of the product.

Parity pinning: the reference (PETSc + loopy + mpi4py) cannot be imported or
built here, so the oracle is pinned against the golden values the
reference's own unit tests assert (tests/test_oracle_golden.py).
"""
