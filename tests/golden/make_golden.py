"""Writes tests/golden/golden.npz: outputs of the oracle (oracle/op2.py, the
CPU restatement of the reference's sequential backend, itself pinned by the
reference's unit-test values) on small seeded instances of the benchmark
configurations.  The fixtures freeze those outputs, so that the oracle
cannot drift unnoticed and the GPU can be compared with stored values.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def compute(op2):
    """The fixture arrays, computed with `op2` (the oracle or the GPU
    package): name -> ndarray."""
    from pyop2_gb300 import workloads as W
    out = {}
    # configuration 1: 2D P1 action + area, 16^2 x 2 triangles
    p = W.build_p1_2d(op2, n=16, seed=3)
    p["run"]()
    out["c1_y"] = np.array(p["y"].data_ro)
    out["c1_area"] = np.array(p["area"].data_ro)
    # configuration 2: P1 tet action, 6^3 x 6 tets, permuted numbering
    q = W.build_p1_3d(op2, n=6, permute=True, seed=4)
    q["run"]()
    out["c2a_y"] = np.array(q["y"].data_ro)
    # sparsity and CSR assembly on the same mesh
    sp = op2.Sparsity((q["verts"] ** 1, q["verts"] ** 1), [(q["c2v"], q["c2v"], None)])
    A = op2.Mat(sp)
    op2.par_loop(op2.Kernel(W.P1_3D_LAPLACE_MATRIX, "p1_laplace_3d_mat"), q["cells"],
                 A(op2.INC, (q["c2v"], q["c2v"])), q["X"](op2.READ, q["c2v"]))
    A.assemble()
    if hasattr(sp, "csr"):
        rp, ci = sp.csr()
        vals = A.csr()[2]
    else:
        rp, ci, vals = sp.rowptr, sp.colidx, A.values_bcsr
    out["c2b_rowptr"] = np.asarray(rp, dtype=np.int64)
    out["c2b_colidx"] = np.asarray(ci, dtype=np.int32)
    out["c2b_values"] = np.asarray(vals, dtype=np.float64).reshape(-1)
    # configuration 5: prism elasticity action, 3^2 x 2 x 4 prisms, 8 RHS
    r = W.build_prisms(op2, n=3, layers=5, seed=5)
    ds = op2.DataSet(r["nodes"], (r["nrhs"], 3))
    u, y = op2.Dat(ds, r["u"]), op2.Dat(ds)
    op2.par_loop(op2.Kernel(W.PRISM_ELASTICITY_ACTION, "prism_elasticity"), r["cells"],
                 y(op2.INC, r["c2n"]), r["X"](op2.READ, r["c2n"]), u(op2.READ, r["c2n"]),
                 r["L"](op2.READ, r["c2c"]))
    out["c5_y"] = np.array(y.data_ro).reshape(-1)
    return out


def main():
    from oracle import op2
    out = compute(op2)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    for k, v in out.items():
        print(k, v.shape, v.dtype)


if __name__ == "__main__":
    main()
