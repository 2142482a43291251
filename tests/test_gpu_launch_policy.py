"""Launch policies of the generated wrappers (map-row prefetch, grid
policy, CTA size) give the oracle's results; map arrays that violate the
vector-load alignment are refused on the host before any launch."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prefetch", [0, 1])
@pytest.mark.parametrize("grid", [0, -1, 7])
@pytest.mark.parametrize("bs", [128, 512])
def test_policies_match_oracle(gpu_op2, oracle_op2, prefetch, grid, bs):
    from pyop2_gb300 import _lib, workloads as W
    from pyop2_gb300.parloop import LegacyParloop
    g = W.build_p1_3d(gpu_op2, n=16, seed=9)
    o = W.build_p1_3d(oracle_op2, n=16, seed=9)
    o["run"]()
    pl = LegacyParloop(g["kernel"], g["cells"], g["y"](gpu_op2.INC, g["c2v"]),
                       g["X"](gpu_op2.READ, g["c2v"]), g["x"](gpu_op2.READ, g["c2v"]))
    pl.build(_lib.SCATTER_ATOMIC, bs, prefetch, grid)
    pl.compute()
    y = g["y"].data_ro
    ref = o["y"].data
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("prefetch", [0, 1])
def test_prefetch_with_subset_and_colours(gpu_op2, oracle_op2, prefetch):
    """Indexed iteration (Subset, colour order) prefetches through the index."""
    from pyop2_gb300.configuration import configuration
    import scenarios as S
    old = configuration["prefetch"], configuration["scatter"]
    configuration["prefetch"] = prefetch
    try:
        S.sc_subset_indirect(gpu_op2)
        configuration["scatter"] = "colour"
        S.sc_itspace_sum_nodes_to_edges(gpu_op2)
        S.sc_mixed_rhs_vector(gpu_op2)
    finally:
        configuration["prefetch"], configuration["scatter"] = old


def test_misaligned_map_is_refused(gpu_op2):
    """A map array that is not 16-byte aligned (arity 4) is rejected by the
    launch's host-side check; nothing runs on the device."""
    from pyop2_gb300 import _lib
    from pyop2_gb300.parloop import LegacyParloop
    op2 = gpu_op2
    cells, verts = op2.Set(8), op2.Set(12)
    m = op2.Map(cells, verts, 4, np.arange(32) % 12)
    y = op2.Dat(verts, np.zeros(12))
    pl = LegacyParloop(op2.Kernel("static void k(double *y) { for (int i = 0; i < 4; ++i) "
                                  "y[i] += 1.0; }", "k"), cells, y(op2.INC, m))
    pl.build()
    D = pl.launch_desc()
    k = pl._built[2]
    nptr = k.nptrs
    good = D.ptrs[nptr - 1]
    D.ptrs[nptr - 1] = good + 4          # shift the map pointer off its 16-byte boundary
    try:
        with pytest.raises(_lib.Op2gError) as e:
            _lib.call("op2g_kernel_launch", k.handle, ctypes.byref(D), None)
        assert "aligned" in str(e.value)
    finally:
        D.ptrs[nptr - 1] = good
    pl.compute()
    assert np.array_equal(y.data_ro, np.bincount(np.arange(32) % 12, minlength=12))
