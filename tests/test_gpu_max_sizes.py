"""Maximum sizes: loops whose element offsets, map offsets or iteration
counts pass 2^31, so every index the wrapper forms must be 64-bit.  Set
sizes themselves stay below 2^31 as in the reference (IntType is int32,
pyop2/datatypes.py:8); what grows past it is entities x dim, entities x
arity and base entities x layers.  Results are checked on the device."""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BIG = 2 ** 31


@pytest.fixture
def release():
    yield
    import torch
    gc.collect()
    torch.cuda.empty_cache()


def test_direct_dat_offsets_past_2_31(gpu_op2, release):
    """750 M entities x dim 3 = 2.25e9 doubles (18 GB): every entity's
    three components are written, the last ones beyond element 2^31."""
    import torch
    op2 = gpu_op2
    n = 750_000_000
    s = op2.Set(n)
    d = op2.Dat(s ** 3)
    assert n * 3 > BIG
    op2.par_loop(op2.Kernel("static void k(double *x) { x[0] += 1.0; x[1] += 2.0; x[2] += 3.0; }",
                            "k"), s, d(op2.INC))
    t = d.tensor
    want = torch.tensor([1.0, 2.0, 3.0], dtype=torch.float64, device=t.device)
    assert bool((t == want).all())
    assert t[-1].tolist() == [1.0, 2.0, 3.0]
    del t, d


def test_map_offsets_past_2_31(gpu_op2, release):
    """537 M cells x arity 4 = 2.148e9 map entries: INC of 1 per entry into
    1000 targets, each reached exactly 2,148,000 times; a READ through the
    same map gathers the targets' ids."""
    op2 = gpu_op2
    ncell, arity, nt = 537_000_000, 4, 1000
    assert ncell * arity > BIG
    vals = np.tile(np.arange(nt, dtype=np.int32), ncell * arity // nt).reshape(ncell, arity)
    cells, targets = op2.Set(ncell), op2.Set(nt)
    m = op2.Map(cells, targets, arity, vals)
    del vals
    y = op2.Dat(targets)
    ids = op2.Dat(targets, np.arange(nt, dtype=np.float64))
    last = op2.Dat(cells)
    op2.par_loop(op2.Kernel("""
static void k(double *y, const double *id, double *last) {
  for (int i = 0; i < 4; ++i) y[i] += 1.0;
  last[0] = id[3];
}""", "k"), cells, y(op2.INC, m), ids(op2.READ, m), last(op2.WRITE))
    t = y.tensor
    assert bool((t == float(ncell * arity // nt)).all())
    lt = last.tensor
    # cell c's last map entry is (4 c + 3) mod 1000
    for c in (0, 1, ncell // 2, ncell - 1):
        assert lt[c].item() == float((4 * c + 3) % nt)
    del t, lt, y, ids, last, m


def test_extruded_iteration_space_past_2_31(gpu_op2, release):
    """40 M base entities x 64 cell layers = 2.56e9 cells.  A loop with only
    Global arguments runs the flat (entity x layer) iteration space: an
    int64 Global counts the cells and a MAX Global sees the top layer.  A
    direct INC into a base-set Dat runs the layers of each column in order
    (direct arguments are indexed by the column): 64 per entry."""
    op2 = gpu_op2
    nb, layers = 40_000_000, 65
    assert nb * (layers - 1) > BIG
    base = op2.Set(nb)
    ext = op2.ExtrudedSet(base, layers)
    count = op2.Global(1, 0, np.int64)
    top = op2.Global(1, -1, np.int32)
    op2.par_loop(op2.Kernel("""
static void k(long long *c, int *top, int layer) {
  c[0] += 1;
  if (layer > top[0]) top[0] = layer;
}""", "k"), ext, count(op2.INC), top(op2.MAX), pass_layer_arg=True)
    assert int(count.data_ro[0]) == nb * (layers - 1)
    assert int(top.data_ro[0]) == layers - 2
    d = op2.Dat(base)
    op2.par_loop(op2.Kernel("static void k(double *x) { x[0] += 1.0; }", "k"), ext, d(op2.INC))
    t = d.tensor
    assert bool((t == float(layers - 1)).all())
    del t, d
