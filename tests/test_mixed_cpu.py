"""Mixed containers on the CPU: caching (test/unit/test_caching.py:185-245),
MixedDat behaviour (test/unit/test_dats.py:76-236, test/unit/test_linalg.py),
and the oracle's mixed par_loops against the reference tests' values
(test/unit/test_matrices.py:864-938, test/unit/test_indirect_loop.py:235-269)."""
import numpy as np
import pytest

import scenarios as S
from pyop2_gb300 import op2
from pyop2_gb300.exceptions import DataValueError, MapTypeError, MapValueError


@pytest.fixture
def sets():
    return op2.Set(5, "a"), op2.Set(3, "b")


@pytest.fixture
def maps(sets):
    a, b = sets
    return (op2.Map(a, b, 1, [0, 1, 2, 0, 1], "m1"),
            op2.Map(a, a, 1, [4, 3, 2, 1, 0], "m2"))


def test_mixedset_cache(sets):
    a, b = sets
    assert op2.MixedSet([a, b]) is op2.MixedSet([a, b])
    assert op2.MixedSet([a, b]) is not op2.MixedSet([b, a])
    ms = op2.MixedSet([a, b])
    assert ms.sizes == (8, 8, 8) and len(ms) == 2 and ms.split == (a, b)


def test_mixedmap_cache(maps):
    m1, m2 = maps
    assert op2.MixedMap([m1, m2]) is op2.MixedMap([m1, m2])
    assert op2.MixedMap([m1, m2]) is not op2.MixedMap([m2, m1])
    mm = op2.MixedMap([m1, m2])
    assert mm.arity == 2 and mm.arities == (1, 1) and mm.arange == (0, 1, 2)
    assert mm.iterset is m1.iterset


def test_mixedmap_rejects_multiple_itersets(sets):
    a, b = sets
    with pytest.raises(RuntimeError):
        op2.MixedMap([op2.Map(a, b, 1, [0] * 5), op2.Map(b, a, 1, [0] * 3)])


def test_mixeddataset_cache(sets):
    a, b = sets
    assert op2.MixedDataSet([a, b]) is op2.MixedDataSet([a, b])
    assert op2.MixedDataSet([a, b]) is not op2.MixedDataSet([b, a])
    assert op2.MixedDataSet([a, b]) is not op2.MixedDataSet([a, a])
    ms = op2.MixedSet([a, b])
    assert ms ** 1 is ms ** 1
    assert op2.MixedDataSet(ms, (1, 2)).cdim == 3
    assert op2.MixedDataSet(ms, 2).dim == ((2,), (2,))
    with pytest.raises(ValueError):
        op2.MixedDataSet(ms, (1, 2, 3))
    assert (ms ** 2).set is ms


def test_mixeddat_copy_constructor_and_copy(sets):
    a, _ = sets
    d1 = op2.Dat(a, np.arange(5), dtype=np.float64)
    mdat = op2.MixedDat([d1, d1])
    mdat2 = op2.MixedDat(mdat)
    assert all((x.data_ro == y.data_ro).all() for x, y in zip(mdat, mdat2))
    for v in mdat.data:
        v[:] = -1
    assert all((x.data_ro != y.data_ro).all() for x, y in zip(mdat, mdat2))
    mdat3 = op2.MixedDat([a, a])
    mdat.copy(mdat3)
    assert all((x.data_ro == y.data_ro).all() for x, y in zip(mdat, mdat3))
    with pytest.raises(NotImplementedError):
        mdat.copy(op2.MixedDat([a, a]), subset=op2.Subset(a, []))


def test_mixeddat_version(sets):
    """test/unit/test_dats.py:207-236 (host part)."""
    a, _ = sets
    d1 = op2.Dat(a, np.arange(5), dtype=np.float64)
    d2 = op2.Dat(a)
    mdat = op2.MixedDat([d1, d1])
    mdat2 = op2.MixedDat([d1, d2])
    assert mdat.dat_version == 0 and mdat2.dat_version == 0
    mdat2.data
    assert d1.dat_version == 1 and d2.dat_version == 1
    assert mdat.dat_version == 2 and mdat2.dat_version == 2
    mdat.zero()
    assert d1.dat_version == 3 and d2.dat_version == 1
    assert mdat.dat_version == 6 and mdat2.dat_version == 4
    d1.zero()
    assert d1.dat_version == 4 and mdat.dat_version == 8 and mdat2.dat_version == 5


def test_mixeddat_save_load(sets, tmp_path):
    a, _ = sets
    d1 = op2.Dat(a, np.arange(5), dtype=np.float64)
    mdat = op2.MixedDat([d1, d1])
    out = str(tmp_path / "output")
    mdat.save(out)
    mdat2 = op2.MixedDat([op2.Dat(a), op2.Dat(a)])
    mdat2.load(out)
    assert all((x.data_ro == y.data_ro).all() for x, y in zip(mdat, mdat2))


def test_mixeddat_dtype_and_access_checks(sets, maps):
    a, b = sets
    with pytest.raises(DataValueError):
        op2.MixedDat([op2.Dat(a, dtype=np.float64), op2.Dat(b, dtype=np.int32)])
    md = op2.MixedDat([op2.Dat(b), op2.Dat(a)])
    with pytest.raises(MapTypeError):
        md(op2.INC, maps[0])
    with pytest.raises(MapValueError):
        md(op2.INC, op2.MixedMap([maps[0]]))
    # a component map reaching past its Dat is refused
    with pytest.raises(MapValueError):
        op2.MixedDat([op2.Dat(b), op2.Dat(b)])(op2.INC, op2.MixedMap(maps))


def test_mixed_signature_groups(sets, maps):
    """A mixed argument is one kernel parameter: its components share a
    group id in the wrapper signature."""
    from pyop2_gb300.parloop import LegacyParloop
    a, b = sets
    md = op2.MixedDat([op2.Dat(b), op2.Dat(a)])
    x = op2.Dat(a)
    k = op2.Kernel("static void k(double *v, double *x) {}", "k")
    pl = LegacyParloop(k, a, md(op2.INC, op2.MixedMap(maps)), x(op2.READ))
    _, args = pl._signature()
    assert [d[8] for d in args] == [1, 1, 0]


# -- the oracle against the reference tests' values
@pytest.mark.parametrize("itspace", [False, True])
@pytest.mark.parametrize("sizes", S.SIZES, ids=["core", "owned", "half"])
def test_oracle_mixed_non_mixed_dat(oracle_op2, sizes, itspace):
    S.sc_mixed_non_mixed_dat(oracle_op2, sizes, itspace)


@pytest.mark.parametrize("nest", [True, False])
def test_oracle_mixed_mat(oracle_op2, nest):
    sp, _ = S.sc_mixed_mat(oracle_op2, nest)
    if not nest:
        # whole-matrix dof rows: element rows see 1 + 2 columns, node rows
        # their element and node neighbours
        assert list(sp.nnz) == [3, 3, 3, 3, 5, 5, 3]


def test_oracle_mixed_rhs(oracle_op2):
    S.sc_mixed_rhs(oracle_op2)


def test_oracle_mixed_rhs_vector(oracle_op2):
    S.sc_mixed_rhs_vector(oracle_op2)
