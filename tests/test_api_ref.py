"""The reference's user-API unit tests (test/unit/test_api.py), run against
pyop2_gb300.op2: constructors, validation and the exceptions they raise,
container semantics, repr/str.  Tests that build a Sparsity, a Mat or run a
loop need the device and are marked ``gpu``; the rest run on the CPU."""
import numpy as np
import pytest
from numpy.testing import assert_equal

from pyop2_gb300 import exceptions, op2

gpu = pytest.mark.gpu


# ----------------------------------------------------------------- fixtures
@pytest.fixture
def set():
    return op2.Set(5, 'foo')


@pytest.fixture
def iterset():
    return op2.Set(2, 'iterset')


@pytest.fixture
def toset():
    return op2.Set(3, 'toset')


@pytest.fixture
def sets(set, iterset, toset):
    return set, iterset, toset


@pytest.fixture
def mset(sets):
    return op2.MixedSet(sets)


@pytest.fixture(params=['sets', 'mset', 'gen'])
def msets(sets, mset, request):
    return {'sets': sets, 'mset': mset, 'gen': iter(sets)}[request.param]


@pytest.fixture(params=[1, 2, (2, 3)])
def dset(request, set):
    return op2.DataSet(set, request.param, 'dfoo')


@pytest.fixture
def diterset(iterset):
    return op2.DataSet(iterset, 1, 'diterset')


@pytest.fixture
def dtoset(toset):
    return op2.DataSet(toset, 1, 'dtoset')


@pytest.fixture
def dsets(dset, diterset, dtoset):
    return dset, diterset, dtoset


@pytest.fixture
def mdset(dsets):
    return op2.MixedDataSet(dsets)


@pytest.fixture
def dat(dtoset):
    return op2.Dat(dtoset, np.arange(dtoset.cdim * dtoset.size, dtype=np.int32))


@pytest.fixture
def dats(dtoset, dset):
    return op2.Dat(dtoset), op2.Dat(dset)


@pytest.fixture
def mdat(dats):
    return op2.MixedDat(dats)


@pytest.fixture
def m_iterset_toset(iterset, toset):
    return op2.Map(iterset, toset, 2, [1] * 2 * iterset.size, 'm_iterset_toset')


@pytest.fixture
def m_iterset_set(iterset, set):
    return op2.Map(iterset, set, 2, [1] * 2 * iterset.size, 'm_iterset_set')


@pytest.fixture
def m_set_toset(set, toset):
    return op2.Map(set, toset, 1, [1] * set.size, 'm_set_toset')


@pytest.fixture
def m_set_set(set):
    return op2.Map(set, set, 1, [1] * set.size, 'm_set_set')


@pytest.fixture
def maps(m_iterset_toset, m_iterset_set):
    return m_iterset_toset, m_iterset_set


@pytest.fixture
def mmap(maps):
    return op2.MixedMap(maps)


@pytest.fixture
def mds(dtoset, set):
    return op2.MixedDataSet((dtoset, set))


@pytest.fixture(params=[('mds', 'mds', 'mmap', 'mmap'),
                        ('mds', 'dtoset', 'mmap', 'm_iterset_toset'),
                        ('dtoset', 'mds', 'm_iterset_toset', 'mmap')])
def ms(request):
    rds, cds, rmm, cmm = [request.getfixturevalue(p) for p in request.param]
    return op2.Sparsity((rds, cds), {(i, j): [(rm, cm, None)] for i, rm in enumerate(rmm)
                                     for j, cm in enumerate(cmm)})


@pytest.fixture
def sparsity(m_iterset_toset, dtoset):
    return op2.Sparsity((dtoset, dtoset), [(m_iterset_toset, m_iterset_toset, None)])


@pytest.fixture
def mat(sparsity):
    return op2.Mat(sparsity)


@pytest.fixture
def diag_mat(toset):
    _d = toset ** 1
    _m = op2.Map(toset, toset, 1, np.arange(toset.size))
    return op2.Mat(op2.Sparsity((_d, _d), [(_m, _m, None)]))


@pytest.fixture
def mmat(ms):
    return op2.Mat(ms)


@pytest.fixture
def g():
    return op2.Global(1, 1)


# ------------------------------------------------------------------ classes
class TestClassAPI:

    def test_isinstance(self, set, dat):
        assert isinstance(set, op2.Set) and isinstance(dat, op2.Dat)
        assert not isinstance(set, op2.Dat) and not isinstance(dat, op2.Set)

    def test_issubclass(self, set, dat):
        assert issubclass(type(set), op2.Set) and issubclass(type(dat), op2.Dat)
        assert not issubclass(type(set), op2.Dat) and not issubclass(type(dat), op2.Set)


class TestSetAPI:

    def test_set_illegal_size(self):
        with pytest.raises(exceptions.SizeTypeError):
            op2.Set('illegalsize')

    def test_set_illegal_name(self):
        with pytest.raises(exceptions.NameTypeError):
            op2.Set(1, 2)

    def test_set_iter(self, set):
        for s in set:
            assert s is set

    def test_set_len(self, set):
        assert len(set) == 1

    def test_set_repr(self, set):
        from pyop2_gb300.op2 import Set  # noqa: F401 (used by eval)
        assert isinstance(eval(repr(set)), op2.Set)

    def test_set_str(self, set):
        assert str(set) == "OP2 Set: %s with size %s" % (set.name, set.size)

    def test_set_eq(self, set):
        assert set == set
        assert not set != set

    def test_dset_in_set(self, set, dset):
        assert dset in set

    def test_dset_not_in_set(self, dset):
        assert dset not in op2.Set(5, 'bar')

    def test_set_exponentiation_builds_dset(self, set):
        dset = set ** 1
        assert isinstance(dset, op2.DataSet) and dset.cdim == 1
        assert (set ** 3).cdim == 3


class TestExtrudedSetAPI:

    def test_illegal_layers_arg(self, set):
        with pytest.raises(exceptions.SizeTypeError):
            op2.ExtrudedSet(set, 1)

    def test_illegal_set_arg(self):
        with pytest.raises(TypeError):
            op2.ExtrudedSet(1, 3)

    def test_set_compatiblity(self, set, iterset):
        e = op2.ExtrudedSet(set, 5)
        assert set in e
        assert iterset not in e

    @gpu
    def test_iteration_compatibility(self, gpu_op2, iterset, m_iterset_toset, m_iterset_set, dats):
        e = op2.ExtrudedSet(iterset, 5)
        k = op2.Kernel('static void k() { }', 'k')
        dat1, dat2 = dats
        op2.par_loop(k, e, dat1(op2.READ, m_iterset_toset))
        op2.par_loop(k, e, dat2(op2.READ, m_iterset_set))

    def test_iteration_incompatibility(self, set, m_iterset_toset, dat):
        e = op2.ExtrudedSet(set, 5)
        k = op2.Kernel('static void k() { }', 'k')
        with pytest.raises(exceptions.MapValueError):
            op2.ParLoop(k, e, dat(op2.READ, m_iterset_toset))


class TestSubsetAPI:

    def test_illegal_set_arg(self):
        with pytest.raises(TypeError):
            op2.Subset("fail", [0, 1])

    def test_out_of_bounds_index(self, set):
        with pytest.raises(exceptions.SubsetIndexOutOfBounds):
            op2.Subset(set, list(range(set.total_size + 1)))

    def test_invalid_index(self, set):
        with pytest.raises(exceptions.SubsetIndexOutOfBounds):
            op2.Subset(set, [-1])

    def test_empty_subset(self, set):
        assert len(op2.Subset(set, []).indices) == 0

    def test_index_construction(self, set):
        assert_equal(set(0, 1).indices, op2.Subset(set, [0, 1]).indices)
        assert_equal(set(0).indices, op2.Subset(set, [0]).indices)
        assert_equal(set(np.arange(5)).indices, op2.Subset(set, np.arange(5)).indices)

    def test_indices_duplicate_removed(self, set):
        ss = op2.Subset(set, [0, 0, 1, 1])
        assert np.sum(ss.indices == 0) == 1 and np.sum(ss.indices == 1) == 1

    def test_indices_sorted(self, set):
        ss = op2.Subset(set, [0, 4, 1, 2, 3])
        assert_equal(ss.indices, list(range(5)))
        assert_equal(ss.indices, op2.Subset(set, list(range(5))).indices)


class TestMixedSetAPI:

    def test_mixed_set_illegal_set(self):
        with pytest.raises(TypeError):
            op2.MixedSet(('foo', 'bar'))

    def test_mixed_set_getitem(self, sets):
        mset = op2.MixedSet(sets)
        for i, s in enumerate(sets):
            assert mset[i] == s

    def test_mixed_set_split(self, sets):
        assert op2.MixedSet(sets).split == sets

    def test_mixed_set_sizes(self, mset):
        assert mset.core_size == sum(s.core_size for s in mset)
        assert mset.size == sum(s.size for s in mset)
        assert mset.total_size == sum(s.total_size for s in mset)
        assert mset.sizes == (mset.core_size, mset.size, mset.total_size)

    def test_mixed_set_name(self, mset):
        assert mset.name == tuple(s.name for s in mset)

    def test_mixed_set_halo(self, mset):
        assert mset.halo is None

    def test_mixed_set_layers(self, mset):
        assert mset.layers == mset[0].layers

    def test_mixed_set_layers_must_match(self, sets):
        sets = [op2.ExtrudedSet(s, layers=i + 4) for i, s in enumerate(sets)]
        with pytest.raises(AssertionError):
            op2.MixedSet(sets)

    def test_mixed_set_iter(self, mset, sets):
        assert tuple(s for s in mset) == sets

    def test_mixed_set_len(self, sets):
        assert len(op2.MixedSet(sets)) == len(sets)

    def test_mixed_set_pow(self, mset):
        expect = op2.MixedDataSet([s ** 1 for s in mset])
        assert mset ** 1 == expect
        assert mset ** ((1,) * len(mset)) == expect
        assert mset ** (1 for _ in mset) == expect

    def test_mixed_set_eq(self, sets):
        assert op2.MixedSet(sets) == op2.MixedSet(sets)
        assert not op2.MixedSet(sets) != op2.MixedSet(sets)

    def test_mixed_set_ne(self, set, iterset, toset):
        assert op2.MixedSet((set, iterset, toset)) != op2.MixedSet((set, toset, iterset))
        assert not op2.MixedSet((set, iterset, toset)) == op2.MixedSet((set, toset, iterset))

    def test_mixed_set_ne_set(self, sets):
        assert op2.MixedSet(sets) != sets[0]
        assert not op2.MixedSet(sets) == sets[0]

    def test_mixed_set_repr(self, mset):
        from pyop2_gb300.op2 import Set, MixedSet  # noqa: F401 (used by eval)
        assert isinstance(eval(repr(mset)), op2.MixedSet)

    def test_mixed_set_str(self, mset):
        assert str(mset) == "OP2 MixedSet composed of Sets: %s" % (mset._sets,)


class TestDataSetAPI:

    def test_dset_illegal_dim(self, iterset):
        with pytest.raises(TypeError):
            op2.DataSet(iterset, 'illegaldim')

    def test_dset_illegal_dim_tuple(self, iterset):
        with pytest.raises(TypeError):
            op2.DataSet(iterset, (1, 'illegaldim'))

    def test_dset_illegal_name(self, iterset):
        with pytest.raises(exceptions.NameTypeError):
            op2.DataSet(iterset, 1, 2)

    def test_dset_dims(self, iterset):
        assert op2.DataSet(iterset).dim == (1,)
        assert op2.DataSet(iterset, 1).dim == (1,)
        assert op2.DataSet(iterset, [2, 3]).dim == (2, 3)

    def test_dset_iter_len(self, dset):
        for s in dset:
            assert s is dset
        assert len(dset) == 1

    def test_dset_repr(self, dset):
        from pyop2_gb300.op2 import Set, DataSet  # noqa: F401 (used by eval)
        assert isinstance(eval(repr(dset)), op2.DataSet)

    def test_dset_str(self, dset):
        assert str(dset) == "OP2 DataSet: %s on set %s, with dim %s" % (dset.name, dset.set,
                                                                         dset.dim)

    def test_dset_eq(self, dset):
        dsetcopy = op2.DataSet(dset.set, dset.dim)
        assert dsetcopy == dset
        assert not dsetcopy != dset

    def test_dset_ne_set(self, dset):
        dsetcopy = op2.DataSet(op2.Set(dset.set.size), dset.dim)
        assert dsetcopy != dset
        assert not dsetcopy == dset

    def test_dset_ne_dim(self, dset):
        dsetcopy = op2.DataSet(dset.set, tuple(d + 1 for d in dset.dim))
        assert dsetcopy != dset
        assert not dsetcopy == dset

    def test_dat_in_dset(self, dset):
        assert op2.Dat(dset) in dset
        assert op2.Dat(dset) not in op2.DataSet(op2.Set(5, 'bar'))


class TestMixedDataSetAPI:

    @pytest.mark.parametrize('arg', ['illegalarg', (set, 'illegalarg'),
                                     iter((set, 'illegalarg'))])
    def test_mixed_dset_illegal_arg(self, arg):
        with pytest.raises(TypeError):
            op2.MixedDataSet(arg)

    @pytest.mark.parametrize('dims', ['illegaldim', (1, 2, 'illegaldim')])
    def test_mixed_dset_dsets_illegal_dims(self, dsets, dims):
        with pytest.raises((TypeError, ValueError)):
            op2.MixedDataSet(dsets, dims)

    def test_mixed_dset_dsets_dims(self, dsets):
        with pytest.raises(TypeError):
            op2.MixedDataSet(dsets, 1)

    def test_mixed_dset_upcast_sets(self, msets, mset):
        assert op2.MixedDataSet(msets) == mset ** 1

    def test_mixed_dset_sets_and_dsets(self, set, dset):
        assert op2.MixedDataSet((set, dset)).split == (set ** 1, dset)
        assert op2.MixedDataSet(iter((set, dset))).split == (set ** 1, dset)

    def test_mixed_dset_dims_default_to_one(self, msets, mset):
        assert op2.MixedDataSet(msets).dim == ((1,),) * len(mset)

    def test_mixed_dset_dims_int(self, msets, mset):
        assert op2.MixedDataSet(msets, 2).dim == ((2,),) * len(mset)

    def test_mixed_dset_dims_gen(self, msets, mset):
        assert op2.MixedDataSet(msets, (2 for _ in mset)).dim == ((2,),) * len(mset)

    def test_mixed_dset_dims_iterable(self, msets):
        dims = ((2,), (2, 2), (1,))
        assert op2.MixedDataSet(msets, dims).dim == dims

    def test_mixed_dset_dims_mismatch(self, msets, sets):
        with pytest.raises(ValueError):
            op2.MixedDataSet(msets, list(range(1, len(sets))))

    def test_mixed_dset_getitem_split(self, mdset, dsets):
        for i, ds in enumerate(mdset):
            assert mdset[i] == ds
        assert op2.MixedDataSet(dsets).split == dsets

    def test_mixed_dset_dim_cdim_name(self, mdset):
        assert mdset.dim == tuple(s.dim for s in mdset)
        assert mdset.cdim == sum(s.cdim for s in mdset)
        assert mdset.name == tuple(s.name for s in mdset)

    def test_mixed_dset_set(self, mset):
        assert op2.MixedDataSet(mset).set == mset

    def test_mixed_dset_iter_len(self, mdset, dsets):
        assert tuple(s for s in mdset) == dsets
        assert len(op2.MixedDataSet(dsets)) == len(dsets)

    def test_mixed_dset_eq(self, dsets):
        assert op2.MixedDataSet(dsets) == op2.MixedDataSet(dsets)
        assert not op2.MixedDataSet(dsets) != op2.MixedDataSet(dsets)

    def test_mixed_dset_ne(self, dset, diterset, dtoset):
        mds1 = op2.MixedDataSet((dset, diterset, dtoset))
        mds2 = op2.MixedDataSet((dset, dtoset, diterset))
        assert mds1 != mds2
        assert not mds1 == mds2

    def test_mixed_dset_ne_dset(self, diterset, dtoset):
        assert op2.MixedDataSet((diterset, dtoset)) != diterset
        assert not op2.MixedDataSet((diterset, dtoset)) == diterset

    def test_mixed_dset_repr(self, mdset):
        from pyop2_gb300.op2 import Set, DataSet, MixedDataSet  # noqa: F401 (used by eval)
        assert isinstance(eval(repr(mdset)), op2.MixedDataSet)

    def test_mixed_dset_str(self, mdset):
        assert str(mdset) == "OP2 MixedDataSet composed of DataSets: %s" % (mdset._dsets,)


class TestDatAPI:

    def test_dat_illegal_set(self):
        with pytest.raises(exceptions.DataSetTypeError):
            op2.Dat('illegalset', 1)

    def test_dat_illegal_name(self, dset):
        with pytest.raises(exceptions.NameTypeError):
            op2.Dat(dset, name=2)

    def test_dat_initialise_data(self, dset):
        d = op2.Dat(dset)
        assert d.data.size == dset.size * dset.cdim and d.data.dtype == np.float64
        assert op2.Dat(dset, dtype=np.int32).data.dtype == np.int32

    def test_dat_subscript(self, dat):
        assert dat[0] is dat
        with pytest.raises(exceptions.IndexValueError):
            dat[1]

    def test_dat_arg_default_map(self, dat):
        assert dat(op2.READ).map_ is None

    def test_dat_arg_illegal_map(self, dset):
        d = op2.Dat(dset)
        to_set2 = op2.Map(op2.Set(3), op2.Set(2), 1, [0, 0, 0])
        with pytest.raises(exceptions.MapValueError):
            d(op2.READ, to_set2)

    def test_dat_on_set_builds_dim_one_dataset(self, set):
        d = op2.Dat(set)
        assert d.cdim == 1 and isinstance(d.dataset, op2.DataSet) and d.dataset.cdim == 1

    def test_dat_dtypes(self, dset):
        n = dset.size * dset.cdim
        assert isinstance(op2.Dat(dset).dtype, np.dtype)
        assert isinstance(op2.Dat(dset, [1.0] * n).dtype, np.dtype)
        assert op2.Dat(dset).dtype == np.double
        assert op2.Dat(dset, [1.0] * n).dtype == np.double
        assert op2.Dat(dset, [1] * n).dtype == np.asarray(1).dtype
        assert op2.Dat(dset, [1] * n, np.double).dtype == np.float64
        assert op2.Dat(dset, [1.5] * n, np.int32).dtype == np.int32

    def test_dat_split(self, dat):
        assert all(d is dat for d in dat.split)

    def test_dat_illegal_dtype(self, dset):
        with pytest.raises(exceptions.DataTypeError):
            op2.Dat(dset, dtype='illegal_type')

    def test_dat_illegal_length(self, dset):
        with pytest.raises(exceptions.DataValueError):
            op2.Dat(dset, [1] * (dset.size * dset.cdim + 1))

    def test_dat_reshape(self, dset):
        d = op2.Dat(dset, [1.0] * dset.size * dset.cdim)
        assert d.data.shape == (dset.size,) + (() if dset.cdim == 1 else dset.dim)

    def test_dat_properties(self, dset):
        d = op2.Dat(dset, [1] * dset.size * dset.cdim, 'double', 'bar')
        assert d.dataset.set == dset.set and d.dtype == np.float64 and d.name == 'bar' \
            and d.data.sum() == dset.size * dset.cdim

    def test_dat_iter_len(self, dat):
        for d in dat:
            assert d is dat
        assert len(dat) == 1

    def test_dat_repr(self, dat):
        from pyop2_gb300.op2 import Dat, DataSet, Set  # noqa: F401 (used by eval)
        from numpy import dtype  # noqa: F401 (used by eval)
        assert isinstance(eval(repr(dat)), op2.Dat)

    def test_dat_str(self, dset):
        d = op2.Dat(dset, dtype='double', name='bar')
        assert str(d) == "OP2 Dat: %s on (%s) with datatype %s" % (d.name, d.dataset,
                                                                   d.data.dtype.name)

    def test_dat_ro_accessor(self, dat):
        x = dat.data_ro
        with pytest.raises((RuntimeError, ValueError)):
            x[0] = 1
        x = dat.data
        x[0] = -100
        assert (dat.data_ro[0] == -100).all()

    def test_dat_lazy_allocation(self, dset):
        assert not op2.Dat(dset)._is_allocated

    def test_dat_zero_cdim(self, set):
        d = op2.Dat(set ** 0)
        assert d.shape == (set.total_size, 0)
        assert d._data.size == 0 and d._data.shape == (set.total_size, 0)


class TestMixedDatAPI:

    def test_mixed_dat_illegal_arg(self):
        with pytest.raises(exceptions.DataSetTypeError):
            op2.MixedDat('illegalarg')

    def test_mixed_dat_illegal_dtype(self, set):
        with pytest.raises(exceptions.DataValueError):
            op2.MixedDat((op2.Dat(set, dtype=np.int32), op2.Dat(set)))

    def test_mixed_dat_dats(self, dats):
        assert op2.MixedDat(dats).split == dats

    def test_mixed_dat_dsets(self, mdset, mset):
        assert op2.MixedDat(mdset).dataset == mdset
        assert op2.MixedDat(mset).dataset == op2.MixedDataSet(mset)

    def test_mixed_dat_getitem(self, mdat):
        for i, d in enumerate(mdat):
            assert mdat[i] == d
        assert mdat[:-1] == tuple(mdat)[:-1]

    def test_mixed_dat_dim_cdim(self, mdset):
        assert op2.MixedDat(mdset).dim == mdset.dim
        assert op2.MixedDat(mdset).cdim == mdset.cdim

    def test_mixed_dat_data(self, mdat):
        assert all((d1 == d2.data).all() for d1, d2 in zip(mdat.data, mdat))
        assert all((d1 == d2.data_ro).all() for d1, d2 in zip(mdat.data_ro, mdat))
        assert all((d1 == d2.data_with_halos).all()
                   for d1, d2 in zip(mdat.data_with_halos, mdat))
        assert all((d1 == d2.data_ro_with_halos).all()
                   for d1, d2 in zip(mdat.data_ro_with_halos, mdat))

    def test_mixed_dat_halo_valid(self, mdat):
        assert mdat.halo_valid
        mdat[0].halo_valid = False
        assert not mdat.halo_valid

    def test_mixed_dat_halo_valid_setter(self, mdat):
        assert mdat.halo_valid
        mdat.halo_valid = False
        assert not any(d.halo_valid for d in mdat)

    def test_mixed_dat_iter_len(self, mdat, dats):
        assert tuple(s for s in mdat) == dats
        assert len(op2.MixedDat(dats)) == len(dats)

    def test_mixed_dat_eq(self, dats):
        assert op2.MixedDat(dats) == op2.MixedDat(dats)
        assert not op2.MixedDat(dats) != op2.MixedDat(dats)

    def test_mixed_dat_ne(self, dats):
        mdat1 = op2.MixedDat(dats)
        mdat2 = op2.MixedDat(reversed(dats))
        assert mdat1 != mdat2
        assert not mdat1 == mdat2

    def test_mixed_dat_ne_dat(self, dats):
        assert op2.MixedDat(dats) != dats[0]
        assert not op2.MixedDat(dats) == dats[0]

    def test_mixed_dat_repr(self, mdat):
        from pyop2_gb300.op2 import Set, DataSet, MixedDataSet, Dat, MixedDat  # noqa: F401
        from numpy import dtype  # noqa: F401 (used by eval)
        assert isinstance(eval(repr(mdat)), op2.MixedDat)

    def test_mixed_dat_str(self, mdat):
        assert str(mdat) == "OP2 MixedDat composed of Dats: %s" % (mdat.split,)


class TestSparsityAPI:

    @pytest.fixture
    def mi(cls, toset):
        iterset = op2.Set(3, 'iterset2')
        return op2.Map(iterset, toset, 1, [1] * iterset.size, 'mi')

    @pytest.fixture
    def dataset2(cls):
        return op2.Set(1, 'dataset2')

    @pytest.fixture
    def md(cls, iterset, dataset2):
        return op2.Map(iterset, dataset2, 1, [0] * iterset.size, 'md')

    @pytest.fixture
    def di(cls, toset):
        return op2.DataSet(toset, 1, 'di')

    @pytest.fixture
    def dd(cls, dataset2):
        return op2.DataSet(dataset2, 1, 'dd')

    @pytest.fixture
    def s(cls, di, mi):
        return op2.Sparsity((di, di), [(mi, mi, None)])

    def test_sparsity_illegal_dsets_and_maps(self, di, mi):
        with pytest.raises(TypeError):
            op2.Sparsity(('illegalrmap', di), [(mi, mi, None)])
        with pytest.raises(TypeError):
            op2.Sparsity((di, 'illegalrmap'), [(mi, mi, None)])
        with pytest.raises(TypeError):
            op2.Sparsity((di, di), [('illegalrmap', mi, None)])
        with pytest.raises(TypeError):
            op2.Sparsity((di, di), [(mi, 'illegalcmap', None)])

    def test_sparsity_illegal_name(self, di, mi):
        with pytest.raises(TypeError):
            op2.Sparsity((di, di), [(mi, mi, None)], 0)

    @gpu
    def test_sparsity_map_pair_different_dataset(self, gpu_op2, mi, md, di, dd, m_iterset_toset):
        s = op2.Sparsity((di, dd), [(m_iterset_toset, md, None)], name="foo")
        assert (s.rcmaps[(0, 0)][0] == (m_iterset_toset, md) and s.dims[0][0] == (1, 1)
                and s.name == "foo" and s.dsets == (di, dd))

    @gpu
    def test_sparsity_unique_map_pairs(self, gpu_op2, mi, di):
        s = op2.Sparsity((di, di), [(mi, mi, None), (mi, mi, None)], name="foo")
        assert s.rcmaps[(0, 0)] == [(mi, mi)] and s.dims[0][0] == (1, 1)

    @gpu
    def test_sparsity_map_pairs_different_itset(self, gpu_op2, mi, di, dd, m_iterset_toset):
        maps = ((m_iterset_toset, m_iterset_toset), (mi, mi))
        s = op2.Sparsity((di, di), [(*maps[0], None), (*maps[1], None)], name="foo")
        assert frozenset(s.rcmaps[(0, 0)]) == frozenset(maps) and s.dims[0][0] == (1, 1)

    @gpu
    def test_sparsity_map_pairs_sorted(self, gpu_op2, mi, di, dd, m_iterset_toset):
        s1 = op2.Sparsity((di, di), [(m_iterset_toset, m_iterset_toset, None), (mi, mi, None)])
        s2 = op2.Sparsity((di, di), [(mi, mi, None), (m_iterset_toset, m_iterset_toset, None)])
        assert s1.rcmaps[(0, 0)] == s2.rcmaps[(0, 0)]

    def test_sparsity_illegal_itersets_and_datasets(self, mi, md, di, dd):
        with pytest.raises(RuntimeError):
            op2.Sparsity((dd, di), [(md, mi, None)])
        with pytest.raises(RuntimeError):
            op2.Sparsity((di, di), [(mi, mi, None), (md, mi, None)])
        with pytest.raises(RuntimeError):
            op2.Sparsity((di, di), [(mi, mi, None), (mi, md, None)])

    @gpu
    def test_sparsity_single_block(self, gpu_op2, s):
        assert s.shape == (1, 1)
        for bs in s:
            assert bs == s
        assert s[0, 0] == s

    @gpu
    def test_sparsity_mmap_blocks(self, gpu_op2, ms):
        cols = ms.shape[1]
        for i, block in enumerate(ms):
            assert block == ms[i // cols, i % cols]
        for i, rds in enumerate(ms.dsets[0]):
            for j, cds in enumerate(ms.dsets[1]):
                block = ms[i, j]
                assert block == ms[i][j]
                assert block.dsets == (rds, cds) and block.rcmaps[(0, 0)] == ms.rcmaps[(i, j)]
        for i, rds in enumerate(ms.dsets[0]):
            for j, (s, cds) in enumerate(zip(ms[i], ms.dsets[1])):
                assert s.dsets == (rds, cds) and s.rcmaps[(0, 0)] == ms.rcmaps[(i, j)]
        assert ms.shape == (len(ms.dsets[0]), len(ms.dsets[1]))

    def test_sparsity_mmap_illegal(self, m_iterset_toset, m_iterset_set, m_set_toset,
                                   m_set_set, mds):
        def build(rmm, cmm):
            op2.Sparsity((mds, mds), {(i, j): [(rm, cm, None)] for i, rm in enumerate(rmm)
                                      for j, cm in enumerate(cmm)})
        with pytest.raises(RuntimeError):     # different itersets in a pair
            build(op2.MixedMap((m_iterset_toset, m_iterset_set)),
                  op2.MixedMap((m_set_toset, m_set_set)))
        with pytest.raises(RuntimeError):     # row maps onto the wrong sets
            build(op2.MixedMap((m_iterset_toset, m_iterset_set)),
                  op2.MixedMap((m_set_toset, m_set_toset)))
        with pytest.raises(RuntimeError):     # column maps onto the wrong sets
            build(op2.MixedMap((m_set_toset, m_set_toset)),
                  op2.MixedMap((m_iterset_toset, m_iterset_set)))

    @gpu
    def test_sparsity_repr_str(self, gpu_op2, sparsity):
        r = "Sparsity(%r, %r, name=%r, nested=%r, block_sparse=%r, diagonal_block=%r)" % (
            sparsity.dsets, sparsity._maps_and_regions, sparsity.name, sparsity._nested,
            sparsity._block_sparse, sparsity._diagonal_block)
        assert repr(sparsity) == r
        s = ("OP2 Sparsity: dsets %s, maps_and_regions %s, name %s, nested %s, "
             "block_sparse %s, diagonal_block %s") % (
            sparsity.dsets, sparsity._maps_and_regions, sparsity.name, sparsity._nested,
            sparsity._block_sparse, sparsity._diagonal_block)
        assert str(sparsity) == s


class TestMatAPI:

    def test_mat_illegal_sets(self):
        with pytest.raises(TypeError):
            op2.Mat('illegalsparsity')

    @gpu
    def test_mat_illegal_name(self, gpu_op2, sparsity):
        with pytest.raises(exceptions.NameTypeError):
            op2.Mat(sparsity, name=2)

    @gpu
    def test_mat_properties(self, gpu_op2, sparsity, mat):
        assert mat.dtype == np.double
        m = op2.Mat(sparsity, 'double', 'bar')
        assert m.sparsity == sparsity and m.dtype == np.float64 and m.name == 'bar'

    @gpu
    def test_mat_mixed(self, gpu_op2, mmat):
        assert mmat.dtype == np.double

    @gpu
    def test_mat_illegal_maps(self, gpu_op2, mat):
        wrongmap = op2.Map(op2.Set(2), op2.Set(3), 2, [0, 0, 0, 0])
        with pytest.raises(exceptions.MapValueError):
            mat(op2.INC, (wrongmap, wrongmap))

    @gpu
    @pytest.mark.parametrize("mode", [op2.READ, op2.RW, op2.MIN, op2.MAX])
    def test_mat_arg_illegal_mode(self, gpu_op2, mat, mode, m_iterset_toset):
        with pytest.raises(exceptions.ModeValueError):
            mat(mode, (m_iterset_toset, m_iterset_toset))

    @gpu
    def test_mat_iter_repr_str(self, gpu_op2, mat):
        for m in mat:
            assert m is mat
        assert repr(mat) == "Mat(%r, %r, %r)" % (mat.sparsity, mat.dtype, mat.name)
        assert str(mat) == "OP2 Mat: %s, sparsity (%s), datatype %s" % (
            mat.name, mat.sparsity, mat.dtype.name)


class TestGlobalAPI:

    def test_global_illegal_dim(self):
        with pytest.raises(TypeError):
            op2.Global('illegaldim')
        with pytest.raises(TypeError):
            op2.Global((1, 'illegaldim'))

    def test_global_illegal_name(self):
        with pytest.raises(exceptions.NameTypeError):
            op2.Global(1, 1, name=2)

    def test_global_dim(self):
        assert op2.Global(1, 1).dim == (1,)
        assert op2.Global([2, 3], [1] * 6).dim == (2, 3)

    def test_global_dtypes(self):
        assert op2.Global(1, 1.0).dtype == np.asarray(1.0).dtype
        assert op2.Global(1, 1).dtype == np.asarray(1).dtype
        assert op2.Global(1, 1, dtype=np.float64).dtype == np.float64
        assert op2.Global(1, 1.5, dtype=np.int64).dtype == np.int64

    def test_global_illegal_dtype(self):
        with pytest.raises(exceptions.DataValueError):
            op2.Global(1, 'illegal_type', 'double')

    @pytest.mark.parametrize("dim", [1, (2, 2)])
    def test_global_illegal_length(self, dim):
        with pytest.raises(exceptions.DataValueError):
            op2.Global(dim, [1] * (np.prod(dim) + 1))

    def test_global_reshape_properties(self):
        g = op2.Global((2, 2), [1.0] * 4)
        assert g.dim == (2, 2) and g.data.shape == (2, 2)
        g = op2.Global((2, 2), [1] * 4, 'double', 'bar')
        assert g.dim == (2, 2) and g.dtype == np.float64 and g.name == 'bar' \
            and g.data.sum() == 4

    def test_global_setter(self, g):
        g.data = 2
        assert g.data.sum() == 2
        with pytest.raises(exceptions.DataValueError):
            g.data = [1, 2]

    def test_global_iter_len(self, g):
        for g_ in g:
            assert g_ is g
        assert len(g) == 1

    def test_global_str(self):
        g = op2.Global(1, 1, 'double')
        assert str(g) == "OP2 Global Argument: %s with dim %s and value %s" % (g.name, g.dim,
                                                                                g.data)

    @pytest.mark.parametrize("mode", [op2.RW, op2.WRITE])
    def test_global_arg_illegal_mode(self, g, mode):
        with pytest.raises(exceptions.ModeValueError):
            g(mode)


class TestMapAPI:

    def test_map_illegal_args(self, set):
        with pytest.raises(exceptions.SetTypeError):
            op2.Map('illegalset', set, 1, [])
        with pytest.raises(exceptions.SetTypeError):
            op2.Map(set, 'illegalset', 1, [])
        with pytest.raises(exceptions.ArityTypeError):
            op2.Map(set, set, 'illegalarity', [])
        with pytest.raises(exceptions.ArityTypeError):
            op2.Map(set, set, (2, 2), [])
        with pytest.raises(exceptions.NameTypeError):
            op2.Map(set, set, 1, [], name=2)

    def test_map_illegal_dtype(self, set):
        with pytest.raises(exceptions.DataValueError):
            op2.Map(set, set, 1, 'abcdefg')

    def test_map_illegal_length(self, iterset, toset):
        with pytest.raises(exceptions.DataValueError):
            op2.Map(iterset, toset, 1, [1] * (iterset.size + 1))

    def test_map_convert_float_int(self, iterset, toset):
        from pyop2_gb300.datatypes import IntType
        m = op2.Map(iterset, toset, 1, [1.5] * iterset.size)
        assert m.values.dtype == IntType and m.values.sum() == iterset.size

    def test_map_reshape(self, iterset, toset):
        m = op2.Map(iterset, toset, 2, [1] * 2 * iterset.size)
        assert m.arity == 2 and m.values.shape == (iterset.size, 2)

    def test_map_split(self, m_iterset_toset):
        assert all(m is m_iterset_toset for m in m_iterset_toset.split)

    def test_map_properties(self, iterset, toset):
        m = op2.Map(iterset, toset, 2, [1] * 2 * iterset.size, 'bar')
        assert (m.iterset == iterset and m.toset == toset and m.arity == 2
                and m.arities == (2,) and m.arange == (0, 2)
                and m.values.sum() == 2 * iterset.size and m.name == 'bar')

    def test_map_eq(self, m_iterset_toset):
        m = m_iterset_toset
        mcopy = op2.Map(m.iterset, m.toset, m.arity, m.values)
        assert m != mcopy and not m == mcopy and mcopy == mcopy

    def test_map_ne(self, m_iterset_toset):
        m = m_iterset_toset
        for mcopy in (op2.Map(op2.Set(m.iterset.size), m.toset, m.arity, m.values),
                      op2.Map(m.iterset, op2.Set(m.toset.size), m.arity, m.values),
                      op2.Map(m.iterset, m.toset, m.arity * 2, list(m.values) * 2)):
            assert m != mcopy and not m == mcopy

    def test_map_ne_values(self, m_iterset_toset):
        m = m_iterset_toset
        m2 = op2.Map(m.iterset, m.toset, m.arity, m.values.copy())
        m2.values[0] = 2
        assert m != m2 and not m == m2

    def test_map_iter_len(self, m_iterset_toset):
        for m_ in m_iterset_toset:
            assert m_ is m_iterset_toset
        assert len(m_iterset_toset) == 1

    def test_map_repr_str(self, m_iterset_toset):
        m = m_iterset_toset
        assert repr(m) == "Map(%r, %r, %r, None, %r, %r, %r)" % (
            m.iterset, m.toset, m.arity, m.name, m._offset, m._offset_quotient)
        assert str(m) == "OP2 Map: %s from (%s) to (%s) with arity %s" % (
            m.name, m.iterset, m.toset, m.arity)


class TestMixedMapAPI:

    def test_mixed_map_illegal_arg(self):
        with pytest.raises(TypeError):
            op2.MixedMap('illegalarg')

    def test_mixed_map_split(self, maps):
        mmap = op2.MixedMap(maps)
        assert mmap.split == maps
        for i, m in enumerate(maps):
            assert mmap.split[i] == m
        assert mmap.split[:-1] == tuple(mmap)[:-1]

    def test_mixed_map_properties(self, mmap):
        for m in mmap:
            assert mmap.iterset == m.iterset
        assert mmap.toset == op2.MixedSet(m.toset for m in mmap)
        assert mmap.arity == sum(m.arity for m in mmap)
        assert mmap.arities == tuple(m.arity for m in mmap)
        assert mmap.arange == (0,) + tuple(np.cumsum(mmap.arities))
        assert all((v == m.values).all() for v, m in zip(mmap.values, mmap))
        assert all((v == m.values_with_halo).all() for v, m in zip(mmap.values_with_halo, mmap))
        assert mmap.name == tuple(m.name for m in mmap)
        assert mmap.offset == tuple(m.offset for m in mmap)

    def test_mixed_map_iter_len(self, maps):
        assert tuple(m for m in op2.MixedMap(maps)) == maps
        assert len(op2.MixedMap(maps)) == len(maps)

    def test_mixed_map_eq_ne(self, maps):
        assert op2.MixedMap(maps) == op2.MixedMap(maps)
        assert not op2.MixedMap(maps) != op2.MixedMap(maps)
        mm1 = op2.MixedMap((maps[0], maps[1]))
        mm2 = op2.MixedMap((maps[1], maps[0]))
        assert mm1 != mm2 and not mm1 == mm2
        assert op2.MixedMap(maps) != maps[0] and not op2.MixedMap(maps) == maps[0]

    def test_mixed_map_repr_str(self, mmap):
        assert repr(mmap) == "MixedMap(%r)" % (mmap.split,)
        assert str(mmap) == "OP2 MixedMap composed of Maps: %s" % (mmap.split,)


class TestKernelAPI:

    def test_kernel_illegal_name(self):
        with pytest.raises(exceptions.NameTypeError):
            op2.Kernel("", name=2)

    def test_kernel_properties(self):
        k = op2.CStringLocalKernel("", "foo", accesses=(), dtypes=())
        assert k.name == "foo"

    def test_kernel_repr_str(self, set):
        k = op2.Kernel("static int foo() { return 0; }", 'foo')
        assert repr(k) == 'Kernel("""%s""", %r)' % (k.code, k.name)
        assert str(k) == "OP2 Kernel: %s" % k.name


class TestParLoopAPI:

    def test_illegal_kernel(self, set, dat, m_iterset_toset):
        with pytest.raises(exceptions.KernelTypeError):
            op2.par_loop('illegal_kernel', set, dat(op2.READ, m_iterset_toset))

    def test_illegal_iterset(self, dat, m_iterset_toset):
        with pytest.raises(exceptions.SetTypeError):
            op2.par_loop(op2.Kernel("", "k"), 'illegal_set', dat(op2.READ, m_iterset_toset))

    def test_illegal_dat_iterset(self):
        set1, set2 = op2.Set(2), op2.Set(3)
        dat = op2.Dat(op2.DataSet(set1, 1))
        map = op2.Map(set2, set1, 1, [0, 0, 0])
        with pytest.raises(exceptions.MapValueError):
            op2.ParLoop(op2.Kernel("void k() { }", "k"), set1, dat(op2.READ, map))

    @gpu
    def test_illegal_mat_iterset(self, gpu_op2, sparsity):
        m = op2.Mat(sparsity)
        rmap, cmap = sparsity.rcmaps[(0, 0)][0]
        with pytest.raises(exceptions.MapValueError):
            op2.par_loop(op2.Kernel("static void k() { }", "k"), op2.Set(2),
                         m(op2.INC, (rmap, cmap)))

    @gpu
    def test_empty_map_and_iterset(self, gpu_op2):
        s1, s2 = op2.Set(0), op2.Set(10)
        m = op2.Map(s1, s2, 3)
        d = op2.Dat(s2 ** 1, [0] * 10, dtype=int)
        op2.par_loop(op2.Kernel("static void k(int *x) {}", "k"), s1, d(op2.READ, m))

    @gpu
    def test_frozen_dats_cannot_use_different_access_mode(self, gpu_op2):
        s1, s2 = op2.Set(2), op2.Set(3)
        m = op2.Map(s1, s2, 3, [0] * 6)
        d = op2.Dat(s2 ** 1, [0] * 3, dtype=int)
        k = op2.Kernel("static void k(int *x) {}", "k")
        with d.frozen_halo(op2.INC):
            op2.par_loop(k, s1, d(op2.INC, m))
            with pytest.raises(RuntimeError):
                op2.par_loop(k, s1, d(op2.WRITE, m))

    def test_frozen_check_needs_no_device(self):
        s1, s2 = op2.Set(2), op2.Set(3)
        m = op2.Map(s1, s2, 3, [0] * 6)
        d = op2.Dat(s2 ** 1, [0] * 3, dtype=int)
        with d.frozen_halo(op2.INC):
            with pytest.raises(RuntimeError):
                op2.ParLoop(op2.Kernel("static void k(int *x) {}", "k"), s1, d(op2.WRITE, m))
        assert not d._halo_frozen


# ------------------------------------------- object caching (test_caching.py)
class TestObjectCaching:

    @pytest.fixture
    def base_set(self):
        return op2.Set(1)

    @pytest.fixture
    def base_set2(self):
        return op2.Set(1)

    @pytest.fixture
    def base_map(self, base_set):
        return op2.Map(base_set, base_set, 1, [0])

    @pytest.fixture
    def base_map2(self, base_set, base_set2):
        return op2.Map(base_set, base_set2, 1, [0])

    def test_set_and_map_identity(self, base_set, base_set2, base_map, base_map2):
        assert base_set is not base_set2 and base_set != base_set2 and not base_set == base_set2
        assert base_map is not base_map2 and base_map != base_map2 and not base_map == base_map2

    def test_dataset_cache(self, base_set, base_set2):
        assert base_set ** 2 is base_set ** 2
        d1 = base_set ** 1
        for other in (base_set ** 2, base_set2 ** 1):
            assert d1 is not other and d1 != other and not d1 == other

    @gpu
    def test_sparsity_cache_hit(self, gpu_op2, base_set, base_map):
        dsets = (base_set ** 1, base_set ** 1)
        sp = op2.Sparsity(dsets, [(base_map, base_map, None)])
        assert sp is op2.Sparsity(dsets, [(base_map, base_map, None)])
        mixed_set = op2.MixedSet([base_set, base_set])
        maps = op2.MixedMap([base_map, base_map])
        blocks = {(i, j): [(rm, cm, None)] for i, rm in enumerate(maps) for j, cm in enumerate(maps)}
        sp = op2.Sparsity((mixed_set ** 1, mixed_set ** 1), blocks)
        mixed_set2 = op2.MixedSet([base_set, base_set])
        maps2 = op2.MixedMap([base_map, base_map])
        blocks2 = {(i, j): [(rm, cm, None)] for i, rm in enumerate(maps2) for j, cm in enumerate(maps2)}
        sp2 = op2.Sparsity((mixed_set2 ** 1, mixed_set2 ** 1), blocks2)
        assert sp is sp2 and sp == sp2 and not sp != sp2

    @gpu
    def test_sparsity_cache_miss(self, gpu_op2, base_set, base_set2, base_map, base_map2):
        sp = op2.Sparsity((base_set ** 1, base_set ** 1), [(base_map, base_map, (op2.ALL,))])
        mixed_set = op2.MixedSet([base_set, base_set])
        maps2 = op2.MixedMap([base_map, base_map])
        sp2 = op2.Sparsity((mixed_set ** 1, mixed_set ** 1),
                           {(i, j): [(rm, cm, (op2.ALL,))] for i, rm in enumerate(maps2)
                            for j, cm in enumerate(maps2)})
        assert sp is not sp2 and sp != sp2
        sp3 = op2.Sparsity((base_set ** 1, base_set2 ** 1), [(base_map, base_map2, (op2.ALL,))])
        assert sp is not sp3 and sp != sp3


@gpu
class TestSparsityCache:

    @pytest.fixture
    def s2(cls):
        return op2.Set(5)

    @pytest.fixture
    def ds2(cls, s2):
        return op2.DataSet(s2, 1)

    @pytest.fixture
    def m1(cls, s2):
        return op2.Map(op2.Set(5), s2, 1, [0, 1, 2, 3, 4])

    @pytest.fixture
    def m2(cls, m1, s2):
        return op2.Map(m1.iterset, s2, 1, [1, 2, 3, 4, 0])

    def test_differing_maps_not_cached(self, gpu_op2, m1, m2, ds2):
        assert op2.Sparsity((ds2, ds2), [(m1, m1, None)]) is not \
            op2.Sparsity((ds2, ds2), [(m2, m2, None)])
        assert op2.Sparsity((ds2, ds2), [(m1, m2, None)]) is not \
            op2.Sparsity((ds2, ds2), [(m2, m1, None)])
        assert op2.Sparsity((ds2, ds2), [(m1, m1, None), (m2, m2, None)]) is not \
            op2.Sparsity((ds2, ds2), [(m2, m2, None), (m2, m2, None)])

    def test_same_maps_cached(self, gpu_op2, m1, m2, ds2):
        assert op2.Sparsity((ds2, ds2), [(m1, m1, None)]) is \
            op2.Sparsity((ds2, ds2), [(m1, m1, None)])
        assert op2.Sparsity((ds2, ds2), [(m1, m1, None), (m2, m2, None)]) is \
            op2.Sparsity((ds2, ds2), [(m1, m1, None), (m2, m2, None)])
        assert op2.Sparsity((ds2, ds2), [(m1, m1, None), (m2, m2, None)]) is \
            op2.Sparsity((ds2, ds2), [(m2, m2, None), (m1, m1, None)])


# ------------------------------------ test_globals.py, test_configuration.py
def test_global_operations():
    g1 = op2.Global(1, data=2.)
    g2 = op2.Global(1, data=5.)
    assert (g1 + g2).data == 7.
    assert (g2 - g1).data == 3.
    assert (-g2).data == -5.
    assert (g1 * g2).data == 10.
    g1 *= g2
    assert g1.data == 10.


def test_global_dat_version():
    g1 = op2.Global(1, data=1.)
    g2 = op2.Global(1, data=2.)
    assert g1.dat_version == 0 and g2.dat_version == 0
    d1 = g1.data
    assert g1.dat_version == 1 and g2.dat_version == 0
    g2.data[:] += 1
    assert g1.dat_version == 1 and g2.dat_version == 1
    g1.zero()
    assert g1.dat_version == 2 and g2.dat_version == 1
    g2.data = d1
    assert g1.dat_version == 2 and g2.dat_version == 2


def test_add_configuration_value():
    from pyop2_gb300.configuration import Configuration
    c = Configuration()
    c.reconfigure(foo='bar')
    assert c['foo'] == 'bar'


@pytest.mark.parametrize(('key', 'val'), [('debug', 'illegal'), ('log_level', 1.5)])
def test_configuration_illegal_types(key, val):
    from pyop2_gb300.configuration import Configuration
    c = Configuration()
    with pytest.raises(exceptions.ConfigurationError):
        c[key] = val
