"""API semantics that need no GPU: construction, validation and exceptions
(following test/unit/test_api.py), host accessors and save/load."""
import numpy as np
import pytest

from pyop2_gb300 import exceptions, op2


@pytest.fixture
def s():
    return op2.Set(5, "s")


def test_set_validation():
    with pytest.raises(exceptions.SizeTypeError):
        op2.Set("illegalsize")
    with pytest.raises(exceptions.NameTypeError):
        op2.Set(1, 2)
    with pytest.raises(exceptions.SizeTypeError):
        op2.Set((3, 2, 4))
    st = op2.Set((1, 3, 4))
    assert (st.core_size, st.size, st.total_size) == (1, 3, 4)
    assert st.core_part.size == 1 and st.owned_part.offset == 1 and st.owned_part.size == 2


def test_extruded_set_validation(s):
    with pytest.raises(exceptions.SizeTypeError):
        op2.ExtrudedSet(s, 1)
    with pytest.raises(TypeError):
        op2.ExtrudedSet(1, 3)
    e = op2.ExtrudedSet(s, 4)
    assert e.constant_layers and e.layers == 4 and e.parent is s
    v = op2.ExtrudedSet(s, [[0, 2]] * 5)
    assert not v.constant_layers
    with pytest.raises(exceptions.SizeTypeError):
        op2.ExtrudedSet(s, [[2, 2]] * 5)


def test_subset(s):
    with pytest.raises(exceptions.SubsetIndexOutOfBounds):
        op2.Subset(s, list(range(6)))
    with pytest.raises(exceptions.SubsetIndexOutOfBounds):
        op2.Subset(s, [-1])
    assert len(op2.Subset(s, []).indices) == 0
    ss = op2.Subset(s, [0, 4, 1, 1, 3])
    assert list(ss.indices) == [0, 1, 3, 4]
    assert list(s(0, 1).indices) == [0, 1]
    sss = op2.Subset(ss, [1, 2])      # indices into the subset
    assert list(sss.indices) == [1, 3] and sss.superset is s


def test_dataset(s):
    with pytest.raises(TypeError):
        op2.DataSet(s, "illegaldim")
    with pytest.raises(TypeError):
        op2.DataSet(s, (1, "illegaldim"))
    assert op2.DataSet(s).dim == (1,)
    d = op2.DataSet(s, (2, 3))
    assert d.dim == (2, 3) and d.cdim == 6 and d.set is s
    assert s ** 2 is s ** 2


def test_dat_construction(s):
    with pytest.raises(exceptions.DataSetTypeError):
        op2.Dat("illegalset", 1)
    with pytest.raises(exceptions.NameTypeError):
        op2.Dat(s ** 1, name=2)
    with pytest.raises(exceptions.DataTypeError):
        op2.Dat(s ** 1, dtype="illegal_type")
    with pytest.raises(exceptions.DataValueError):
        op2.Dat(s ** 1, [1] * 6)
    assert op2.Dat(s ** 1, [1.5] * 5, np.int32).dtype == np.int32
    d = op2.Dat(s ** 2, [1.0] * 10)
    assert d.data.shape == (5, 2) and d.dtype == np.float64
    with pytest.raises(exceptions.IndexValueError):
        d[1]
    assert d[0] is d
    assert d(op2.READ).map_ is None
    z = op2.Dat(s ** 0)
    assert z.shape == (5, 0) and z._data.size == 0
    assert not op2.Dat(s ** 1)._is_allocated


def test_dat_accessors_and_copy(s):
    d = op2.Dat(s, np.arange(5.0))
    x = d.data_ro
    with pytest.raises(ValueError):
        x[0] = 1
    d.data[0] = -100
    assert d.data_ro[0] == -100
    c = op2.Dat(d)
    assert np.all(c.data_ro == d.data_ro)
    d.zero()
    assert np.all(d.data_ro == 0) and c.data_ro[0] == -100


def test_dat_save_load(s, tmp_path):
    d = op2.Dat(s ** 2, np.arange(10.0))
    f = str(tmp_path / "dat")
    d.save(f)
    e = op2.Dat(s ** 2)
    e.load(f)
    assert np.all(e.data_ro == d.data_ro)


def test_map_validation(s):
    t = op2.Set(3)
    with pytest.raises(exceptions.SetTypeError):
        op2.Map("illegal", t, 1, [0] * 5)
    with pytest.raises(exceptions.ArityTypeError):
        op2.Map(s, t, "illegal", [0] * 5)
    with pytest.raises(exceptions.DataValueError):
        op2.Map(s, t, 2, [0] * 5)
    m = op2.Map(s, t, 2, np.zeros((5, 2)))
    assert m.values.shape == (5, 2) and m.arity == 2
    m.values[0, 0] = 1              # editable until the map is first used on the device
    d = op2.Dat(op2.Set(2))
    with pytest.raises(exceptions.MapValueError):
        d(op2.READ, m)


def test_access_modes(s):
    d = op2.Dat(s)
    g = op2.Global(1, 0.0)
    with pytest.raises(exceptions.ModeValueError):
        d("illegal")
    with pytest.raises(exceptions.ModeValueError):
        g(op2.WRITE)
    with pytest.raises(exceptions.ModeValueError):
        op2.Constant(1, 2.0)(op2.INC)
    assert int(op2.READ) == 1 and int(op2.MAX) == 6 and int(op2.ALL) == 4


def test_parloop_validation_before_any_device_work(s):
    """test_mismatching_iterset, test_mismatching_indset and
    test_uninitialized_map (test/unit/test_indirect_loop.py:109-129): refused
    on the host, before anything is uploaded or compiled."""
    indset = op2.Set(5)
    x = op2.Dat(indset, np.arange(5.0))
    with pytest.raises(exceptions.MapValueError):          # map iterset mismatch
        op2.par_loop(op2.Kernel("", "dummy"), s, x(op2.WRITE, op2.Map(op2.Set(5), indset, 1)))
    with pytest.raises(exceptions.MapValueError):          # toset mismatch
        op2.par_loop(op2.Kernel("", "dummy"), s, x(op2.WRITE, op2.Map(s, op2.Set(5), 1)))
    with pytest.raises(exceptions.MapValueError):          # uninitialised map
        op2.par_loop(op2.Kernel("static void k(double *x) {}", "k"), s,
                     x(op2.WRITE, op2.Map(s, indset, 1)))
    with pytest.raises(exceptions.SetTypeError):
        op2.par_loop(op2.Kernel("", "dummy"), "notaset", x(op2.WRITE))
    with pytest.raises(exceptions.KernelTypeError):
        op2.par_loop("notakernel", s, x(op2.WRITE))
    with pytest.raises(exceptions.MapValueError):          # direct arg on another set
        op2.par_loop(op2.Kernel("", "dummy"), s, op2.Dat(op2.Set(5))(op2.WRITE))


def test_global(s):
    g = op2.Global(2, (1, 2), np.int32, "g")
    assert g.dim == (2,) and g.cdim == 2 and list(g.data_ro) == [1, 2]
    g.data = (3, 4)
    assert list(g.data_ro) == [3, 4]
    h = op2.Global(g)
    assert list(h.data_ro) == [3, 4] and h.dtype == np.int32
    g.zero()
    assert list(g.data_ro) == [0, 0]


def test_kernel_rejects_host_only_options():
    with pytest.raises(NotImplementedError):
        op2.Kernel("static void k(double *x) {}", "k", user_code="srandom(1);")
    with pytest.raises(TypeError):
        op2.Kernel(42, "k")


def test_configuration():
    from pyop2_gb300.configuration import configuration
    from pyop2_gb300.exceptions import ConfigurationError
    configuration["no_such_key"] = 1           # other keys are stored (as the reference does)
    assert configuration["no_such_key"] == 1
    with pytest.raises(ConfigurationError):
        configuration["debug"] = "yes"          # known keys are type-checked
    with pytest.raises(ConfigurationError):
        configuration["scatter"] = "sometimes"
    op2.init(debug=False, scatter="atomic")
    assert op2.initialised()


def test_mpi_and_halo_stand_ins():
    """op2.MPI and op2.Halo, as exported by the reference (pyop2/op2.py:61-68):
    single-rank communicators whose collectives return their input, and the
    abstract Halo base class."""
    import pytest
    from pyop2_gb300 import op2
    w = op2.MPI.COMM_WORLD
    assert (w.rank, w.size, w.Get_rank(), w.Get_size()) == (0, 1, 0, 1)
    assert w.allreduce(3.5) == 3.5 and w.bcast({"a": 1}) == {"a": 1} and w.allgather(2) == [2]
    assert op2.MPI.internal_comm(None) is w and op2.MPI.is_pyop2_comm(op2.MPI.COMM_SELF)
    s = op2.Set(5, "s", comm=w)
    assert s.comm is w
    with pytest.raises(TypeError):
        op2.Halo()

    class MyHalo(op2.Halo):
        comm = w
        local_to_global_numbering = None

        def global_to_local_begin(self, dat, insert_mode):
            pass

        def global_to_local_end(self, dat, insert_mode):
            pass

        def local_to_global_begin(self, dat, insert_mode):
            pass

        def local_to_global_end(self, dat, insert_mode):
            pass

    assert isinstance(MyHalo(), op2.Halo)


def test_map_serials_are_never_reused():
    """Colouring plans are cached per map serial: a map created after another
    was freed (which may reuse its id()) still gets a new serial."""
    import gc
    from pyop2_gb300 import op2
    s, t = op2.Set(4), op2.Set(3)
    seen = set()
    for _ in range(50):
        m = op2.Map(s, t, 1, [0, 1, 2, 0])
        assert m._serial not in seen
        seen.add(m._serial)
        assert m._serial == m._serial
        del m
        gc.collect()
    pm = op2.PermutedMap(op2.Map(s, t, 1, [0, 1, 2, 0]), [0])
    assert pm._serial not in seen
