"""test/unit/test_dats.py: copies, nbytes, save/load, versioning (including
the vector views), and DatView -- on the CPU where no loop runs, on the GPU
where one does."""
import numpy as np
import pytest

from pyop2_gb300 import op2

NEL = 5
gpu = pytest.mark.gpu


@pytest.fixture
def s():
    return op2.Set(NEL)


@pytest.fixture
def d1(s):
    return op2.Dat(s, list(range(NEL)), dtype=np.float64)


@pytest.fixture
def vdat(s):
    return op2.Dat(op2.DataSet(s, 2), np.zeros(2 * NEL), dtype=np.float64)


def test_copy_constructor(d1):
    d2 = op2.Dat(d1)
    assert d1.dataset.set == d2.dataset.set and (d1.data_ro == d2.data_ro).all()
    d1.data[:] = -1
    assert (d1.data_ro != d2.data_ro).all()


def test_copy(s, d1):
    d2 = op2.Dat(s)
    d1.copy(d2)
    assert d1.dataset.set == d2.dataset.set and (d1.data_ro == d2.data_ro).all()
    d1.data[:] = -1
    assert (d1.data_ro != d2.data_ro).all()


def test_copy_subset(s, d1):
    d2 = op2.Dat(s)
    ss = op2.Subset(s, list(range(1, NEL, 2)))
    d1.copy(d2, subset=ss)
    assert (d1.data_ro[ss.indices] == d2.data_ro[ss.indices]).all()
    assert (d2.data_ro[::2] == 0).all()


@pytest.mark.parametrize('dim', [1, 2])
def test_dat_nbytes(dim):
    assert op2.Dat(op2.Set(10) ** dim).nbytes == 10 * 8 * dim


def test_dat_save_and_load(tmp_path, d1, s):
    out = str(tmp_path / 'output')
    d1.save(out)
    d2 = op2.Dat(s)
    d2.load(out)
    assert (d1.data_ro == d2.data_ro).all()


def test_dat_version_host(s, d1):
    d2 = op2.Dat(s)
    assert d1.dat_version == 0 and d2.dat_version == 0
    d1.data
    assert d1.dat_version == 1 and d2.dat_version == 0
    d2.data[:] += 1
    assert d1.dat_version == 1 and d2.dat_version == 1
    d1.zero()
    assert d1.dat_version == 2 and d2.dat_version == 1
    d2.copy(d1)
    assert d1.dat_version == 3 and d2.dat_version == 1


@gpu
def test_dat_version_vec_and_parloop(gpu_op2, s, d1):
    d2 = op2.Dat(s)
    d1.data
    d2.data[:] += 1
    d1.zero()
    d2.copy(d1)
    assert d1.dat_version == 3 and d2.dat_version == 1
    # entering and leaving the vector views changes nothing
    with d1.vec_wo as _:
        pass
    with d2.vec as _:
        pass
    assert d1.dat_version == 3 and d2.dat_version == 1
    # modifying through them does
    with d1.vec_wo as x:
        x += 1
    with d2.vec as x:
        x += 1
    assert d1.dat_version == 4 and d2.dat_version == 2
    assert (d1.data_ro == 2).all() and (d2.data_ro == 2).all()
    d3 = op2.Dat(s ** 1, data=None, dtype=np.uint32)
    assert d3.dat_version == 0
    op2.par_loop(op2.Kernel("static void write(unsigned int* v) { *v = 1; }", "write"), s,
                 d3(op2.WRITE))
    assert d3.dat_version == 1


def test_accessing_data_with_halos_increments_dat_version(d1):
    assert d1.dat_version == 0
    d1.data_ro_with_halos
    assert d1.dat_version == 0
    d1.data_with_halos
    assert d1.dat_version == 1


class TestDatView:

    def test_dat_view_assign(self, vdat):
        vdat.data[:, 0] = 3
        vdat.data[:, 1] = 4
        comp = op2.DatView(vdat, 1)
        comp.data[:] = 7
        assert not vdat.halo_valid and not comp.halo_valid
        expected = np.zeros_like(vdat.data)
        expected[:, 0] = 3
        expected[:, 1] = 7
        assert all(comp.data == expected[:, 1])
        assert all(vdat.data[:, 0] == expected[:, 0]) and all(vdat.data[:, 1] == expected[:, 1])

    @gpu
    def test_dat_view_zero(self, gpu_op2, vdat):
        vdat.data[:, 0] = 3
        vdat.data[:, 1] = 4
        comp = op2.DatView(vdat, 1)
        comp.zero()
        assert vdat.halo_valid and comp.halo_valid
        assert all(comp.data == 0)
        assert all(vdat.data[:, 0] == 3) and all(vdat.data[:, 1] == 0)

    def test_dat_view_halo_valid(self, vdat):
        comp = op2.DatView(vdat, 1)
        assert vdat.halo_valid and comp.halo_valid
        assert vdat.dat_version == 0 and comp.dat_version == 0
        comp.data_ro_with_halos
        assert vdat.halo_valid and comp.halo_valid
        assert vdat.dat_version == 0 and comp.dat_version == 0
        comp.data_with_halos
        assert not vdat.halo_valid and not comp.halo_valid
        assert vdat.dat_version == 1 and comp.dat_version == 1

    def test_dat_view_index_checked(self, vdat):
        from pyop2_gb300.exceptions import IndexValueError
        with pytest.raises(IndexValueError):
            op2.DatView(vdat, 2)


@gpu
class TestDatViewInLoops:
    """A DatView in a par_loop: the kernel sees one component (dim 1) of a
    vector Dat, read or written, directly or through a map."""

    def test_direct_view(self, gpu_op2):
        s = op2.Set(100)
        v = op2.Dat(s ** (2, 3), np.arange(600.0))
        out = op2.Dat(s)
        comp = op2.DatView(v, (1, 2))
        op2.par_loop(op2.Kernel("static void k(double *o, const double *c) { o[0] = 2 * c[0]; }",
                                "k"), s, out(op2.WRITE), comp(op2.READ))
        assert np.array_equal(out.data_ro, 2 * v.data_ro[:, 1, 2])
        op2.par_loop(op2.Kernel("static void w(double *c) { c[0] = -1.0; }", "w"), s,
                     comp(op2.WRITE))
        full = v.data_ro
        assert (full[:, 1, 2] == -1).all()
        ref = np.arange(600.0).reshape(100, 2, 3)
        mask = np.ones((2, 3), bool)
        mask[1, 2] = False
        assert np.array_equal(full[:, mask], ref[:, mask])

    @pytest.mark.parametrize("scatter", ["atomic", "warp", "colour", "shared", "staged"])
    def test_indirect_view_inc_and_read(self, gpu_op2, scatter):
        from pyop2_gb300.configuration import configuration
        old = configuration["scatter"]
        configuration["scatter"] = scatter
        try:
            cells, verts = op2.Set(300), op2.Set(120)
            rng = np.random.default_rng(2)
            vals = rng.integers(0, 120, (300, 3)).astype(np.int32)
            m = op2.Map(cells, verts, 3, vals)
            src = op2.Dat(verts ** 3, rng.uniform(-1, 1, (120, 3)))
            acc = op2.Dat(verts ** 3, np.zeros((120, 3)))
            op2.par_loop(op2.Kernel("""static void k(double *a, const double *x) {
                for (int i = 0; i < 3; ++i) a[i] += x[i]; }""", "k"), cells,
                op2.DatView(acc, 1)(op2.INC, m), op2.DatView(src, 2)(op2.READ, m))
        finally:
            configuration["scatter"] = old
        expect = np.zeros((120, 3))
        np.add.at(expect[:, 1], vals.reshape(-1), src.data_ro[vals.reshape(-1), 2])
        out = acc.data_ro
        assert np.max(np.abs(out - expect)) <= 1e-12
