"""test/unit/test_subset.py: direct and indirect loops over Subsets (and
subsets of subsets), Mat assembly over subsets, set algebra."""
import numpy as np
import pytest

NEL = 32
gpu = pytest.mark.gpu
INC = "static void inc(unsigned int* v) { *v += 1; }"


@pytest.fixture(params=[(NEL, NEL, NEL), (0, NEL, NEL), (NEL // 2, NEL, NEL)])
def iterset(request, gpu_op2):
    return gpu_op2.Set(request.param, "iterset")


@gpu
class TestSubSet:

    def test_direct_loop(self, gpu_op2, iterset):
        op2 = gpu_op2
        indices = np.arange(0, NEL, 2, dtype=np.int32)
        d = op2.Dat(iterset ** 1, data=None, dtype=np.uint32)
        op2.par_loop(op2.Kernel(INC, "inc"), op2.Subset(iterset, indices), d(op2.RW))
        inds, = np.where(d.data)
        assert (inds == indices).all()

    def test_direct_loop_empty(self, gpu_op2, iterset):
        op2 = gpu_op2
        d = op2.Dat(iterset ** 1, data=None, dtype=np.uint32)
        op2.par_loop(op2.Kernel(INC, "inc"), op2.Subset(iterset, []), d(op2.RW))
        assert not d.data.any()

    @pytest.mark.parametrize("by_call", [False, True])
    def test_direct_complementary_subsets(self, gpu_op2, iterset, by_call):
        """by_call=True is test_direct_complementary_subsets_with_indexing."""
        op2 = gpu_op2
        even, odd = np.arange(0, NEL, 2, dtype=np.int32), np.arange(1, NEL, 2, dtype=np.int32)
        mk = iterset if by_call else (lambda idx: op2.Subset(iterset, idx))
        d = op2.Dat(iterset ** 1, data=None, dtype=np.uint32)
        k = op2.Kernel(INC, "inc")
        op2.par_loop(k, mk(even), d(op2.RW))
        op2.par_loop(k, mk(odd), d(op2.RW))
        assert (d.data == 1).all()

    @pytest.mark.parametrize("by_call", [False, True])
    def test_direct_loop_sub_subset(self, gpu_op2, iterset, by_call):
        """by_call=True is test_direct_loop_sub_subset_with_indexing."""
        op2 = gpu_op2
        k = op2.Kernel(INC, "inc")
        ss = iterset(np.arange(0, NEL, 2, dtype=np.int32)) if by_call else \
            op2.Subset(iterset, np.arange(0, NEL, 2, dtype=np.int32))
        idx = np.arange(0, NEL // 2, 2, dtype=np.int32)
        sss = ss(idx) if by_call else op2.Subset(ss, idx)
        d = op2.Dat(iterset ** 1, data=None, dtype=np.uint32)
        op2.par_loop(k, sss, d(op2.RW))
        d2 = op2.Dat(iterset ** 1, data=None, dtype=np.uint32)
        op2.par_loop(k, op2.Subset(iterset, np.arange(0, NEL, 4, dtype=np.int32)), d2(op2.RW))
        assert (d.data == d2.data).all()

    def test_indirect_loop(self, gpu_op2, iterset):
        op2 = gpu_op2
        ss = op2.Subset(iterset, np.arange(0, NEL, 2, dtype=np.int32))
        indset = op2.Set(2, "indset")
        map = op2.Map(iterset, indset, 1, [(1 if i % 2 else 0) for i in range(NEL)])
        d = op2.Dat(indset ** 1, data=None, dtype=np.uint32)
        op2.par_loop(op2.Kernel("static void inc(unsigned int* v) { *v += 1;}", "inc"), ss,
                     d(op2.INC, map))
        assert d.data[0] == NEL // 2

    def test_indirect_loop_empty(self, gpu_op2, iterset):
        op2 = gpu_op2
        indset = op2.Set(2, "indset")
        map = op2.Map(iterset, indset, 1, [(1 if i % 2 else 0) for i in range(NEL)])
        d = op2.Dat(indset ** 1, data=None, dtype=np.uint32)
        d.data[:] = 0
        op2.par_loop(op2.Kernel("static void inc(unsigned int* v) { *v += 1;}", "inc"),
                     op2.Subset(iterset, []), d(op2.INC, map))
        assert (d.data == 0).all()

    def test_indirect_loop_with_direct_dat(self, gpu_op2, iterset):
        op2 = gpu_op2
        ss = op2.Subset(iterset, np.arange(0, NEL, 2, dtype=np.int32))
        indset = op2.Set(2, "indset")
        map = op2.Map(iterset, indset, 1, [(1 if i % 2 else 0) for i in range(NEL)])
        values = [2976579765] * NEL
        values[::2] = [i // 2 for i in range(NEL)][::2]
        dat1 = op2.Dat(iterset ** 1, data=values, dtype=np.uint32)
        dat2 = op2.Dat(indset ** 1, data=None, dtype=np.uint32)
        op2.par_loop(op2.Kernel("static void inc(unsigned* d, unsigned int* s) { *d += *s;}",
                                "inc"), ss, dat2(op2.INC, map), dat1(op2.READ))
        assert dat2.data[0] == sum(values[::2])

    def test_complementary_subsets(self, gpu_op2, iterset):
        op2 = gpu_op2
        even, odd = np.arange(0, NEL, 2, dtype=np.int32), np.arange(1, NEL, 2, dtype=np.int32)
        indset = op2.Set(NEL, "indset")
        map = op2.Map(iterset, indset, 1, list(range(NEL)))
        dat1 = op2.Dat(iterset ** 1, data=None, dtype=np.uint32)
        dat2 = op2.Dat(indset ** 1, data=None, dtype=np.uint32)
        k = op2.Kernel("""static void inc(unsigned int* v1, unsigned int* v2) {
          *v1 += 1; *v2 += 1; }""", "inc")
        op2.par_loop(k, op2.Subset(iterset, even), dat1(op2.RW), dat2(op2.INC, map))
        op2.par_loop(k, op2.Subset(iterset, odd), dat1(op2.RW), dat2(op2.INC, map))
        assert np.sum(dat1.data) == NEL and np.sum(dat2.data) == NEL

    def test_matrix(self, gpu_op2):
        op2 = gpu_op2
        iterset, idset, indset = op2.Set(2), op2.Set(2), op2.Set(4)
        ss01, ss10 = op2.Subset(iterset, [0, 1]), op2.Subset(iterset, [1, 0])
        dat = op2.Dat(idset ** 1, data=[0, 1], dtype=np.float64)
        map = op2.Map(iterset, indset, 4, [0, 1, 2, 3, 0, 1, 2, 3])
        idmap = op2.Map(iterset, idset, 1, [0, 1])
        sparsity = op2.Sparsity((indset ** 1, indset ** 1), {(0, 0): [(map, map, None)]})
        mats = [op2.Mat(sparsity, np.float64) for _ in range(3)]
        k = op2.Kernel("""static void unique_id(double mat[4][4], double *dat) {
          for (int i=0; i<4; ++i)
            for (int j=0; j<4; ++j)
              mat[i][j] += (*dat)*16+i*4+j; }""", "unique_id")
        for m, its in zip(mats, (iterset, ss01, ss10)):
            m.zero()
            op2.par_loop(k, its, m(op2.INC, (map, map)), dat(op2.READ, idmap))
            m.assemble()
        assert (mats[1].values == mats[0].values).all()
        assert (mats[2].values == mats[0].values).all()


class TestSetOperations:

    def test_set_set_operations(self):
        from pyop2_gb300 import op2
        a = op2.Set(10)
        assert a.union(a) is a and a.intersection(a) is a
        assert a.difference(a)._indices.size == 0
        assert a.symmetric_difference(a)._indices.size == 0

    def test_set_subset_operations(self):
        from pyop2_gb300 import op2
        a = op2.Set(10)
        b = op2.Subset(a, np.array([2, 3, 5, 7], dtype=np.int32))
        assert a.union(b) is a and a.intersection(b) is b
        d = a.difference(b)
        assert (d._indices == [0, 1, 4, 6, 8, 9]).all()
        assert (a.symmetric_difference(b)._indices == d._indices).all()

    def test_subset_set_operations(self):
        from pyop2_gb300 import op2
        a = op2.Set(10)
        b = op2.Subset(a, np.array([2, 3, 5, 7], dtype=np.int32))
        assert b.union(a) is a and b.intersection(a) is b
        assert b.difference(a)._indices.size == 0
        assert (b.symmetric_difference(a)._indices == [0, 1, 4, 6, 8, 9]).all()

    def test_subset_subset_operations(self):
        from pyop2_gb300 import op2
        a = op2.Set(10)
        b = op2.Subset(a, np.array([2, 3, 5, 7], dtype=np.int32))
        c = op2.Subset(a, np.array([2, 4, 6, 8], dtype=np.int32))
        assert (b.union(c)._indices == [2, 3, 4, 5, 6, 7, 8]).all()
        assert (b.intersection(c)._indices == [2]).all()
        assert (b.difference(c)._indices == [3, 5, 7]).all()
        assert (b.symmetric_difference(c)._indices == [3, 4, 5, 6, 7, 8]).all()
