"""oracle.op2 -- TEST INFRASTRUCTURE ONLY: the parity oracle.

A small, independent CPU implementation of the PyOP2 API used to check
pyop2_gb300.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline import it; the product never does.

It restates the reference's sequential backend:
  * the per-signature C wrapper of pyop2/codegen/builder.py:683-989 --
    for n in [start, end): pack every argument (pyop2/codegen/builder.py:
    240-300 GlobalPack, 303-410 DatPack, 501-606 MatPack), call the kernel,
    unpack -- generated here as C text and compiled with gcc, exactly as the
    reference compiles its loopy output (pyop2/compilation.py:324-328);
  * Global INC through a zeroed temporary added at the end
    (pyop2/parloop.py:274-277, 449-452, 514-530); MIN/MAX packs start from
    the current value (pyop2/codegen/builder.py:275-278);
  * extruded layer loops and offsets (pyop2/codegen/builder.py:81-125,
    742-812);
  * the sparsity of pyop2/sparsity.pyx (oracle/sparsity.c) and PETSc's
    MatSetValuesBlockedLocal ADD/INSERT on the preallocated pattern.
Execution is strictly sequential in entity order, so INC sums happen in the
reference's order.
"""
import ctypes
import hashlib
import os
import subprocess
import threading

import numpy as np

from oracle import build as _build

READ, WRITE, RW, INC, MIN, MAX = 1, 2, 3, 4, 5, 6
ON_BOTTOM, ON_TOP, ON_INTERIOR_FACETS, ALL = 1, 2, 3, 4

_CTYPE = {"float64": "double", "float32": "float", "int32": "int", "uint32": "unsigned int",
          "int64": "long long", "uint64": "unsigned long long", "int16": "short",
          "uint16": "unsigned short", "int8": "signed char", "uint8": "unsigned char"}

# "parity": strict IEEE (no contraction) so results are reproducible;
# "timing": the reference's JIT flags (pyop2/compilation.py:324-328).
PROFILES = {
    "parity": ["-O2", "-ffp-contract=off"],
    "timing": ["-O3", "-march=native", "-ffast-math"],
}


# ------------------------------------------------------------------- sets
class Set:
    _extruded = False

    def __init__(self, size, name=None):
        if isinstance(size, (int, np.integer)):
            size = (size, size, size)
        self.sizes = tuple(int(s) for s in size)
        self.name = name

    @property
    def size(self):
        return self.sizes[1]

    @property
    def total_size(self):
        return self.sizes[2]

    def __pow__(self, dim):
        return DataSet(self, dim)


class ExtrudedSet(Set):
    _extruded = True

    def __init__(self, parent, layers, periodic=False, extruded_periodic=None):
        if extruded_periodic is not None:
            periodic = extruded_periodic
        self.parent = parent
        self.sizes = parent.sizes
        lay = np.asarray(layers, dtype=np.int32)
        if lay.ndim == 0:
            self.constant_layers = True
            lay = np.array([[0, int(lay)]], dtype=np.int32)
        else:
            self.constant_layers = False
            lay = lay.reshape(parent.total_size, 2)
        self.layers_array = np.ascontiguousarray(lay)
        self.periodic = periodic


class Subset:
    def __init__(self, superset, indices):
        self.superset = superset
        self.indices = np.ascontiguousarray(np.unique(np.asarray(indices)), dtype=np.int32)
        self._extruded = superset._extruded

    @property
    def size(self):
        return len(self.indices)

    def __getattr__(self, k):
        if k.startswith("__"):
            raise AttributeError(k)
        return getattr(self.superset, k)


class DataSet:
    def __init__(self, set_, dim, name=None):
        self.set = set_
        self.dim = (dim,) if isinstance(dim, (int, np.integer)) else tuple(dim)
        self.cdim = int(np.prod(self.dim))


class MixedSet:
    """Tuple of Sets (pyop2/types/set.py:540-662)."""

    def __init__(self, sets):
        self.split = tuple(sets)

    def __iter__(self):
        return iter(self.split)

    def __len__(self):
        return len(self.split)

    def __getitem__(self, i):
        return self.split[i]

    def __pow__(self, dim):
        return MixedDataSet([s ** dim for s in self.split])


class MixedDataSet:
    """Tuple of DataSets (pyop2/types/dataset.py:304-460)."""

    def __init__(self, dsets, dims=None):
        if dims is not None:
            sets = dsets.split if isinstance(dsets, MixedSet) else tuple(dsets)
            dims = (dims,) * len(sets) if isinstance(dims, int) else tuple(dims)
            dsets = [DataSet(s, d) for s, d in zip(sets, dims)]
        self.split = tuple(d if isinstance(d, DataSet) else DataSet(d, 1) for d in dsets)

    def __iter__(self):
        return iter(self.split)

    def __len__(self):
        return len(self.split)

    def __getitem__(self, i):
        return self.split[i]


def _same_space(a, b):
    """Row and column spaces coincide (the reference compares DataSets)."""
    if a is b:
        return True
    sa = a.split if isinstance(a, MixedDataSet) else (a,)
    sb = b.split if isinstance(b, MixedDataSet) else (b,)
    return len(sa) == len(sb) and all(x.set is y.set and x.dim == y.dim for x, y in zip(sa, sb))


# ------------------------------------------------------------------- maps
class Map:
    def __init__(self, iterset, toset, arity, values, name=None, offset=None,
                 offset_quotient=None):
        self.iterset = iterset
        self.toset = toset
        self.arity = int(arity)
        self.values = np.ascontiguousarray(np.asarray(values, dtype=np.int32).reshape(
            iterset.total_size, arity))
        self.offset = None if offset is None else np.ascontiguousarray(offset, dtype=np.int32)
        self.offset_quotient = None if offset_quotient is None else \
            np.ascontiguousarray(offset_quotient, dtype=np.int32)


class PermutedMap:
    def __init__(self, map_, permutation):
        self.map_ = map_
        self.permutation = np.asarray(permutation, dtype=np.int32)
        self.arity = map_.arity
        self.iterset, self.toset = map_.iterset, map_.toset
        self.offset, self.offset_quotient = map_.offset, map_.offset_quotient


class ComposedMap:
    def __init__(self, *maps_):
        self.maps_ = maps_
        flat = []
        for m in maps_:
            flat.extend(m.flat if isinstance(m, ComposedMap) else [m])
        self.flat = flat
        self.arity = maps_[0].arity
        self.iterset, self.toset = maps_[-1].iterset, maps_[0].toset
        self.offset = flat[0].offset
        self.offset_quotient = flat[0].offset_quotient


class MixedMap:
    """Tuple of Maps from one iteration set (pyop2/types/map.py:297-434)."""

    def __init__(self, maps):
        self.split = tuple(maps)
        self.iterset = self.split[0].iterset

    def __iter__(self):
        return iter(self.split)

    def __len__(self):
        return len(self.split)

    def __getitem__(self, i):
        return self.split[i]


# ------------------------------------------------------------------- data
class Dat:
    def __init__(self, dataset, data=None, dtype=None, name=None):
        if isinstance(dataset, Set):
            dataset = DataSet(dataset, 1)
        self.dataset = dataset
        shape = (dataset.set.total_size,) + (() if dataset.cdim == 1 else dataset.dim)
        if data is None:
            self.data = np.zeros(shape, dtype=dtype or np.float64)
        else:
            self.data = np.array(np.asarray(data, dtype=dtype).reshape(shape), copy=True)
        self.cdim = dataset.cdim

    def __call__(self, access, map_=None):
        return ("dat", self, access, map_)

    @property
    def data_ro(self):
        return self.data

    def zero(self):
        self.data[...] = 0


class MixedDat:
    """Tuple of Dats (pyop2/types/dat.py:787-1151); accessed through a
    MixedMap as one kernel argument."""

    def __init__(self, items):
        items = items.split if isinstance(items, (MixedSet, MixedDataSet)) else items
        self.split = tuple(d if isinstance(d, Dat) else Dat(d) for d in items)

    def __iter__(self):
        return iter(self.split)

    def __len__(self):
        return len(self.split)

    def __getitem__(self, i):
        return self.split[i]

    def __call__(self, access, map_):
        return ("mdat", self.split, access, tuple(map_))

    @property
    def data(self):
        return tuple(d.data for d in self.split)

    @property
    def data_ro(self):
        return self.data


class Global:
    def __init__(self, dim, data=None, dtype=None, name=None, comm=None):
        self.dim = int(np.prod(dim))
        self._data = np.zeros(self.dim, dtype=dtype or np.float64) if data is None else \
            np.array(np.asarray(data, dtype=dtype).reshape(self.dim), copy=True)

    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, v):
        self._data[:] = v

    @property
    def data_ro(self):
        return self._data

    def __call__(self, access):
        return ("glob", self, access, None)


class Kernel:
    def __init__(self, code, name, headers=()):
        self.code = "\n".join(list(headers) + [code])
        self.name = name


# ------------------------------------------------------------- sparsity/mat
class _Pair(ctypes.Structure):
    _fields_ = [("rmap", ctypes.c_void_p), ("cmap", ctypes.c_void_p), ("rarity", ctypes.c_int32),
                ("carity", ctypes.c_int32), ("nent", ctypes.c_int64), ("region", ctypes.c_int32),
                ("nrc", ctypes.c_int32), ("ncc", ctypes.c_int32), ("rc", ctypes.c_void_p * 8),
                ("cc", ctypes.c_void_p * 8), ("roff", ctypes.c_void_p), ("coff", ctypes.c_void_p),
                ("rq", ctypes.c_void_p), ("cq", ctypes.c_void_p)]


class _Sp(ctypes.Structure):
    _fields_ = [("nrows", ctypes.c_int64), ("ncols", ctypes.c_int64), ("set_diag", ctypes.c_int32),
                ("extruded", ctypes.c_int32), ("constant_layers", ctypes.c_int32),
                ("periodic", ctypes.c_int32), ("layers", ctypes.c_void_p), ("npairs", ctypes.c_int32),
                ("pairs", ctypes.POINTER(_Pair))]


def _outer_values(m):
    """(values array of the outermost map with any permutation applied, chain)."""
    flat = m.flat if isinstance(m, ComposedMap) else [m]
    o = flat[0]
    if isinstance(o, PermutedMap):
        vals = np.ascontiguousarray(o.map_.values[:, o.permutation])
    else:
        vals = o.values
    chain = [(c.map_ if isinstance(c, PermutedMap) else c).values for c in flat[1:]]
    return vals, chain, o


class Sparsity:
    """Block pattern from (rmap, cmap, regions) triples (oracle/sparsity.c).

    Between MixedDataSets the sparsity is a grid of block sparsities, block
    (i, j) built from ``maps_and_regions[(i, j)]`` with the diagonal on
    i == j when the row and column spaces coincide (pyop2/types/mat.py:86-95,
    pyop2/sparsity.pyx:144-159).  ``nnz`` is the tuple of the blocks' counts
    when nested, else the dof-row counts of the whole (blocks of a block row
    side by side)."""

    def __init__(self, dsets, maps_and_regions, block_sparse=True, diagonal_block=True,
                 nest=True):
        if isinstance(dsets[0], MixedDataSet) or isinstance(dsets[1], MixedDataSet):
            self._init_mixed(dsets, maps_and_regions, block_sparse, diagonal_block, nest)
            return
        if isinstance(maps_and_regions, dict):
            maps_and_regions = maps_and_regions.get((0, 0), [])
        self.shape = (1, 1)
        rds, cds = dsets
        self.dsets = dsets
        self.dims = (rds.cdim, cds.cdim)
        self.block_sparse = block_sparse
        set_diag = (rds is cds or (rds.set is cds.set and rds.dim == cds.dim)) and diagonal_block
        keep = []
        triples = []
        for rmap, cmap, regions in maps_and_regions:
            for reg in (regions or (ALL,)):
                triples.append((rmap, cmap, int(reg)))
        pairs = (_Pair * max(1, len(triples)))()
        extr = False
        const = 1
        periodic = 0
        layers = None
        for k, (rmap, cmap, reg) in enumerate(triples):
            P = pairs[k]
            it = rmap.iterset
            for side, m in (("r", rmap), ("c", cmap)):
                vals, chain, outer = _outer_values(m)
                keep.append(vals)
                setattr(P, side + "map", vals.ctypes.data)
                setattr(P, side + "arity", m.arity)
                arr = getattr(P, side + "c")
                for i, c in enumerate(chain):
                    keep.append(c)
                    arr[i] = c.ctypes.data
                setattr(P, "n" + side + "c", len(chain))
                if it._extruded:
                    off = outer.offset if outer.offset is not None else np.zeros(m.arity, np.int32)
                    q = outer.offset_quotient
                    if isinstance(outer, PermutedMap):
                        off = off[outer.permutation]
                        q = None if q is None else q[outer.permutation]
                    off = np.ascontiguousarray(off, dtype=np.int32)
                    keep.append(off)
                    setattr(P, side + "off", off.ctypes.data)
                    if q is not None:
                        q = np.ascontiguousarray(q, dtype=np.int32)
                        keep.append(q)
                        setattr(P, side + "q", q.ctypes.data)
            P.nent = it.size
            P.region = reg
            if it._extruded:
                extr = True
                const = 1 if it.constant_layers else 0
                periodic = 1 if it.periodic else 0
                layers = it.layers_array
        S = _Sp(rds.set.size, cds.set.size, 1 if set_diag else 0, 1 if extr else 0, const,
                periodic, layers.ctypes.data if layers is not None else None, len(triples), pairs)
        lib = _build.liboracle()
        # full prototypes: without them ctypes passes a Python int as a C int,
        # truncating any address above 2^31
        lib.oracle_sparsity_build.argtypes = [
            ctypes.POINTER(_Sp), ctypes.c_void_p,
            ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)), ctypes.POINTER(ctypes.c_int64)]
        lib.oracle_free.argtypes = [ctypes.c_void_p]
        rowptr = np.zeros(S.nrows + 1, dtype=np.int64)
        col = ctypes.POINTER(ctypes.c_int32)()
        nnz = ctypes.c_int64()
        rc = lib.oracle_sparsity_build(ctypes.byref(S), rowptr.ctypes.data, ctypes.byref(col),
                                       ctypes.byref(nnz))
        if rc != 0:
            raise ValueError("oracle sparsity build failed (%d)" % rc)
        self.rowptr = rowptr
        self.colidx = np.ctypeslib.as_array(col, shape=(max(nnz.value, 1),))[:nnz.value].copy()
        lib.oracle_free(col)
        counts = np.diff(rowptr).astype(np.int32)
        rdim, cdim = self.dims
        if not (block_sparse and rdim == cdim):
            counts = np.repeat(counts * cdim, rdim).astype(np.int32)
        self.nnz = counts

    def _init_mixed(self, dsets, maps_and_regions, block_sparse, diagonal_block, nest):
        rsets = dsets[0].split if isinstance(dsets[0], MixedDataSet) else (dsets[0],)
        csets = dsets[1].split if isinstance(dsets[1], MixedDataSet) else (dsets[1],)
        self.dsets = dsets
        self.shape = (len(rsets), len(csets))
        same = _same_space(dsets[0], dsets[1])
        self.blocks = [[Sparsity((r, c), maps_and_regions.get((i, j), []),
                                 block_sparse=block_sparse,
                                 diagonal_block=(i == j and same and (nest or diagonal_block)))
                        for j, c in enumerate(csets)] for i, r in enumerate(rsets)]
        if nest:
            self.nnz = tuple(b.nnz for row in self.blocks for b in row)
        else:
            rows = []
            for i, row in enumerate(self.blocks):
                acc = np.zeros(rsets[i].set.size, dtype=np.int64)
                for j, b in enumerate(row):
                    acc += np.diff(b.rowptr) * csets[j].cdim
                rows.append(np.repeat(acc, rsets[i].cdim))
            self.nnz = np.concatenate(rows).astype(np.int32)

    def __getitem__(self, ij):
        i, j = ij
        return self.blocks[i][j]


class Mat:
    """Block-CSR values on an oracle Sparsity (row-major blocks)."""

    def __init__(self, sparsity):
        self.sparsity = sparsity
        if sparsity.shape != (1, 1):
            self.blocks = [[Mat(b) for b in row] for row in sparsity.blocks]
            return
        self.blocks = [[self]]
        rdim, cdim = sparsity.dims
        self.values_bcsr = np.zeros((len(sparsity.colidx), rdim, cdim))
        self.err = np.zeros(1, dtype=np.int32)

    def __call__(self, access, maps):
        if self.sparsity.shape != (1, 1):
            return ("mmat", self.blocks, access, (tuple(maps[0]), tuple(maps[1])))
        return ("mat", self, access, tuple(maps))

    def __getitem__(self, ij):
        i, j = ij
        return self.blocks[i][j]

    def zero(self):
        for row in self.blocks:
            for b in row:
                b.values_bcsr[...] = 0

    def assemble(self):
        for row in self.blocks:
            for b in row:
                if b.err[0]:
                    raise RuntimeError("oracle Mat: insertion outside the sparsity pattern")

    def to_scipy(self):
        import scipy.sparse as sps
        if self.sparsity.shape != (1, 1):
            return sps.bmat([[b.to_scipy() for b in row] for row in self.blocks], format="csr")
        rdim, cdim = self.sparsity.dims
        sp = self.sparsity
        shape = ((len(sp.rowptr) - 1) * rdim, sp.dsets[1].set.size * cdim)
        return sps.bsr_matrix((self.values_bcsr, sp.colidx, sp.rowptr), shape=shape,
                              blocksize=(rdim, cdim))

    @property
    def values(self):
        return self.to_scipy().toarray()


# --------------------------------------------------------- C wrapper codegen
_MATSET = r"""
static int op2o_find(const int64_t *rp, const int32_t *ci, int64_t r, int32_t c) {
  int64_t lo = rp[r], hi = rp[r + 1] - 1;
  while (lo <= hi) { int64_t m = (lo + hi) / 2; if (ci[m] == c) return (int)(m - rp[r]);
    if (ci[m] < c) lo = m + 1; else hi = m - 1; }
  return -1;
}
/* MatSetValuesBlockedLocal on block-CSR: vals is (nr*rd) x (nc*cd) row-major */
static void op2o_matset(double *v, const int64_t *rp, const int32_t *ci, int rd, int cd,
                        int nr, const int *rows, int nc, const int *cols, const double *vals,
                        int add, int32_t *err) {
  for (int i = 0; i < nr; ++i) { if (rows[i] < 0) continue;
    for (int j = 0; j < nc; ++j) { if (cols[j] < 0) continue;
      int q = op2o_find(rp, ci, rows[i], cols[j]);
      if (q < 0) { *err |= 2; continue; }
      double *b = v + (rp[rows[i]] + q) * rd * cd;
      for (int a = 0; a < rd; ++a) for (int c = 0; c < cd; ++c) {
        double x = vals[(i * rd + a) * (nc * cd) + j * cd + c];
        if (add) b[a * cd + c] += x; else b[a * cd + c] = x; } } }
}
"""


def _generate(kernel, sig):
    """C source of the sequential wrapper for signature `sig`."""
    extr, const, periodic, subset, region, pass_layer, args, maps = sig
    nf = 2 if (extr and region == ON_INTERIOR_FACETS) else 1
    o = ["#include <stdint.h>", "#include <math.h>", "#include <string.h>",
         "#define restrict __restrict", kernel.code, _MATSET]
    for mi, (kind, arity, base, comps, off, oq, perm) in enumerate(maps):
        for nm, v in (("off", off), ("oq", oq), ("perm", perm)):
            if v is not None:
                o.append("static const int op2o_%s%d[%d] = {%s};" % (nm, mi, len(v),
                                                                      ", ".join(map(str, v))))
    params = ["int start", "int end", "const int32_t *layers", "const int32_t *subset"]
    for ai, a in enumerate(args):
        kind = a[0]
        if kind == "mat":
            params += ["double *mv%d" % ai, "const int64_t *mrp%d" % ai, "const int32_t *mci%d" % ai,
                       "int32_t *merr%d" % ai]
        else:
            params.append("void *a%d" % ai)
    for mi in range(len(maps)):
        params.append("const int32_t *m%d" % mi)
    o.append("void op2o_wrap(%s) {" % ", ".join(params))
    # global temporaries for INC (zeroed per call, added at the end)
    for ai, a in enumerate(args):
        if a[0] == "glob" and a[2] == INC:
            ct = _CTYPE[a[3]]
            o.append("  %s gtmp%d[%d]; memset(gtmp%d, 0, sizeof gtmp%d);" % (ct, ai, a[4], ai, ai))
    o.append("  for (int n0 = start; n0 < end; ++n0) {")
    o.append("    const int n = subset ? subset[n0] : n0;")
    ind = "    "
    if extr:
        o.append("    const int32_t *L = layers + (%s);" % ("0" if const else "2 * n"))
        o.append("    const int cs = L[0], ce = L[1] - 1, nlay = ce - cs;")
        if region == ON_BOTTOM:
            o.append("    const int ls = cs, le = cs + 1, bottom = cs;")
        elif region == ON_TOP:
            o.append("    const int ls = ce - 1, le = ce, bottom = cs;")
        elif region == ON_INTERIOR_FACETS:
            o.append("    const int ls = cs, le = %s, bottom = cs;" % ("ce" if periodic else "ce - 1"))
        else:
            o.append("    const int ls = cs, le = ce, bottom = cs;")
        o.append("    (void)nlay;")
        o.append("    for (int layer = ls; layer < le; ++layer) {")
        ind = "      "

    def entity_row(mi, ent):
        return "m%d[(int64_t)(%s) * %d + i]" % (mi, ent, maps[mi][1])

    # index arrays per map and facet
    used = set()
    for a in args:
        if a[0] == "dat" and a[5] is not None:
            used.add(a[5])
        if a[0] == "mat":
            used.update(a[5])
    for mi in sorted(used):
        kind, arity, base, comps, off, oq, perm = maps[mi]
        # base row values and the map providing offsets
        if kind == "plain":
            src = mi
            rowexpr = "m%d[(int64_t)n * %d + i]" % (mi, arity)
            oidx = "i"
        elif kind == "perm":
            src = base
            rowexpr = "m%d[(int64_t)n * %d + op2o_perm%d[i]]" % (base, arity, mi)
            oidx = "op2o_perm%d[i]" % mi
        else:
            outer = comps[0]
            ok, _, obase, _, _, _, operm = maps[outer]
            o.append(ind + "int64_t ce%d = n;" % mi)
            for c in reversed(comps[1:]):
                ck, _, cb, _, _, _, _ = maps[c]
                croot = cb if ck == "perm" else c
                o.append(ind + "if (ce%d >= 0) ce%d = m%d[ce%d];" % (mi, mi, croot, mi))
            root = obase if ok == "perm" else outer
            pidx = ("op2o_perm%d[i]" % outer) if ok == "perm" else "i"
            rowexpr = "(ce%d >= 0 ? m%d[ce%d * %d + %s] : -1)" % (mi, root, mi, arity, pidx)
            src = root
            oidx = pidx
        soff = maps[src][4]
        soq = maps[src][5]
        for f in range(nf):
            o.append(ind + "int x%d_%d[%d];" % (mi, f, arity))
            o.append(ind + "for (int i = 0; i < %d; ++i) {" % arity)
            o.append(ind + "  int b = %s;" % rowexpr)
            if extr and soff is not None:
                e = "(layer - bottom + %d)" % f
                if periodic:
                    def R(a, b):
                        return "((%s) < (%s) ? (%s) : (%s) - (%s))" % (a, b, a, a, b)
                    if soq is not None:
                        q = "op2o_oq%d[%s]" % (src, oidx)
                        e = "(%s - %s)" % (R(e + " + " + q, "nlay"), R(q, "nlay"))
                    else:
                        e = R(e, "nlay")
                o.append(ind + "  if (b >= 0) b += op2o_off%d[%s] * %s;" % (src, oidx, e))
            o.append(ind + "  x%d_%d[i] = b;" % (mi, f))
            o.append(ind + "}")
    # Mixed arguments (pyop2/codegen/builder.py:413-498, 609-680): the
    # components of one group share one kernel parameter.  Dat components'
    # packs are concatenated; a mixed Mat's blocks are sub-blocks of one
    # element matrix, copied out block by block before insertion.
    first, off, gsize, mrc = {}, {}, {}, {}
    ai = 0
    while ai < len(args):
        g = args[ai][6]
        bj = ai + 1
        while g and bj < len(args) and args[bj][6] == g:
            bj += 1
        a0 = args[ai]
        if a0[0] == "dat":
            o_ = 0
            for k in range(ai, bj):
                first[k], off[k] = ai, o_
                if args[k][5] is not None:
                    o_ += nf * maps[args[k][5]][1] * args[k][4]
            gsize[ai] = o_
        elif a0[0] == "mat":
            ncols = a0[7] if g else 1
            nrows = (bj - ai) // ncols

            def rows_of(k):
                return nf * maps[args[k][5][0]][1] * args[k][3][0]

            def cols_of(k):
                return nf * maps[args[k][5][1]][1] * args[k][3][1]
            roffs = [sum(rows_of(ai + q * ncols) for q in range(i)) for i in range(nrows)]
            coffs = [sum(cols_of(ai + q) for q in range(j)) for j in range(ncols)]
            R = sum(rows_of(ai + q * ncols) for q in range(nrows))
            C = sum(cols_of(ai + q) for q in range(ncols))
            for k in range(ai, bj):
                i, j = divmod(k - ai, ncols)
                first[k] = ai
                mrc[k] = (roffs[i], coffs[j], rows_of(k), cols_of(k), C, g != 0)
            gsize[ai] = R * C
        else:
            first[ai] = ai
        ai = bj
    # packs
    kargs = []
    for ai, a in enumerate(args):
        kind = a[0]
        if kind == "glob":
            _, _, acc, dt, dim = a[:5]
            ct = _CTYPE[dt]
            if acc == READ:
                kargs.append("(%s *)a%d" % (ct, ai))
            else:
                o.append(ind + "%s g%d[%d];" % (ct, ai, dim))
                if acc == INC:
                    o.append(ind + "for (int j = 0; j < %d; ++j) g%d[j] = 0;" % (dim, ai))
                else:
                    o.append(ind + "for (int j = 0; j < %d; ++j) g%d[j] = ((%s *)a%d)[j];"
                             % (dim, ai, ct, ai))
                kargs.append("g%d" % ai)
        elif kind == "dat":
            _, _, acc, dt, dim, mi = a[:6]
            ct = _CTYPE[dt]
            if mi is None:
                kargs.append("((%s *)a%d) + (int64_t)n * %d" % (ct, ai, dim))
                continue
            ar = maps[mi][1]
            tp, po = first[ai], off[ai]
            if tp == ai:
                o.append(ind + "%s t%d[%d];" % (ct, ai, gsize[ai]))
            if acc in (INC, WRITE):
                if tp == ai:
                    o.append(ind + "for (int k = 0; k < %d; ++k) t%d[k] = 0;" % (gsize[ai], ai))
            else:
                for f in range(nf):
                    o.append(ind + "for (int i = 0; i < %d; ++i) for (int j = 0; j < %d; ++j) "
                             "t%d[%d + (%d + i) * %d + j] = x%d_%d[i] >= 0 ? ((%s *)a%d)[(int64_t)x%d_%d[i] * %d + j] : 0;"
                             % (ar, dim, tp, po, f * ar, dim, mi, f, ct, ai, mi, f, dim))
            if tp == ai:
                kargs.append("t%d" % ai)
        elif kind == "mat":
            if first[ai] == ai:
                tot = gsize[ai]
                o.append(ind + "double t%d[%d]; for (int k = 0; k < %d; ++k) t%d[k] = 0;"
                         % (ai, tot, tot, ai))
                kargs.append("t%d" % ai)
    if pass_layer:
        kargs.append("layer")
    o.append(ind + "%s(%s);" % (kernel.name, ", ".join(kargs)))
    # unpacks
    for ai, a in enumerate(args):
        kind = a[0]
        if kind == "glob":
            _, _, acc, dt, dim = a[:5]
            ct = _CTYPE[dt]
            if acc == INC:
                o.append(ind + "for (int j = 0; j < %d; ++j) gtmp%d[j] += g%d[j];" % (dim, ai, ai))
            elif acc in (MIN, MAX):
                cmp = "<" if acc == MIN else ">"
                o.append(ind + "for (int j = 0; j < %d; ++j) { %s *G = (%s *)a%d; "
                         "if (g%d[j] %s G[j]) G[j] = g%d[j]; }" % (dim, ct, ct, ai, ai, cmp, ai))
        elif kind == "dat":
            _, _, acc, dt, dim, mi = a[:6]
            if mi is None or acc == READ:
                continue
            ct = _CTYPE[dt]
            ar = maps[mi][1]
            for f in range(nf):
                dst = "((%s *)a%d)[(int64_t)x%d_%d[i] * %d + j]" % (ct, ai, mi, f, dim)
                src = "t%d[%d + (%d + i) * %d + j]" % (first[ai], off[ai], f * ar, dim)
                if acc == INC:
                    stmt = "%s += %s;" % (dst, src)
                elif acc == MIN:
                    stmt = "if (%s < %s) %s = %s;" % (src, dst, dst, src)
                elif acc == MAX:
                    stmt = "if (%s > %s) %s = %s;" % (src, dst, dst, src)
                else:
                    stmt = "%s = %s;" % (dst, src)
                o.append(ind + "for (int i = 0; i < %d; ++i) { if (x%d_%d[i] < 0) continue; "
                         "for (int j = 0; j < %d; ++j) { %s } }" % (ar, mi, f, dim, stmt))
        elif kind == "mat":
            _, _, acc, (rd, cd), _, (rm, cm) = a[:6]
            ra, ca = maps[rm][1], maps[cm][1]
            rows = "rr%d" % ai
            cols = "cc%d" % ai
            r0, c0, nr_, nc_, C, grouped = mrc[ai]
            vals = "t%d" % ai
            if grouped:
                # mixed element matrix -> this block's local matrix
                vals = "tb%d" % ai
                o.append(ind + "double %s[%d];" % (vals, nr_ * nc_))
                o.append(ind + "for (int i = 0; i < %d; ++i) for (int j = 0; j < %d; ++j) "
                         "%s[i * %d + j] = t%d[(%d + i) * %d + %d + j];"
                         % (nr_, nc_, vals, nc_, first[ai], r0, C, c0))
            o.append(ind + "int %s[%d], %s[%d];" % (rows, nf * ra, cols, nf * ca))
            for f in range(nf):
                o.append(ind + "for (int i = 0; i < %d; ++i) %s[%d + i] = x%d_%d[i];"
                         % (ra, rows, f * ra, rm, f))
                o.append(ind + "for (int i = 0; i < %d; ++i) %s[%d + i] = x%d_%d[i];"
                         % (ca, cols, f * ca, cm, f))
            o.append(ind + "op2o_matset(mv%d, mrp%d, mci%d, %d, %d, %d, %s, %d, %s, %s, %d, merr%d);"
                     % (ai, ai, ai, rd, cd, nf * ra, rows, nf * ca, cols, vals,
                        1 if acc == INC else 0, ai))
    if extr:
        o.append("    }")
    o.append("  }")
    for ai, a in enumerate(args):
        if a[0] == "glob" and a[2] == INC:
            ct = _CTYPE[a[3]]
            o.append("  for (int j = 0; j < %d; ++j) ((%s *)a%d)[j] += gtmp%d[j];" % (a[4], ct, ai, ai))
    o.append("}")
    return "\n".join(o) + "\n"


_SO_CACHE = {}
_LOCK = threading.Lock()


def _compile(src, profile):
    key = hashlib.sha256((src + repr(PROFILES[profile])).encode()).hexdigest()[:24]
    with _LOCK:
        if key in _SO_CACHE:
            return _SO_CACHE[key]
        d = os.path.join(_build.REF_DIR, "wrappers")
        os.makedirs(d, exist_ok=True)
        so = os.path.join(d, "w_%s_%s.so" % (profile, key))
        if not os.path.exists(so):
            c = os.path.join(d, "w_%s_%s.c" % (profile, key))
            with open(c, "w") as f:
                f.write(src)
            cmd = ["gcc", "-std=gnu11", "-fPIC", "-shared", *PROFILES[profile], c, "-o",
                   so + ".tmp", "-lm"]
            p = subprocess.run(cmd, capture_output=True, text=True)
            if p.returncode != 0 and "-march=native" in cmd:
                cmd.remove("-march=native")
                p = subprocess.run(cmd, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError("oracle: gcc failed\n%s\n%s" % (p.stderr, src))
            os.replace(so + ".tmp", so)
        lib = ctypes.CDLL(so)
        _SO_CACHE[key] = lib
        return lib


class _Table:
    def __init__(self):
        self.entries = []
        self.arrays = []
        self.idx = {}

    def add(self, m):
        if id(m) in self.idx:
            return self.idx[id(m)]
        if isinstance(m, ComposedMap):
            comps = tuple(self.add(c) for c in m.flat)
            e = ("comp", m.arity, -1, comps, None, None, None)
            arr = None
        elif isinstance(m, PermutedMap):
            b = self.add(m.map_)
            e = ("perm", m.arity, b, (), None, None, tuple(int(x) for x in m.permutation))
            arr = None
        else:
            e = ("plain", m.arity, -1, (),
                 None if m.offset is None else tuple(int(x) for x in m.offset),
                 None if m.offset_quotient is None else tuple(int(x) for x in m.offset_quotient),
                 None)
            arr = m.values
        self.idx[id(m)] = len(self.entries)
        self.entries.append(e)
        self.arrays.append(arr)
        return self.idx[id(m)]


class ParLoop:
    """A compiled sequential loop; ``compute(start, end)`` runs a range."""

    def __init__(self, kernel, iterset, *args, iteration_region=ALL, pass_layer_arg=False,
                 profile="parity"):
        table = _Table()
        sig_args = []
        group = 0
        for a in args:
            kind, obj, acc, m = a
            if kind == "glob":
                sig_args.append(("glob", obj, acc, obj.data.dtype.name, obj.dim, None, 0, 0))
            elif kind == "dat":
                mi = table.add(m) if m is not None else None
                sig_args.append(("dat", obj, acc, obj.data.dtype.name, obj.cdim, mi, 0, 0))
            elif kind == "mdat":
                # ("mdat", [Dat, ...], access, [Map, ...]): one mixed argument
                group += 1
                for d, mm in zip(obj, m):
                    sig_args.append(("dat", d, acc, d.data.dtype.name, d.cdim, table.add(mm),
                                     group, 0))
            elif kind == "mmat":
                # ("mmat", [[Mat, ...], ...], access, ([rmap, ...], [cmap, ...]))
                group += 1
                rms, cms = m
                for i, row in enumerate(obj):
                    for j, mat in enumerate(row):
                        sig_args.append(("mat", mat, acc, mat.sparsity.dims, None,
                                         (table.add(rms[i]), table.add(cms[j])), group, len(cms)))
            else:
                sig_args.append(("mat", obj, acc, obj.sparsity.dims, None,
                                 (table.add(m[0]), table.add(m[1])), 0, 0))
        self.iterset = iterset
        extr = bool(iterset._extruded)
        const = bool(extr and iterset.constant_layers)
        periodic = bool(extr and getattr(iterset, "periodic", False))
        sub = isinstance(iterset, Subset)
        sig_norm = (extr, const, periodic, sub, int(iteration_region), bool(pass_layer_arg),
                    [(s[0], None) + tuple(s[2:]) for s in sig_args], table.entries)
        self.src = _generate(kernel, sig_norm)
        self.fn = getattr(_compile(self.src, profile), "op2o_wrap")
        self.fn.restype = None
        self.args = sig_args
        self.table = table

    def argv(self, overrides=None):
        """ctypes argument values; overrides maps arg index -> ndarray."""
        it = self.iterset
        v = [None, None]
        v.append(it.layers_array.ctypes.data if it._extruded else None)
        v.append(it.indices.ctypes.data if isinstance(it, Subset) else None)
        for i, s in enumerate(self.args):
            obj = s[1]
            if s[0] == "mat":
                v += [obj.values_bcsr.ctypes.data, obj.sparsity.rowptr.ctypes.data,
                      obj.sparsity.colidx.ctypes.data, obj.err.ctypes.data]
            else:
                arr = overrides[i] if overrides and i in overrides else obj.data
                v.append(arr.ctypes.data)
        for arr in self.table.arrays:
            v.append(arr.ctypes.data if arr is not None else None)
        return v

    def compute(self, start=0, end=None, overrides=None):
        end = self.iterset.size if end is None else end
        v = self.argv(overrides)
        v[0], v[1] = ctypes.c_int(start), ctypes.c_int(end)
        self.fn(*[ctypes.c_void_p(x) if not isinstance(x, ctypes.c_int) else x for x in v])


def par_loop(kernel, iterset, *args, **kwargs):
    """Run a loop sequentially (the reference's execution order)."""
    ParLoop(kernel, iterset, *args, **kwargs).compute()
