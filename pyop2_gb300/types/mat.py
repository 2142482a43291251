"""Sparsity and Mat (pyop2/types/mat.py:26-865) on the device.

A Sparsity is built from its Map pairs by GPU kernels (op2g_sparsity_count /
op2g_sparsity_fill) into block-CSR: int64 row pointers and sorted, unique
int32 block-column indices per block row -- the pattern PETSc's preallocator
holds in the reference (pyop2/sparsity.pyx:121-175).  A Mat stores
``rdim x cdim`` row-major blocks over that pattern (BAIJ when the reference
would use BAIJ, AIJ otherwise: the stored values are the same, only
``nnz`` is reported per dof row for AIJ, as pyop2/sparsity.pyx:168-173 does).
"""
import ctypes
import warnings
from collections.abc import Sequence

import numpy as np
import torch

from pyop2_gb300 import _lib, device
from pyop2_gb300 import exceptions as ex
from pyop2_gb300 import utils
from pyop2_gb300.configuration import configuration
from pyop2_gb300.datatypes import IntType, ScalarType
from pyop2_gb300.types.access import ALL, Access, IterationRegion
from pyop2_gb300.types.dat import DataCarrier
from pyop2_gb300.types.dataset import DataSet, GlobalDataSet, MixedDataSet
from pyop2_gb300.types.map import ComposedMap, Map, PermutedMap


def _is_mixed_map(m):
    from pyop2_gb300.types.map import MixedMap
    return isinstance(m, MixedMap)


def _flatten_map(m):
    """(base plain Map, permutation or None) of a Map/PermutedMap."""
    if isinstance(m, PermutedMap):
        return m.map_, m.permutation
    return m, None


class Sparsity:
    """Non-zero structure of a matrix from pairs of Maps.

    ``Sparsity((row_dset, col_dset), [(rmap, cmap, iteration_regions), ...],
    name=None, nest=None, block_sparse=None, diagonal_block=True)``.
    Cached per (dsets, maps, block_sparse) like the reference's ObjectCached.
    """

    def __new__(cls, dsets, maps_and_regions, name=None, nest=None, block_sparse=None,
                diagonal_block=True):
        dsets_p, mr, kw = cls._process_args(dsets, maps_and_regions, name, nest, block_sparse,
                                            diagonal_block)
        key = ("Sparsity", dsets_p, tuple(sorted(mr.items(), key=lambda kv: kv[0])),
               kw["block_sparse"], kw["diagonal_block"], kw["nest"])
        cache = dsets_p[0].set._cache if not isinstance(dsets_p[0], GlobalDataSet) else {}
        obj = cache.get(key)
        if obj is None:
            obj = super().__new__(cls)
            obj._initialized = False
            obj._args = (dsets_p, mr, kw)
            cache[key] = obj
        return obj

    def __init__(self, dsets, maps_and_regions, name=None, nest=None, block_sparse=None,
                 diagonal_block=True):
        if self._initialized:
            return
        dsets, mr, kw = self._args
        self._dsets = dsets
        self._maps_and_regions = mr
        self._block_sparse = kw["block_sparse"]
        self._diagonal_block = kw["diagonal_block"]
        self._name = kw["name"] or "sparsity_#x%x" % id(self)
        rset, cset = dsets
        self._has_diagonal = (rset == cset) and self._diagonal_block
        self.comm = rset.comm
        self._nest = bool(kw["nest"])
        if isinstance(rset, MixedDataSet) or isinstance(cset, MixedDataSet):
            self._init_mixed()
            self._initialized = True
            return
        self._dims = (((rset.cdim, cset.cdim),),)
        self._nested = False
        self._blocks = [[self]]
        from pyop2_gb300.profiling import timed_region
        with timed_region("CreateSparsity"):      # pyop2/types/mat.py:105-113
            self._build()
        self._initialized = True

    def _init_mixed(self):
        """Blocks of a sparsity between MixedDataSets (pyop2/types/mat.py:86-95,
        pyop2/sparsity.pyx:144-159).  Every block (i, j) is built on the GPU
        from its own map pairs; block (i, i) carries the diagonal.  Nested:
        ``nnz`` is the tuple of the blocks' ``nnz``.  Monolithic: ``nnz``
        counts the dof columns of each row of the assembled whole, i.e. the
        blocks of a block row laid side by side."""
        rset, cset = self._dsets
        rsets = tuple(rset) if isinstance(rset, MixedDataSet) else (rset,)
        csets = tuple(cset) if isinstance(cset, MixedDataSet) else (cset,)
        self._dims = tuple(tuple((r.cdim, c.cdim) for c in csets) for r in rsets)
        self._nested = self._nest
        self._blocks = []
        for i, rds in enumerate(rsets):
            row = []
            for j, cds in enumerate(csets):
                pairs = tuple(self._maps_and_regions.get((i, j), ()))
                if self._nested:
                    diag = rset is cset and i == j
                else:
                    diag = i == j and self._has_diagonal
                row.append(Sparsity((rds, cds), pairs, block_sparse=self._block_sparse,
                                    diagonal_block=diag, nest=False))
            self._blocks.append(row)
        if self._nested:
            self._d_nnz = tuple(b.nnz for row in self._blocks for b in row)
            self._o_nnz = tuple(b.onnz for row in self._blocks for b in row)
        else:
            rows = []
            for i, row in enumerate(self._blocks):
                rdim = rsets[i].cdim
                acc = np.zeros(rsets[i].size, dtype=np.int64)
                for j, b in enumerate(row):
                    acc += np.diff(b.rowptr.cpu().numpy()) * csets[j].cdim
                rows.append(np.repeat(acc, rdim))
            self._d_nnz = np.concatenate(rows).astype(IntType)
            self._o_nnz = np.zeros_like(self._d_nnz)

    @classmethod
    def _process_args(cls, dsets, maps_and_regions, name, nest, block_sparse, diagonal_block):
        """Normalise the map pairs (pyop2/types/mat.py:118-176)."""
        if name is not None and not isinstance(name, str):
            raise ex.NameTypeError("Sparsity name must be a string, not %r" % type(name))
        if len(dsets) != 2:
            raise RuntimeError("dsets must be a tuple of two DataSets: got %s" % (dsets,))
        for d in dsets:
            if not isinstance(d, DataSet) and d is not None:
                raise ex.DataSetTypeError("All data sets must be of type DataSet, not type %r" % type(d))
        if isinstance(maps_and_regions, Sequence):
            maps_and_regions = {(0, 0): maps_and_regions}
        elif not isinstance(maps_and_regions, dict):
            raise TypeError("maps_and_regions must be dict or Sequence: got %s" % type(maps_and_regions))
        nr, nc = len(dsets[0]), len(dsets[1])
        out = {}
        for key, val in maps_and_regions.items():
            i, j = key
            if i >= nr or j >= nc:
                raise RuntimeError("(i, j) must be < %s: got %s" % ((nr, nc), (i, j)))
            rds, cds = dsets[0][i], dsets[1][j]
            processed = set()
            for item in set(val):
                rmap, cmap, regions = item
                for m in (rmap, cmap):
                    if not isinstance(m, Map):
                        raise ex.MapTypeError("All maps must be of type map, not type %r" % type(m))
                    if not isinstance(m, ComposedMap) and len(m.values_with_halo) == 0 \
                            and m.iterset.total_size > 0:
                        raise ex.MapValueError("Unpopulated map values when trying to build sparsity.")
                if rmap.toset is not rds.set or cmap.toset is not cds.set:
                    raise RuntimeError("Map toset must be the same as DataSet set")
                if rmap.iterset is not cmap.iterset:
                    raise RuntimeError("Iterset of both maps in a pair must be the same")
                regions = (ALL,) if regions is None else tuple(sorted(regions))
                processed.add((rmap, cmap, regions))
            if processed:
                out[key] = frozenset(processed)
        if nest is None:
            nest = configuration["matnest"]
        if not (isinstance(dsets[0], MixedDataSet) or isinstance(dsets[1], MixedDataSet)):
            nest = False      # only meaningful between mixed spaces
        if block_sparse is None:
            block_sparse = configuration["block_sparsity"]
        return tuple(dsets), out, {"name": name, "nest": nest, "block_sparse": block_sparse,
                                   "diagonal_block": diagonal_block}

    # ---- GPU build
    def _pairs(self):
        """Deterministic list of (rmap, cmap, region) triples."""
        items = sorted(self._maps_and_regions.get((0, 0), ()),
                       key=lambda t: (id(t[0]), id(t[1]), t[2]))
        return [(r, c, reg) for r, c, regs in items for reg in regs]

    def _build(self):
        device.require()
        rset, cset = self._dsets
        nrows, ncols = rset.size, cset.size
        triples = self._pairs()
        keep = []  # keep host arrays alive for the duration of the calls
        pairs = (_lib.SparsityPair * max(1, len(triples)))()
        extruded = False
        constant_layers = True
        periodic = False
        layers_dev = None
        slots = 1
        for k, (rmap, cmap, region) in enumerate(triples):
            P = pairs[k]
            it = rmap.iterset
            if it._extruded:
                extruded = True
                constant_layers = it.constant_layers
                periodic = it._extruded_periodic
                layers_dev = it._layers_device()
                slots = max(slots, it.layer_slots())
            for side, m in (("r", rmap), ("c", cmap)):
                flat = m.flattened_maps if isinstance(m, ComposedMap) else (m,)
                outer, perm = _flatten_map(flat[0])
                vals = outer._device_values()
                if perm is not None:
                    # permute the columns of the outer map's values once
                    pv = np.ascontiguousarray(outer.values_with_halo[:, perm])
                    t = torch.from_numpy(pv).to(device.device())
                    keep.append(t)
                    vptr = t.data_ptr()
                else:
                    vptr = vals.data_ptr()
                setattr(P, side + "map", vptr)
                setattr(P, side + "arity", m.arity)
                chain = []
                for inner in flat[1:]:
                    b, _ = _flatten_map(inner)
                    chain.append(b._device_values().data_ptr())
                arr = getattr(P, side + "composed")
                for i, pch in enumerate(chain):
                    arr[i] = pch
                setattr(P, "n" + side + "composed", len(chain))
                if it._extruded:
                    off = m.offset if m.offset is not None else np.zeros(m.arity, IntType)
                    off = np.ascontiguousarray(off, dtype=IntType)
                    if perm is not None:
                        off = np.ascontiguousarray(off[perm])
                    keep.append(off)
                    setattr(P, side + "offset", off.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
                    if m.offset_quotient is not None:
                        q = np.ascontiguousarray(m.offset_quotient, dtype=IntType)
                        if perm is not None:
                            q = np.ascontiguousarray(q[perm])
                        keep.append(q)
                        setattr(P, side + "offset_quotient",
                                q.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
            P.nent = it.size
            P.region = int(region)
        D = _lib.SparsityDesc()
        D.nrows = nrows
        D.ncols = ncols
        D.set_diag = 1 if self._has_diagonal else 0
        D.extruded = 1 if extruded else 0
        D.constant_layers = 1 if constant_layers else 0
        D.extruded_periodic = 1 if periodic else 0
        D.layers = layers_dev.data_ptr() if layers_dev is not None else None
        D.layer_slots = slots
        D.npairs = len(triples)
        D.pairs = pairs
        ws = ctypes.c_size_t()
        _lib.call("op2g_sparsity_workspace", ctypes.byref(D), ctypes.byref(ws))
        work = device.empty_bytes(ws.value)
        rowptr = torch.empty(nrows + 1, dtype=torch.int64, device=device.device())
        nnz = ctypes.c_int64()
        st = device.stream_handle()
        _lib.call("op2g_sparsity_count", ctypes.byref(D), work.data_ptr(), ws.value,
                  rowptr.data_ptr(), ctypes.byref(nnz), st)
        colidx = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=device.device())
        _lib.call("op2g_sparsity_fill", ctypes.byref(D), work.data_ptr(), ws.value,
                  rowptr.data_ptr(), colidx.data_ptr(), st)
        del work, keep
        self._rowptr = rowptr
        self._colidx = colidx
        self._nnz_blocks = int(nnz.value)
        # row counts are read back from the device when first asked for
        self._d_nnz = self._o_nnz = None

    def _row_counts(self):
        """(nnz, onnz) per row: dof rows with dof columns unless the matrix
        is BAIJ (block_sparse and rdim == cdim), where they count blocks
        (pyop2/sparsity.pyx:168-173); onnz is zero on one process."""
        if self._d_nnz is None:
            rset, cset = self._dsets
            counts = torch.diff(self._rowptr).to(torch.int32).cpu().numpy().astype(IntType)
            rdim, cdim = rset.cdim, cset.cdim
            if not (self._block_sparse and rdim == cdim):
                counts = np.repeat(counts * cdim, rdim).astype(IntType)
            self._d_nnz = counts
            self._o_nnz = np.zeros_like(counts)
        return self._d_nnz, self._o_nnz

    # ---- properties
    @property
    def dsets(self):
        return self._dsets

    @property
    def maps(self):
        return [(r, c) for r, c, _ in self._maps_and_regions.get((0, 0), ())]

    @property
    def rcmaps(self):
        return {k: [(r, c) for r, c, _ in v] for k, v in self._maps_and_regions.items()}

    @property
    def iteration_regions(self):
        return {k: [regs for _, _, regs in v] for k, v in self._maps_and_regions.items()}

    @property
    def dims(self):
        return self._dims

    @property
    def shape(self):
        """Number of block rows and columns."""
        return (len(self._dsets[0]), len(self._dsets[1]))

    @property
    def nested(self):
        return self._nested

    @property
    def name(self):
        return self._name

    @property
    def nnz(self):
        return self._row_counts()[0]

    @property
    def onnz(self):
        return self._row_counts()[1]

    @property
    def nz(self):
        return int(self.nnz.sum())

    @property
    def onz(self):
        return int(self.onnz.sum())

    @property
    def rowptr(self):
        """Device int64 block-row pointers ``[nrows + 1]``."""
        return self._rowptr

    @property
    def colidx(self):
        """Device int32 block-column indices ``[nnz_blocks]``."""
        return self._colidx[:self._nnz_blocks]

    @property
    def nblocks(self):
        return self._nnz_blocks

    def csr(self):
        """Host (rowptr, colidx) of the block pattern."""
        return self._rowptr.cpu().numpy(), self.colidx.cpu().numpy()

    def __getitem__(self, idx):
        """Block (i, j), or block row i."""
        try:
            i, j = idx
            return self._blocks[i][j]
        except TypeError:
            return self._blocks[idx]

    def __iter__(self):
        """Blocks by row, then by column."""
        for row in self._blocks:
            yield from row

    def __contains__(self, other):
        """True if the (row map, column map) pair -- of MixedMaps for a mixed
        sparsity -- is one this sparsity was built from (block by block)."""
        rmaps = tuple(other[0]) if len(self._dsets[0]) > 1 or _is_mixed_map(other[0]) else (other[0],)
        cmaps = tuple(other[1]) if len(self._dsets[1]) > 1 or _is_mixed_map(other[1]) else (other[1],)
        for i, rm in enumerate(rmaps):
            for j, cm in enumerate(cmaps):
                if not any((rm, cm) == (pr, pc) for pr, pc in self.rcmaps.get((i, j), [])):
                    return False
        return True

    def __str__(self):
        return ("OP2 Sparsity: dsets %s, maps_and_regions %s, name %s, nested %s, "
                "block_sparse %s, diagonal_block %s") % (
            self._dsets, self._maps_and_regions, self._name, self._nested, self._block_sparse,
            self._diagonal_block)

    def __repr__(self):
        return "Sparsity(%r, %r, name=%r, nested=%r, block_sparse=%r, diagonal_block=%r)" % (
            self._dsets, self._maps_and_regions, self._name, self._nested, self._block_sparse,
            self._diagonal_block)


class Mat(DataCarrier):
    """OP2 matrix on a Sparsity: FP64 block-CSR values in HBM.

    par_loops add (INC) or insert (WRITE) element blocks; ``assemble()``
    finalises and reports insertions outside the pattern.
    """

    ASSEMBLED = "ASSEMBLED"
    INSERT_VALUES = "INSERT_VALUES"
    ADD_VALUES = "ADD_VALUES"
    _modes = [Access.WRITE, Access.INC]

    @utils.validate_type(('sparsity', Sparsity, ex.SparsityTypeError),
                         ('name', str, ex.NameTypeError))
    def __init__(self, sparsity, dtype=None, name=None, mat_type=None):
        self._sparsity = sparsity
        self._datatype = np.dtype(dtype or ScalarType)
        if self._datatype != ScalarType:
            raise RuntimeError("Can only create a matrix of type %s, %s is not supported"
                               % (ScalarType, self._datatype))
        self._name = name or "mat_#x%x" % id(self)
        self.mat_type = mat_type
        self.comm = sparsity.comm
        if sparsity.shape != (1, 1):
            # A mixed Mat: one device matrix per block (MatNest-like for both
            # nested and monolithic sparsities; pyop2/types/mat.py:572-666).
            self._parent = None
            self._state = Mat.ASSEMBLED
            self._blocks = [[Mat(sparsity[i, j], self._datatype,
                                 "_".join([self._name, str(i), str(j)]))
                             for j in range(sparsity.shape[1])]
                            for i in range(sparsity.shape[0])]
            if not sparsity.nested:
                # blocks of a monolithic matrix share its assembly state
                # (the reference's MatBlock, pyop2/types/mat.py:868-960)
                for b in self:
                    b._parent = self
            self._values = None
            self._err = None
            self._version = 0
            return
        self._parent = None
        self._state = Mat.ASSEMBLED
        self._blocks = [[self]]
        rdim, cdim = sparsity.dims[0][0]
        self._values = torch.zeros(max(sparsity.nblocks * rdim * cdim, 1), dtype=torch.float64,
                                   device=device.device())
        self._err = torch.zeros(1, dtype=torch.int32, device=device.device())
        self._version = 0

    @utils.validate_in(('access', _modes, ex.ModeValueError))
    def __call__(self, access, path, lgmaps=None, unroll_map=False):
        from pyop2_gb300.parloop import MatLegacyArg, MixedMatLegacyArg
        if self._mixed:
            rm, cm = path
            if not (_is_mixed_map(rm) and _is_mixed_map(cm)):
                raise ex.MapTypeError("A mixed Mat is accessed through a pair of MixedMaps")
            if (len(rm), len(cm)) != self._sparsity.shape:
                raise ex.MapValueError("MixedMaps do not match the Mat's block shape")
            if configuration["type_check"] and (rm, cm) not in self.sparsity:
                raise ex.MapValueError("Path maps not in sparsity maps")
            if unroll_map:
                raise NotImplementedError("unrolled (MatSetValuesLocal) insertion is not supported")
            return MixedMatLegacyArg(self, (rm, cm), access, lgmaps, unroll_map)
        path_maps = utils.as_tuple(path, Map, 2)
        if configuration["type_check"] and tuple(path_maps) not in self.sparsity:
            raise ex.MapValueError("Path maps not in sparsity maps")
        if unroll_map:
            raise NotImplementedError("unrolled (MatSetValuesLocal) insertion is not supported")
        return MatLegacyArg(self, tuple(path_maps), access, lgmaps, unroll_map)

    # ---- properties
    @property
    def sparsity(self):
        return self._sparsity

    @property
    def dims(self):
        return self._sparsity.dims

    @property
    def dtype(self):
        return self._datatype

    @property
    def name(self):
        return self._name

    @property
    def _mixed(self):
        return self._sparsity.shape != (1, 1)

    @property
    def nrows(self):
        return sum(d.size * d.cdim for d in self._sparsity.dsets[0])

    @property
    def ncols(self):
        return sum(d.size * d.cdim for d in self._sparsity.dsets[1])

    @property
    def nblock_rows(self):
        return self._sparsity.dsets[0].size

    @property
    def nblock_cols(self):
        return self._sparsity.dsets[1].size

    @property
    def nbytes(self):
        if self._mixed:
            return sum(b.nbytes for b in self)
        rdim, cdim = self.dims[0][0]
        return self._sparsity.nblocks * rdim * cdim * self.dtype.itemsize

    @property
    def tensor(self):
        """Device FP64 values, ``[nnz_blocks * rdim * cdim]`` (row-major blocks)."""
        return self._values[:self._sparsity.nblocks * self.dims[0][0][0] * self.dims[0][0][1]]

    def _bcsr(self):
        sp = self._sparsity
        rdim, cdim = self.dims[0][0]
        b = _lib.BCSR()
        b.nrows = sp.dsets[0].size
        b.ncols = sp.dsets[1].size
        b.rdim = rdim
        b.cdim = cdim
        b.rowptr = sp.rowptr.data_ptr()
        b.colidx = sp._colidx.data_ptr()
        b.values = self._values.data_ptr()
        return b

    def __iter__(self):
        """Blocks by row, then by column (the Mat itself when not mixed)."""
        for row in self._blocks:
            yield from row

    def __getitem__(self, idx):
        """Block (i, j), or block row i."""
        try:
            i, j = idx
            return self._blocks[i][j]
        except TypeError:
            return self._blocks[idx]

    @property
    def blocks(self):
        return self._blocks

    # ---- assembly state machine (pyop2/types/mat.py:488-501, 820-835)
    @property
    def assembly_state(self):
        return self._parent.assembly_state if self._parent is not None else self._state

    @assembly_state.setter
    def assembly_state(self, value):
        if self._parent is not None:
            self._parent.assembly_state = value
        else:
            self._state = value

    def change_assembly_state(self, new_state):
        if new_state == Mat.ASSEMBLED or self.assembly_state == Mat.ASSEMBLED:
            self.assembly_state = new_state
        elif new_state != self.assembly_state:
            self._flush_assembly()
            self.assembly_state = new_state

    def _flush_assembly(self):
        if self._parent is not None:
            self._parent._flush_assembly()
        else:
            self._check_err()

    def _check_err(self):
        if self._mixed:
            for b in self:
                b._check_err()
            return
        err = int(self._err.item())
        if err:
            self._err.zero_()
            if err & _lib.DEVERR_NEW_NONZERO:
                raise RuntimeError("Mat %s: insertion outside the sparsity pattern "
                                   "(new nonzero location)" % self._name)
            if err & _lib.DEVERR_MAP_BOUNDS:
                raise ex.MapValueError("Mat %s: map value out of range" % self._name)

    def assemble(self):
        if self._parent is not None:
            raise RuntimeError("Should never call assemble on MatBlock")
        if self._mixed and self._sparsity.nested:
            for b in self:
                b.assemble()
        elif self.assembly_state != Mat.ASSEMBLED:
            # only a write since the last assembly can have set the error
            # word, so an assembled matrix is not synchronised with again
            self._check_err()
        self.change_assembly_state(Mat.ASSEMBLED)

    def _assemble_owner(self):
        """Assemble this matrix, or its monolithic parent."""
        (self._parent or self).assemble()

    def zero(self):
        self._assemble_owner()
        if self._mixed:
            for b in self:
                b._values.zero_()
                b.increment_dat_version()
        else:
            self._values.zero_()
        self.increment_dat_version()

    def _not_mixed(self, what):
        if self._mixed:
            raise NotImplementedError("%s on a mixed Mat: call it on a block, mat[i, j]" % what)

    def zero_rows(self, rows, diag_val=1.0):
        """Zero the given (dof) rows keeping the pattern; put diag_val on the
        diagonal (PETSc zeroRowsLocal)."""
        from pyop2_gb300.types.set import Subset
        self._not_mixed("zero_rows")
        self.assemble()
        rows = rows.indices if isinstance(rows, Subset) else rows
        r = torch.as_tensor(np.asarray(rows, dtype=IntType).reshape(-1), device=device.device())
        b = self._bcsr()
        _lib.call("op2g_mat_zero_rows", ctypes.byref(b), r.data_ptr(), r.numel(),
                  float(diag_val), device.stream_handle())
        self.increment_dat_version()

    def set_local_diagonal_entries(self, rows, diag_val=1.0, idx=None):
        """INSERT diag_val at the diagonal of the given rows
        (pyop2/types/mat.py:806-827 semantics for block rows)."""
        self._not_mixed("set_local_diagonal_entries")
        rows = np.asarray(rows, dtype=IntType)
        rbs, _ = self.dims[0][0]
        if rbs > 1:
            if idx is not None:
                rows = rbs * rows + idx
            else:
                rows = np.dstack([rbs * rows + i for i in range(rbs)]).flatten()
        rows = rows.reshape(-1)
        self.change_assembly_state(Mat.INSERT_VALUES)
        if len(rows) > 0:
            r = torch.as_tensor(rows.astype(IntType), device=device.device())
            b = self._bcsr()
            _lib.call("op2g_mat_set_diagonal", ctypes.byref(b), r.data_ptr(), r.numel(),
                      float(diag_val), self._err.data_ptr(), device.stream_handle())
        self.increment_dat_version()

    def _insert(self, rows, cols, values, add):
        """MatSetValuesBlockedLocal semantics from the host: rows/cols are
        block indices, values a (len(rows) * rdim) x (len(cols) * cdim) array."""
        self._not_mixed("addto_values/set_values")
        rows = np.atleast_1d(np.asarray(rows, dtype=np.int64))
        cols = np.atleast_1d(np.asarray(cols, dtype=np.int64))
        rdim, cdim = self.dims[0][0]
        vals = np.asarray(values, dtype=np.float64).reshape(len(rows) * rdim, len(cols) * cdim)
        rp, ci = self._sparsity.csr()
        pos = []
        src = []
        for a, r in enumerate(rows):
            if r < 0:
                continue
            seg = ci[rp[r]:rp[r + 1]]
            for b, c in enumerate(cols):
                if c < 0:
                    continue
                k = np.searchsorted(seg, c)
                if k >= len(seg) or seg[k] != c:
                    raise RuntimeError("Mat %s: insertion outside the sparsity pattern "
                                       "(new nonzero location)" % self._name)
                base = (rp[r] + k) * rdim * cdim
                for i in range(rdim):
                    for j in range(cdim):
                        pos.append(base + i * cdim + j)
                        src.append(vals[a * rdim + i, b * cdim + j])
        if not pos:
            return
        idx = torch.as_tensor(np.asarray(pos, dtype=np.int64), device=self._values.device)
        v = torch.as_tensor(np.asarray(src), device=self._values.device)
        if add:
            self._values.index_add_(0, idx, v)
        else:
            self._values.index_copy_(0, idx, v)

    def addto_values(self, rows, cols, values):
        """Add a block of values (pyop2/types/mat.py:837-842)."""
        self.change_assembly_state(Mat.ADD_VALUES)
        if len(np.atleast_1d(values)) > 0:
            self._insert(rows, cols, values, True)

    def set_values(self, rows, cols, values):
        """Set a block of values (pyop2/types/mat.py:844-849)."""
        self.change_assembly_state(Mat.INSERT_VALUES)
        if len(np.atleast_1d(values)) > 0:
            self._insert(rows, cols, values, False)

    # ---- exports
    def csr(self):
        """(rowptr, block colidx, values[nblocks, rdim, cdim]) on the host."""
        self._not_mixed("csr")
        rp, ci = self._sparsity.csr()
        rdim, cdim = self.dims[0][0]
        v = self.tensor.cpu().numpy().reshape(-1, rdim, cdim)
        return rp, ci, v

    def to_torch(self):
        """The matrix as a torch sparse tensor on the device, for solvers:
        CSR for 1x1 blocks, BSR (``blocksize = (rdim, cdim)``) otherwise.
        Values and column indices are views of the Mat's own device arrays
        (no copy: later assemblies show through); the row pointers are
        converted to the column indices' int32.  A mixed Mat is exported as
        its monolithic whole, assembled from its blocks (a copy)."""
        self._assemble_owner()
        if self._mixed:
            s = self.to_scipy().tocsr()
            dev = device.device()
            with warnings.catch_warnings():
                # torch flags its sparse compressed layouts as beta
                warnings.simplefilter("ignore", UserWarning)
                return torch.sparse_csr_tensor(
                    torch.as_tensor(s.indptr.astype(np.int64), device=dev),
                    torch.as_tensor(s.indices.astype(np.int64), device=dev),
                    torch.as_tensor(s.data, device=dev), size=s.shape)
        sp = self._sparsity
        rdim, cdim = self.dims[0][0]
        if sp.nblocks >= 2 ** 31:
            raise ValueError("to_torch: more than 2^31 - 1 blocks")
        crow = sp.rowptr.to(torch.int32)
        col = sp.colidx
        shape = (self.nrows, self.ncols)
        with warnings.catch_warnings():
            # torch flags its sparse compressed layouts as beta
            warnings.simplefilter("ignore", UserWarning)
            if rdim == 1 and cdim == 1:
                return torch.sparse_csr_tensor(crow, col, self.tensor, size=shape)
            return torch.sparse_bsr_tensor(crow, col, self.tensor.view(-1, rdim, cdim),
                                           size=shape)

    def to_scipy(self):
        """scipy.sparse BSR (or CSR for 1x1 blocks) copy of the matrix."""
        import scipy.sparse as sps
        if self._mixed:
            # the monolithic view: blocks laid out by the dof offsets of the
            # mixed spaces
            return sps.bmat([[b.to_scipy() for b in row] for row in self._blocks],
                            format="csr")
        rp, ci, v = self.csr()
        rdim, cdim = self.dims[0][0]
        shape = (self.nrows, self.ncols)
        if rdim == 1 and cdim == 1:
            return sps.csr_matrix((v.reshape(-1), ci, rp), shape=shape)
        return sps.bsr_matrix((v, ci, rp), shape=shape, blocksize=(rdim, cdim))

    @property
    def values(self):
        """Dense copy of the matrix (refused above 1e6 entries, as the reference does)."""
        self._assemble_owner()
        if self.nrows * self.ncols > 1000000:
            raise ValueError("Printing dense matrix with more than 1 million entries not allowed.\n"
                             "Are you sure you wanted to do this?")
        return self.to_scipy().toarray()

    def mult(self, x, y, transpose=False):
        """y = A x (or A^T x) for float64 Dats x, y (MixedDats for a mixed
        Mat: y_i = sum_j A_ij x_j)."""
        if self._mixed:
            self.assemble()
            nr, nc = self._sparsity.shape
            outer, inner = (nc, nr) if transpose else (nr, nc)
            for i in range(outer):
                acc = None
                for j in range(inner):
                    b = self._blocks[j][i] if transpose else self._blocks[i][j]
                    if b.sparsity.nblocks == 0:
                        continue
                    t = y[i].__class__(y[i].dataset, None, y[i].dtype)
                    b.mult(x[j], t, transpose=transpose)
                    acc = t.tensor.clone() if acc is None else acc.add_(t.tensor)
                if acc is None:
                    y[i].tensor.zero_()
                else:
                    y[i].tensor.copy_(acc)
                y[i].mark_device_modified()
            return
        self._assemble_owner()
        b = self._bcsr()
        if transpose:
            y.tensor.zero_()
        _lib.call("op2g_mat_spmv", ctypes.byref(b), x._device_ptr(), y._device_ptr(),
                  1 if transpose else 0, device.stream_handle())
        y.mark_device_modified()

    def __str__(self):
        return "OP2 Mat: %s, sparsity (%s), datatype %s" % (self._name, self._sparsity,
                                                          self._datatype.name)

    def __repr__(self):
        return "Mat(%r, %r, %r)" % (self._sparsity, self._datatype, self._name)
