"""Element types (pyop2/datatypes.py).  IntType is PETSc's default int32 and
ScalarType float64, fixed here because there is no PETSc."""
import numpy

from pyop2_gb300 import _lib

IntType = numpy.dtype(numpy.int32)
RealType = numpy.dtype(numpy.float64)
ScalarType = numpy.dtype(numpy.float64)

_CODES = {
    "float64": _lib.F64, "float32": _lib.F32, "int32": _lib.I32, "uint32": _lib.U32,
    "int64": _lib.I64, "uint64": _lib.U64, "int16": _lib.I16, "uint16": _lib.U16,
    "int8": _lib.I8, "uint8": _lib.U8,
}


_CODE_OF = {}     # dtype (or type) -> code, filled on first use


def as_code(dtype):
    """libop2g element-type code of a numpy dtype (an OpaqueType travels as
    bytes: the kernel gets an untyped pointer)."""
    if isinstance(dtype, OpaqueType):
        return _CODES["uint8"]
    try:
        return _CODE_OF[dtype]
    except (KeyError, TypeError):
        pass
    name = numpy.dtype(dtype).name
    try:
        code = _CODES[name]
    except KeyError:
        raise TypeError("pyop2_gb300 has no device element type for %s" % name)
    try:
        _CODE_OF[dtype] = code
    except TypeError:
        pass
    return code


def as_cstr(dtype):
    """C type name of a numpy dtype (pyop2/datatypes.py:13-29)."""
    return {"bool": "unsigned char", "int8": "int8_t", "int16": "int16_t",
            "int32": "int32_t", "int64": "int64_t", "uint8": "uint8_t",
            "uint16": "uint16_t", "uint32": "uint32_t", "uint64": "uint64_t",
            "float32": "float", "float64": "double"}[numpy.dtype(dtype).name]


def dtype_limits(dtype):
    """(min, max) of a numpy dtype."""
    try:
        info = numpy.iinfo(dtype)
    except ValueError:
        info = numpy.finfo(dtype)
    return info.min, info.max


class OpaqueType:
    """A C type the kernel knows by name (loopy's OpaqueType in the
    reference, used with PassthroughArg for handles such as a PETSc Mat).
    The wrapper hands the kernel the raw pointer; it converts to whatever
    type the kernel's parameter declares."""

    def __init__(self, name):
        self.name = name

    def __repr__(self):
        return "OpaqueType(%r)" % self.name
