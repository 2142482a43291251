"""Exception types of the PyOP2 API (same names and bases as
pyop2/exceptions.py:37-158), so code that catches the reference's exceptions
keeps working."""


class DataTypeError(TypeError):
    """Invalid type for data."""


class DimTypeError(TypeError):
    """Invalid type for dimension."""


class ArityTypeError(TypeError):
    """Invalid type for arity."""


class IndexTypeError(TypeError):
    """Invalid type for index."""


class NameTypeError(TypeError):
    """Invalid type for name."""


class SetTypeError(TypeError):
    """Invalid type for :class:`pyop2_gb300.op2.Set`."""


class SizeTypeError(TypeError):
    """Invalid type for size."""


class SubsetIndexOutOfBounds(TypeError):
    """Out of bound index."""


class SparsityTypeError(TypeError):
    """Invalid type for :class:`pyop2_gb300.op2.Sparsity`."""


class MapTypeError(TypeError):
    """Invalid type for :class:`pyop2_gb300.op2.Map`."""


class DataSetTypeError(TypeError):
    """Invalid type for :class:`pyop2_gb300.op2.DataSet`."""


class MatTypeError(TypeError):
    """Invalid type for :class:`pyop2_gb300.op2.Mat`."""


class DatTypeError(TypeError):
    """Invalid type for :class:`pyop2_gb300.op2.Dat`."""


class KernelTypeError(TypeError):
    """Invalid type for :class:`pyop2_gb300.op2.Kernel`."""


class DataValueError(ValueError):
    """Illegal value for data."""


class IndexValueError(ValueError):
    """Illegal value for index."""


class ModeValueError(ValueError):
    """Illegal value for mode."""


class IterateValueError(ValueError):
    """Illegal value for iterate."""


class SetValueError(ValueError):
    """Illegal value for :class:`pyop2_gb300.op2.Set`."""


class MapValueError(ValueError):
    """Illegal value for :class:`pyop2_gb300.op2.Map`."""


class ConfigurationError(RuntimeError):
    """Illegal configuration value or type."""


class CompilationError(RuntimeError):
    """Error during JIT compilation (here: NVRTC)."""


class SparsityFormatError(ValueError):
    """Unable to produce a sparsity for this matrix format."""


class CachingError(ValueError):
    """A caching error."""


class HashError(CachingError):
    """Something is wrong with the hash."""
