"""The PyOP2 API (pyop2/op2.py:36-121), executed on a GB300.

    from pyop2_gb300 import op2
    op2.par_loop(op2.Kernel(code, "name"), cells, y(op2.INC, c2v), x(op2.READ, c2v))
"""
from pyop2_gb300.configuration import configuration
from pyop2_gb300.logger import debug, info, warning, error, critical, set_log_level  # noqa: F401
from pyop2_gb300.types import (  # noqa: F401
    Set, ExtrudedSet, MixedSet, Subset, DataSet, MixedDataSet, GlobalDataSet,
    Map, MixedMap, PermutedMap, ComposedMap, Sparsity,
    Global, Constant, Dat, DatView, MixedDat, Mat,
    READ, WRITE, RW, INC, MIN, MAX, ON_BOTTOM, ON_TOP, ON_INTERIOR_FACETS, ALL)
from pyop2_gb300.local_kernel import CStringLocalKernel, Kernel  # noqa: F401
from pyop2_gb300.datatypes import OpaqueType  # noqa: F401
from pyop2_gb300 import mpi as MPI  # noqa: F401
from pyop2_gb300.types.halo import Halo  # noqa: F401
from pyop2_gb300.parloop import (Parloop, ParLoop, LegacyParloop, parloop, par_loop,  # noqa: F401
                                 GlobalLegacyArg, DatLegacyArg, MatLegacyArg, PassthroughArg,
                                 MixedDatLegacyArg, MixedMatLegacyArg,
                                 GlobalParloopArg, DatParloopArg, MixedDatParloopArg,
                                 MatParloopArg, MixedMatParloopArg, PassthroughParloopArg)
from pyop2_gb300.global_kernel import (GlobalKernelArg, DatKernelArg,  # noqa: F401
                                       MixedDatKernelArg, MatKernelArg, MixedMatKernelArg,
                                       MapKernelArg, PermutedMapKernelArg,
                                       ComposedMapKernelArg, PassthroughKernelArg,
                                       GlobalKernel)

__all__ = ['configuration', 'READ', 'WRITE', 'RW', 'INC', 'MIN', 'MAX',
           'ON_BOTTOM', 'ON_TOP', 'ON_INTERIOR_FACETS', 'ALL',
           'debug', 'info', 'warning', 'error', 'critical', 'initialised',
           'set_log_level', 'init', 'exit', 'Kernel', 'Set', 'ExtrudedSet',
           'MixedSet', 'Subset', 'DataSet', 'GlobalDataSet', 'MixedDataSet',
           'Dat', 'MixedDat', 'Mat', 'Global', 'Constant', 'Map', 'MixedMap',
           'Sparsity', 'parloop', 'Parloop', 'ParLoop', 'par_loop',
           'PermutedMap', 'ComposedMap', 'MixedDat', 'DatView', 'PassthroughArg', 'OpaqueType',
           'MPI', 'Halo']

_initialised = False
set_log_level(configuration['log_level'])


def initialised():
    """True between init() and exit()."""
    return _initialised


def init(**kwargs):
    """Update the configuration (pyop2/op2.py:82-108); any configuration key
    is accepted as a keyword."""
    global _initialised
    configuration.reconfigure(**kwargs)
    set_log_level(configuration['log_level'])
    _initialised = True


def exit():
    """Reset the configuration."""
    global _initialised
    configuration.reset()
    _initialised = False
