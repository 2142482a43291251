"""Data model of the PyOP2 API (pyop2/types/)."""
from pyop2_gb300.types.access import (Access, READ, WRITE, RW, INC, MIN, MAX,  # noqa: F401
                                      IterationRegion, ON_BOTTOM, ON_TOP, ON_INTERIOR_FACETS, ALL)
from pyop2_gb300.types.set import Set, ExtrudedSet, Subset, MixedSet, GlobalSet, SetPartition  # noqa: F401
from pyop2_gb300.types.dataset import DataSet, GlobalDataSet, MixedDataSet  # noqa: F401
from pyop2_gb300.types.map import Map, PermutedMap, ComposedMap, MixedMap  # noqa: F401
from pyop2_gb300.types.dat import Dat, DatView, MixedDat, AbstractDat, DataCarrier  # noqa: F401
from pyop2_gb300.types.glob import Global, Constant  # noqa: F401
from pyop2_gb300.types.mat import Sparsity, Mat  # noqa: F401
