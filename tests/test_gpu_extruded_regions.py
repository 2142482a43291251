"""Extruded iteration regions (ON_BOTTOM / ON_TOP / ON_INTERIOR_FACETS /
ALL), periodic extrusion with offset quotients, variable layers, and
composed maps over extruded sets: GPU against the oracle / the reference
test's expected values."""
import numpy as np
import pytest

import scenarios as S

pytestmark = pytest.mark.gpu

REGIONS = ["ON_BOTTOM", "ON_TOP", "ON_INTERIOR_FACETS", "ALL"]


@pytest.mark.parametrize("region", REGIONS)
@pytest.mark.parametrize("variable", [False, True])
def test_regions_vs_oracle(gpu_op2, oracle_op2, region, variable):
    g = S.sc_extruded_regions(gpu_op2, getattr(gpu_op2, region), variable=variable)
    o = S.sc_extruded_regions(oracle_op2, getattr(oracle_op2, region), variable=variable)
    assert np.array_equal(g, o)
    assert g.sum() > 0


@pytest.mark.parametrize("region", ["ON_INTERIOR_FACETS", "ALL"])
def test_periodic_vs_oracle(gpu_op2, oracle_op2, region):
    g = S.sc_extruded_regions(gpu_op2, getattr(gpu_op2, region), periodic=True)
    o = S.sc_extruded_regions(oracle_op2, getattr(oracle_op2, region), periodic=True)
    assert np.array_equal(g, o)


@pytest.mark.parametrize("variable", [False, True])
@pytest.mark.parametrize("subset", [False, True])
def test_composed_map_extrusion(gpu_op2, variable, subset):
    S.sc_composed_map_extrusion(gpu_op2, variable, subset)
