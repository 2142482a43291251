"""Randomised differential tests of par_loop: random sets, maps and argument
lists (every access mode, direct and indirect, Globals, dims 1-3, float64 and
int32, core/owned/total splits, Subsets, and extruded column meshes under
every iteration region) with a generated kernel whose results are integers.
The oracle must equal the access-semantics model bit for bit (CPU), and the
GPU must equal the oracle bit for bit under every INC strategy."""
import numpy as np
import pytest

import fuzz_loops as F

CPU_SEEDS = range(48)
GPU_SEEDS = range(48)
STRATEGIES = ["atomic", "warp", "colour", "shared"]


def _equal(got, want):
    assert len(got) == len(want)
    for k, (g, w) in enumerate(zip(got, want)):
        assert g.dtype == w.dtype and g.shape == w.shape, k
        assert np.array_equal(g, w), (k, g, w)


@pytest.mark.parametrize("seed", CPU_SEEDS)
def test_oracle_matches_model(oracle_op2, seed):
    spec = F.make_spec(seed)
    _equal(F.run(oracle_op2, spec), F.model(spec))


def test_specs_cover_every_access_and_shape():
    """The seeds above draw every access mode of every argument kind, both
    dtypes, Subsets, empty iteration sets and the bijective map."""
    seen = set()
    subset = empty = bij = False
    for seed in CPU_SEEDS:
        s = F.make_spec(seed)
        subset |= s["subset"] is not None
        empty |= (s["sizes"][1] == 0 if s["subset"] is None else len(s["subset"]) == 0)
        bij |= any(m["arity"] == 1 and m["values"].shape[0] == s["targets"][m["target"]]
                   and len(np.unique(m["values"])) == m["values"].shape[0] > 1
                   for m in s["maps"])
        for a in s["args"]:
            seen.add((a["kind"], a["access"]))
            seen.add(a["dtype"])
    want = {("direct", x) for x in F.DIRECT_ACCESS} | {("global", x) for x in F.GLOBAL_ACCESS} \
        | {("indirect", x) for x in F.INDIRECT_ACCESS} | {"float64", "int32"}
    assert want <= seen
    assert subset and empty and bij


@pytest.fixture(params=STRATEGIES)
def strategy(request, gpu_op2):
    from pyop2_gb300.configuration import configuration
    old = configuration["scatter"]
    configuration["scatter"] = request.param
    yield request.param
    configuration["scatter"] = old


@pytest.mark.gpu
@pytest.mark.parametrize("seed", GPU_SEEDS)
def test_gpu_matches_oracle(gpu_op2, oracle_op2, strategy, seed):
    spec = F.make_spec(seed)
    _equal(F.run(gpu_op2, spec), F.run(oracle_op2, spec))


def test_extruded_specs_cover_regions_and_layouts(oracle_op2):
    """The seeds draw every iteration region, every layer layout (constant,
    per-entity, periodic) and both settings of the layer argument; each
    spec runs on the oracle."""
    seen = set()
    for seed in GPU_SEEDS:
        s = F.make_extruded_spec(seed)
        lay = "periodic" if s["periodic"] else \
            ("constant" if isinstance(s["layers"], int) else "variable")
        seen.add((s["region"], lay))
        seen.add(("layer_arg", s["layer_arg"]))
        F.run_extruded(oracle_op2, s)
    regions = {r for r, lay in seen if r in F.REGIONS}
    layouts = {lay for r, lay in seen if r in F.REGIONS}
    assert regions == set(F.REGIONS)
    assert layouts == {"constant", "variable", "periodic"}
    assert ("layer_arg", True) in seen and ("layer_arg", False) in seen


@pytest.mark.gpu
@pytest.mark.parametrize("seed", GPU_SEEDS)
def test_gpu_matches_oracle_extruded(gpu_op2, oracle_op2, strategy, seed):
    spec = F.make_extruded_spec(seed)
    _equal(F.run_extruded(gpu_op2, spec), F.run_extruded(oracle_op2, spec))
