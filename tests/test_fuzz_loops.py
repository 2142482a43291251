"""Randomised differential tests of par_loop: random sets, maps and argument
lists (every access mode, direct and indirect, Globals, MixedDats through
MixedMaps, dims 1-3, float64, float32, int32 and int64, core/owned/total
splits, Subsets, and extruded column meshes under every iteration region)
with a generated kernel whose results are integers.  The oracle must equal
the access-semantics models bit for bit (CPU: flat, extruded and matrix
loops), and the GPU must equal the oracle bit for bit under every INC
strategy."""
import numpy as np
import pytest

import fuzz_loops as F

CPU_SEEDS = range(48)
GPU_SEEDS = range(48)
STRATEGIES = ["atomic", "warp", "colour", "shared", "staged", "atomic_cells2"]


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
    dtypes, plain, permuted and composed maps, MixedDat arguments, Subsets,
    empty iteration sets and the bijective map."""
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
            if a["map"] is not None:
                seen.add(("map", s["maps"][a["map"]].get("kind", "plain")))
    want = {("direct", x) for x in F.DIRECT_ACCESS} | {("global", x) for x in F.GLOBAL_ACCESS} \
        | {("indirect", x) for x in F.INDIRECT_ACCESS} | set(F.CTYPES) \
        | {("map", k) for k in ("plain", "perm", "composed")} \
        | {("mixed", "READ"), ("mixed", "INC")}
    assert want <= seen
    assert subset and empty and bij


@pytest.fixture(params=STRATEGIES)
def strategy(request, gpu_op2):
    from pyop2_gb300.configuration import configuration
    old = configuration["scatter"], configuration["cells_per_thread"]
    # "atomic_cells2": hardware atomics, two cells per thread per sweep step
    configuration["scatter"] = request.param.split("_")[0]
    configuration["cells_per_thread"] = 2 if request.param.endswith("cells2") else 1
    yield request.param
    configuration["scatter"], configuration["cells_per_thread"] = old


@pytest.mark.gpu
@pytest.mark.parametrize("seed", GPU_SEEDS)
def test_gpu_matches_oracle(gpu_op2, oracle_op2, strategy, seed):
    spec = F.make_spec(seed)
    _equal(F.run(gpu_op2, spec), F.run(oracle_op2, spec))


def test_extruded_specs_cover_regions_and_layouts(oracle_op2):
    """The seeds draw every iteration region, every layer layout (constant,
    per-entity, periodic), Subsets of columns and both settings of the layer
    argument; each spec runs on the oracle."""
    seen = set()
    for seed in GPU_SEEDS:
        s = F.make_extruded_spec(seed)
        lay = "periodic" if s["periodic"] else \
            ("constant" if isinstance(s["layers"], int) else "variable")
        seen.add((s["region"], lay))
        seen.add(("layer_arg", s["layer_arg"]))
        seen.add(("subset", s["subset"] is not None))
        F.run_extruded(oracle_op2, s)
    regions = {r for r, lay in seen if r in F.REGIONS}
    layouts = {lay for r, lay in seen if r in F.REGIONS}
    assert regions == set(F.REGIONS)
    assert layouts == {"constant", "variable", "periodic"}
    assert ("layer_arg", True) in seen and ("layer_arg", False) in seen
    assert ("subset", True) in seen


@pytest.mark.parametrize("seed", CPU_SEEDS)
def test_oracle_extruded_matches_model(oracle_op2, seed):
    """The oracle's extruded loops against the plain-Python statement of
    their layers, offsets and accesses."""
    spec = F.make_extruded_spec(seed)
    _equal(F.run_extruded(oracle_op2, spec), F.model_extruded(spec))


@pytest.mark.gpu
@pytest.mark.parametrize("seed", GPU_SEEDS)
def test_gpu_matches_oracle_extruded(gpu_op2, oracle_op2, strategy, seed):
    spec = F.make_extruded_spec(seed)
    _equal(F.run_extruded(gpu_op2, spec), F.run_extruded(oracle_op2, spec))


MAT_SEEDS = range(48)
MAT_KEYS = ("rowptr", "colidx", "nnz", "values", "y")


def _equal_mat(got, want):
    for k in MAT_KEYS:
        assert got[k].shape == want[k].shape, k
        assert np.array_equal(got[k], want[k]), k


@pytest.mark.parametrize("seed", MAT_SEEDS)
def test_oracle_mat_matches_model(oracle_op2, seed):
    """Random sparsities, assemblies and products: the oracle equals the
    plain Python restatement of sparsity.pyx and MatSetValuesBlockedLocal."""
    spec = F.make_mat_spec(seed)
    _equal_mat(F.run_mat(oracle_op2, spec), F.mat_model(spec))


def test_mat_specs_cover_shapes_and_layouts():
    seen = set()
    for seed in MAT_SEEDS:
        s = F.make_mat_spec(seed)
        seen.add(("extruded", s["extruded"]))
        seen.add(("square", s["square"]))
        seen.add(("block", s["rdim"], s["cdim"]))
        seen.add(("negative", any((m["values"] < 0).any() for m in s["rmaps"] + s["cmaps"])))
        seen.add(("all_only", s["assemble_all_only"]))
        if s["extruded"]:
            seen.add(("layers", "periodic" if s["periodic"] else
                      ("constant" if isinstance(s["layers"], int) else "variable")))
            for _, _, regs in s["pairs"]:
                seen.update(("region", r) for r in regs)
    for want in [("extruded", True), ("extruded", False), ("square", True), ("square", False),
                 ("negative", True), ("all_only", True), ("layers", "constant"),
                 ("layers", "variable"), ("layers", "periodic")] + \
            [("region", r) for r in F.REGIONS] + [("block", d, d) for d in (1, 2, 3)]:
        assert want in seen, want


@pytest.mark.gpu
@pytest.mark.parametrize("seed", MAT_SEEDS)
def test_gpu_mat_matches_oracle(gpu_op2, oracle_op2, seed):
    """GPU sparsity build (bit-exact pattern and row counts), INC assembly
    and SpMV (exact: integer values) against the oracle."""
    spec = F.make_mat_spec(seed)
    _equal_mat(F.run_mat(gpu_op2, spec), F.run_mat(oracle_op2, spec))


LAUNCH_CONFIGS = [dict(block_size=128, prefetch=1, grid=0),
                  dict(block_size=512, prefetch=0, grid=-1),
                  dict(block_size=64, prefetch=1, grid=3)]


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", LAUNCH_CONFIGS, ids=["bs128-pf", "bs512-uncapped", "bs64-pf-grid3"])
@pytest.mark.parametrize("seed", range(0, 48, 4))
def test_gpu_matches_oracle_launch_configs(gpu_op2, oracle_op2, cfg, seed):
    """Other CTA sizes, map-row prefetch and grid policies (uncapped, and 3
    CTAs striding over everything) under the atomic and warp strategies."""
    from pyop2_gb300.configuration import configuration
    old = {k: configuration[k] for k in list(cfg) + ["scatter"]}
    try:
        for k, v in cfg.items():
            configuration[k] = v
        for sc in ("atomic", "warp"):
            configuration["scatter"] = sc
            spec = F.make_spec(seed)
            _equal(F.run(gpu_op2, spec), F.run(oracle_op2, spec))
            spec = F.make_extruded_spec(seed)
            _equal(F.run_extruded(gpu_op2, spec), F.run_extruded(oracle_op2, spec))
    finally:
        for k, v in old.items():
            configuration[k] = v


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(1, 48, 6))
def test_gpu_autotuned_matches_oracle(gpu_op2, oracle_op2, seed):
    """configuration['scatter'] = 'auto': the autotuner runs every candidate
    on the loop's own arguments and restores them; the result must still be
    the oracle's, bit for bit."""
    from pyop2_gb300.configuration import configuration
    old = configuration["scatter"]
    configuration["scatter"] = "auto"
    try:
        spec = F.make_spec(seed)
        _equal(F.run(gpu_op2, spec), F.run(oracle_op2, spec))
        spec = F.make_extruded_spec(seed)
        _equal(F.run_extruded(gpu_op2, spec), F.run_extruded(oracle_op2, spec))
    finally:
        configuration["scatter"] = old


@pytest.mark.gpu
@pytest.mark.parametrize("replay", [False, True], ids=["launch", "graph"])
@pytest.mark.parametrize("seed", range(0, 48, 3))
def test_gpu_batch_matches_oracle(gpu_op2, oracle_op2, seed, replay):
    """Three loops of one random signature over different random meshes in
    one persistent batched launch (16-entity work items), launched directly
    or replayed from its CUDA graph, against the oracle running each loop."""
    specs = [F.make_spec(seed, 100 * seed + d) for d in range(3)]
    got = F.run_batch(gpu_op2, specs, replay=replay)
    want = F.run_batch(oracle_op2, specs)
    for g, w in zip(got, want):
        _equal(g, w)
