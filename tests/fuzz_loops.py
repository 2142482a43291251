"""Random par_loop signatures for differential tests.

``make_spec(seed)`` draws one loop: an iteration set with random
core/owned/total sizes (or a Subset of one), up to three target sets, maps of
arity 1-4 (sometimes also a PermutedMap of one of them, a ComposedMap through
an intermediate set, and a bijection onto a set as large as the iteration
set), and one to six arguments -- direct Dats (READ, WRITE, RW,
INC), indirect Dats (READ, INC, MIN, MAX; WRITE and RW only through the
bijection, where the result does not depend on the order of iteration),
Globals (READ, INC, MIN, MAX) and sometimes a MixedDat through a MixedMap
(READ or INC, one concatenated pack) -- of dimension 1-4 and dtype float64,
float32, int32 or int64.
The kernel is generated C: it sums its inputs with fixed integer weights and
writes integer-valued results into every written argument, so every
implementation must agree bit for bit whatever its order of summation.

``run(op2, spec)`` builds and runs the loop with an op2 module (the GPU
package or the oracle) and returns the final contents of every Dat and
Global; ``model(spec)`` computes the same from the access semantics alone
(pyop2/codegen/builder.py:240-410: READ packs gathered, INC packs zeroed and
added back, MIN/MAX packs initialised from the target and reduced back,
direct arguments pointing at the entity; pyop2/parloop.py:243-260: entities
0 .. size-1, ghosts never iterated), in a plain Python loop over entities.

``make_extruded_spec(seed)`` / ``run_extruded(op2, spec)`` draw and run the
extruded counterpart: a column mesh (constant or per-entity layers, or
periodic), iterated whole or through a Subset of its columns, an iteration
region, maps with per-entry layer offsets (and
offset quotients when periodic), the layer argument or not, and arguments
whose results do not depend on the order of iteration (indirect READ, INC,
MIN, MAX; direct READ and INC on the base set; Globals).  They are compared
between implementations only.
"""
import numpy as np

CTYPES = {"float64": "double", "float32": "float", "int32": "int", "int64": "long long"}


def _dtype_of(u):
    # every value the kernels produce is an integer small enough to be exact
    # in each of these types
    return "float64" if u < 0.6 else "int32" if u < 0.75 else "float32" if u < 0.875 else "int64"


DIRECT_ACCESS = ["READ", "WRITE", "RW", "INC"]
INDIRECT_ACCESS = ["READ", "INC", "MIN", "MAX"]
BIJECTION_ACCESS = ["READ", "INC", "MIN", "MAX", "WRITE", "RW"]
GLOBAL_ACCESS = ["READ", "INC", "MIN", "MAX"]


def make_spec(seed, data_seed=None):
    """One random loop.  The signature (argument kinds, accesses, dims,
    dtypes, map kinds and arities) is drawn from `seed`; sizes, map values
    and data from `data_seed` (default: derived from `seed`), so that specs
    sharing a seed and differing in data_seed are loops of one signature
    over different meshes (a batch)."""
    rs = np.random.default_rng(seed)
    rd = np.random.default_rng(1_000_000 + (seed if data_seed is None else data_seed))
    # a third stream for draws added later, so that rs and rd draw what
    # they always drew
    rx = np.random.default_rng(2_000_000 + seed)
    want_subset = rs.random() < 0.25
    want_bij = rs.random() < 0.35
    total = int(rd.integers(1 if want_bij else 0, 160))
    owned = int(rd.integers(0, total + 1))
    core = int(rd.integers(0, owned + 1))
    subset = None
    if want_subset:
        # a Subset iterates its own indices, all of them owned
        core = owned = total
        subset = np.sort(rd.choice(total, int(rd.integers(0, total + 1)), replace=False))
    targets = [int(rd.integers(1, 60)) for _ in range(int(rs.integers(1, 4)))]
    maps = []
    for _ in range(int(rs.integers(1, 4))):
        t = int(rs.integers(0, len(targets)))
        a = int(rs.integers(1, 5))
        maps.append({"target": t, "arity": a,
                     "values": rd.integers(0, targets[t], (total, a)).astype(np.int32)})
    # index transforms: a PermutedMap of a plain map, and a ComposedMap
    # (an arity-1 map into an intermediate set, then a plain map from it)
    if rs.random() < 0.4:
        b = int(rs.integers(0, len(maps)))
        perm = rs.permutation(maps[b]["arity"]).astype(np.int32)
        maps.append({"kind": "perm", "base": b, "perm": perm, "target": maps[b]["target"],
                     "arity": maps[b]["arity"], "values": maps[b]["values"][:, perm]})
    if rs.random() < 0.4:
        ni = int(rd.integers(1, 40))
        t = int(rs.integers(0, len(targets)))
        a = int(rs.integers(1, 5))
        outer = rd.integers(0, targets[t], (ni, a)).astype(np.int32)
        inner = rd.integers(0, ni, (total, 1)).astype(np.int32)
        maps.append({"kind": "composed", "ni": ni, "outer": outer, "inner": inner, "target": t,
                     "arity": a, "values": outer[inner[:, 0]].reshape(total, a)})
    bij = None
    if want_bij:
        targets.append(total)
        bij = len(maps)
        maps.append({"target": len(targets) - 1, "arity": 1,
                     "values": rd.permutation(total).astype(np.int32).reshape(total, 1)})
    args = []
    for _ in range(int(rs.integers(1, 7))):
        kind = rs.choice(["direct", "indirect", "global"], p=[0.3, 0.45, 0.25])
        dtype = _dtype_of(rs.random())
        dim = int(rs.integers(1, 4))
        if dim == 3 and rx.random() < 0.5:
            dim = 4      # rows of 16 / 32 bytes: the aligned wrapper variant
        if kind == "direct":
            acc = str(rs.choice(DIRECT_ACCESS))
            mp = None
        elif kind == "indirect":
            mp = int(rs.integers(0, len(maps)))
            acc = str(rs.choice(BIJECTION_ACCESS if mp == bij else INDIRECT_ACCESS))
        else:
            acc = str(rs.choice(GLOBAL_ACCESS))
            mp = None
        if kind == "global":
            shape = (dim,)
        else:
            size = total if mp is None else targets[maps[mp]["target"]]
            shape = (size, dim)
        init = rd.integers(-4, 5, shape)
        if kind == "global" and acc in ("MIN", "MAX"):
            init = init * 1000
        args.append({"kind": kind, "dtype": dtype, "dim": dim, "access": acc, "map": mp,
                     "init": init})
    if rs.random() < 0.3:
        # a MixedDat argument through a MixedMap: 2-3 components, each on its
        # own set through its own map, one concatenated pack
        comps = []
        for _ in range(int(rs.integers(2, 4))):
            targets.append(int(rd.integers(1, 30)))
            a = int(rs.integers(1, 4))
            maps.append({"target": len(targets) - 1, "arity": a,
                         "values": rd.integers(0, targets[-1], (total, a)).astype(np.int32)})
            dim = int(rs.integers(1, 4))
            comps.append({"map": len(maps) - 1, "dim": dim,
                          "init": rd.integers(-4, 5, (targets[-1], dim))})
        args.insert(int(rs.integers(0, len(args) + 1)),
                    {"kind": "mixed", "dtype": "float64", "access": str(rs.choice(["READ", "INC"])),
                     "map": None, "dim": None, "comps": comps,
                     "init": np.concatenate([c["init"].reshape(-1) for c in comps])})
    spec = {"seed": seed, "sizes": (core, owned, total), "subset": subset, "targets": targets,
            "maps": maps, "args": args}
    spec["code"], spec["name"] = kernel_code(spec)
    return spec


def _width(spec, a):
    if a["kind"] == "mixed":
        return sum(spec["maps"][c["map"]]["arity"] * c["dim"] for c in a["comps"])
    if a["map"] is None:
        return a["dim"]
    return spec.get("nfacets", 1) * spec["maps"][a["map"]]["arity"] * a["dim"]


def kernel_code(spec):
    """C source of the loop's kernel: s = sum_k sum_i (i + 1 + k) * in_k[i] over
    the READ and RW arguments, then, for argument k and pack slot i,
    INC: += s + i + k;  WRITE: = s - i - k;  RW: = 2 * old + s + k;
    MIN: = min(old, s + i - k);  MAX: = max(old, s - i + k)."""
    name = "fz%d" % spec["seed"]
    params, reads, writes = [], [], []
    for k, a in enumerate(spec["args"]):
        t = CTYPES[a["dtype"]]
        n = _width(spec, a)
        const = "const " if a["access"] == "READ" else ""
        params.append("%s%s *a%d" % (const, t, k))
        if a["access"] in ("READ", "RW"):
            reads.append("  for (int i = 0; i < %d; ++i) s += (double)(i + 1 + %d) * (double)a%d[i];"
                         % (n, k, k))
        acc = a["access"]
        if acc == "READ":
            continue
        if acc == "INC":
            e = "a%d[i] += (%s)(s + i + %d);" % (k, t, k)
        elif acc == "WRITE":
            e = "a%d[i] = (%s)(s - i - %d);" % (k, t, k)
        elif acc == "RW":
            e = "a%d[i] = (%s)(2.0 * (double)a%d[i] + s + %d);" % (k, t, k, k)
        elif acc == "MIN":
            e = "{ %s v = (%s)(s + i - %d); if (v < a%d[i]) a%d[i] = v; }" % (t, t, k, k, k)
        else:
            e = "{ %s v = (%s)(s - i + %d); if (v > a%d[i]) a%d[i] = v; }" % (t, t, k, k, k)
        writes.append("  for (int i = 0; i < %d; ++i) %s" % (n, e))
    if spec.get("layer_arg"):
        params.append("int layer")
        reads.append("  s += 3.0 * (double)layer;")
    body = "\n".join(["  double s = 0.0;"] + reads + writes)
    return "static void %s(%s)\n{\n%s\n}\n" % (name, ", ".join(params), body), name


def run(op2, spec):
    knl, it, largs, objs = build_loop(op2, spec)
    op2.par_loop(knl, it, *largs)
    return _results(objs, spec)


def run_batch(op2, specs, replay=False):
    """Loops of one signature (make_spec(seed, d) for several d): one
    BatchedParLoop on the GPU package (or, with replay, its graph replayed
    once), one par_loop each on the oracle."""
    built = [build_loop(op2, s) for s in specs]
    if op2.__name__.startswith("pyop2_gb300"):
        from pyop2_gb300.batch import BatchedParLoop
        b = BatchedParLoop([op2.ParLoop(k, it, *la) for k, it, la, _ in built], chunk=16)
        if replay:
            b.replay()
        else:
            b.compute()
    else:
        for k, it, la, _ in built:
            op2.par_loop(k, it, *la)
    return [_results(objs, s) for (_, _, _, objs), s in zip(built, specs)]


def build_loop(op2, spec):
    core, owned, total = spec["sizes"]
    iterset = op2.Set((core, owned, total), "it")
    targets = [op2.Set(n, "t%d" % i) for i, n in enumerate(spec["targets"])]
    maps = []
    for i, m in enumerate(spec["maps"]):
        kind = m.get("kind", "plain")
        if kind == "perm":
            maps.append(op2.PermutedMap(maps[m["base"]], m["perm"]))
        elif kind == "composed":
            mid = op2.Set(m["ni"], "mid%d" % i)
            outer = op2.Map(mid, targets[m["target"]], m["arity"], m["outer"], "o%d" % i)
            inner = op2.Map(iterset, mid, 1, m["inner"], "i%d" % i)
            maps.append(op2.ComposedMap(outer, inner))
        else:
            maps.append(op2.Map(iterset, targets[m["target"]], m["arity"], m["values"],
                                "m%d" % i))
    objs, largs = [], []
    for a in spec["args"]:
        dt = np.dtype(a["dtype"])
        acc = getattr(op2, a["access"])
        if a["kind"] == "global":
            g = op2.Global(a["dim"], a["init"].astype(dt), dt)
            objs.append(g)
            largs.append(g(acc))
            continue
        if a["kind"] == "mixed":
            dats = [op2.Dat(targets[spec["maps"][c["map"]]["target"]] ** c["dim"],
                            c["init"].astype(dt), dt) for c in a["comps"]]
            md = op2.MixedDat(dats)
            objs.append(md)
            largs.append(md(acc, op2.MixedMap([maps[c["map"]] for c in a["comps"]])))
            continue
        s = iterset if a["map"] is None else targets[spec["maps"][a["map"]]["target"]]
        d = op2.Dat(s ** a["dim"], a["init"].astype(dt), dt)
        objs.append(d)
        largs.append(d(acc) if a["map"] is None else d(acc, maps[a["map"]]))
    it = iterset if spec["subset"] is None else op2.Subset(iterset, spec["subset"])
    return op2.Kernel(spec["code"], spec["name"]), it, largs, objs


def _results(objs, spec):
    # every entry, ghosts included (the reference's data_ro stops at the
    # owned entries; the oracle keeps no such distinction)
    out = []
    for o, a in zip(objs, spec["args"]):
        if a["kind"] == "global":
            out.append(np.array(o.data_ro).reshape(-1))
        elif a["kind"] == "mixed":
            out.append(np.concatenate([
                np.array(getattr(d, "data_ro_with_halos", d.data_ro)).reshape(-1) for d in o]))
        else:
            out.append(np.array(getattr(o, "data_ro_with_halos", o.data_ro))
                       .reshape(a["init"].shape))
    return out


def model(spec):
    core, owned, total = spec["sizes"]
    data = [[c["init"].astype(a["dtype"]).copy() for c in a["comps"]] if a["kind"] == "mixed"
            else a["init"].astype(a["dtype"]).copy() for a in spec["args"]]
    ents = range(owned) if spec["subset"] is None else spec["subset"]
    for e in ents:
        e = int(e)
        rows = []
        for a in spec["args"]:
            if a["kind"] == "global":
                rows.append(None)
            elif a["kind"] == "mixed":
                rows.append([[int(v) for v in spec["maps"][c["map"]]["values"][e]]
                             for c in a["comps"]])
            elif a["map"] is None:
                rows.append([e])
            else:
                rows.append([int(v) for v in spec["maps"][a["map"]]["values"][e]])
        packs = []
        for k, a in enumerate(spec["args"]):
            if a["kind"] == "global":
                p = data[k].astype(np.float64).copy()
            elif a["kind"] == "mixed":
                p = np.concatenate([data[k][ci][r] for ci, rr in enumerate(rows[k])
                                    for r in rr]).astype(np.float64)
                if a["access"] == "INC":
                    p[:] = 0
            else:
                p = np.concatenate([data[k][r] for r in rows[k]]).astype(np.float64)
            if a["access"] == "INC" and a["map"] is not None:
                p[:] = 0
            packs.append(p)
        s = 0.0
        for k, a in enumerate(spec["args"]):
            if a["access"] in ("READ", "RW"):
                s += sum(float(i + 1 + k) * packs[k][i] for i in range(len(packs[k])))
        for k, a in enumerate(spec["args"]):
            acc, p = a["access"], packs[k]
            cast = (lambda v: float(v)) if a["dtype"].startswith("float") else \
                (lambda v: float(int(v)))
            for i in range(len(p)):
                if acc == "INC":
                    p[i] = p[i] + cast(s + i + k)
                elif acc == "WRITE":
                    p[i] = cast(s - i - k)
                elif acc == "RW":
                    p[i] = cast(2.0 * p[i] + s + k)
                elif acc == "MIN":
                    p[i] = min(p[i], cast(s + i - k))
                elif acc == "MAX":
                    p[i] = max(p[i], cast(s - i + k))
            if acc == "READ":
                continue
            if a["kind"] == "mixed":        # INC, component by component
                o = 0
                for ci, rr in enumerate(rows[k]):
                    d = a["comps"][ci]["dim"]
                    for r in rr:
                        data[k][ci][r] += p[o:o + d]
                        o += d
                continue
            if a["kind"] == "global":
                if acc == "INC":
                    data[k] += (p - data[k].astype(np.float64)).astype(data[k].dtype)
                else:
                    data[k][:] = p.astype(data[k].dtype)
                continue
            d = a["dim"]
            for j, r in enumerate(rows[k]):
                chunk = p[j * d:(j + 1) * d]
                if a["map"] is not None and acc == "INC":
                    data[k][r] += chunk.astype(data[k].dtype)
                elif acc == "MIN":
                    data[k][r] = np.minimum(data[k][r], chunk.astype(data[k].dtype))
                elif acc == "MAX":
                    data[k][r] = np.maximum(data[k][r], chunk.astype(data[k].dtype))
                else:
                    data[k][r] = chunk.astype(data[k].dtype)
    return [np.concatenate([c.reshape(-1) for c in x]) if a["kind"] == "mixed"
            else x.reshape(-1) if a["kind"] == "global" else x.reshape(a["init"].shape)
            for x, a in zip(data, spec["args"])]


# ------------------------------------------------------------------ extruded
EXT_INDIRECT_ACCESS = ["READ", "INC", "MIN", "MAX"]
EXT_DIRECT_ACCESS = ["READ", "INC"]
REGIONS = ["ALL", "ON_BOTTOM", "ON_TOP", "ON_INTERIOR_FACETS"]
LTOP = 7      # largest top layer of a column
LNODES = 9    # node numbers reserved per base node (>= LTOP + 2)


def make_extruded_spec(seed):
    rng = np.random.default_rng(10_000 + seed)
    nb = int(rng.integers(0, 14))
    kind = rng.choice(["constant", "variable", "periodic"])
    if kind == "variable":
        bottom = rng.integers(0, 3, nb)
        layers = np.stack([bottom, bottom + rng.integers(2, LTOP - 1, nb)], axis=1)
        layers = np.minimum(layers, LTOP).astype(np.int32)
    else:
        layers = int(rng.integers(2, LTOP + 1))
    region = str(rng.choice(REGIONS))
    nf = 2 if region == "ON_INTERIOR_FACETS" else 1
    targets = [int(rng.integers(1, 12)) for _ in range(int(rng.integers(1, 3)))]
    maps = []
    for _ in range(int(rng.integers(1, 4))):
        t = int(rng.integers(0, len(targets)))
        a = int(rng.integers(1, 5))
        base_nodes = rng.integers(0, targets[t], (nb, a))
        m = {"target": t, "arity": a, "values": (base_nodes * LNODES + 1).astype(np.int32),
             "offset": rng.integers(0, 2, a).astype(np.int32)}
        if kind == "periodic":
            m["offset_quotient"] = rng.integers(0, 2, a).astype(np.int32)
        maps.append(m)
    args = []
    for _ in range(int(rng.integers(1, 6))):
        k = rng.choice(["direct", "indirect", "global"], p=[0.25, 0.5, 0.25])
        dtype = _dtype_of(rng.random())
        dim = int(rng.integers(1, 4))
        mp = None
        if k == "direct":
            acc = str(rng.choice(EXT_DIRECT_ACCESS))
            shape = (nb, dim)
        elif k == "indirect":
            mp = int(rng.integers(0, len(maps)))
            acc = str(rng.choice(EXT_INDIRECT_ACCESS))
            shape = (targets[maps[mp]["target"]] * LNODES, dim)
        else:
            acc = str(rng.choice(GLOBAL_ACCESS))
            shape = (dim,)
        init = rng.integers(-4, 5, shape)
        if k == "global" and acc in ("MIN", "MAX"):
            init = init * 1000
        args.append({"kind": k, "dtype": dtype, "dim": dim, "access": acc, "map": mp,
                     "init": init})
    subset = None
    if nb > 0 and rng.random() < 0.25:
        subset = np.sort(rng.choice(nb, int(rng.integers(0, nb + 1)), replace=False))
    spec = {"seed": 10_000 + seed, "nb": nb, "layers": layers, "periodic": kind == "periodic",
            "region": region, "nfacets": nf, "layer_arg": bool(rng.random() < 0.5),
            "targets": targets, "maps": maps, "args": args, "subset": subset}
    spec["code"], spec["name"] = kernel_code(spec)
    return spec


def run_extruded(op2, spec):
    base = op2.Set(spec["nb"], "base")
    if spec["periodic"]:
        ext = op2.ExtrudedSet(base, spec["layers"], extruded_periodic=True)
    else:
        ext = op2.ExtrudedSet(base, spec["layers"])
    targets = [op2.Set(n * LNODES, "t%d" % i) for i, n in enumerate(spec["targets"])]
    maps = []
    for i, m in enumerate(spec["maps"]):
        kw = {"offset": m["offset"]}
        if "offset_quotient" in m:
            kw["offset_quotient"] = m["offset_quotient"]
        maps.append(op2.Map(ext, targets[m["target"]], m["arity"], m["values"], "m%d" % i, **kw))
    objs, largs = [], []
    for a in spec["args"]:
        dt = np.dtype(a["dtype"])
        acc = getattr(op2, a["access"])
        if a["kind"] == "global":
            g = op2.Global(a["dim"], a["init"].astype(dt), dt)
            objs.append(g)
            largs.append(g(acc))
            continue
        s = base if a["map"] is None else targets[spec["maps"][a["map"]]["target"]]
        d = op2.Dat(s ** a["dim"], a["init"].astype(dt), dt)
        objs.append(d)
        largs.append(d(acc) if a["map"] is None else d(acc, maps[a["map"]]))
    it = ext if spec.get("subset") is None else op2.Subset(ext, spec["subset"])
    op2.par_loop(op2.Kernel(spec["code"], spec["name"]), it, *largs,
                 iteration_region=getattr(op2, spec["region"]),
                 pass_layer_arg=spec["layer_arg"])
    return _results(objs, spec)


# ------------------------------------------------------------------ matrices
def make_mat_spec(seed):
    """A random sparsity and its assembly: 1-3 (row map, column map) pairs
    over one iteration set (flat, or extruded under random iteration
    regions), block shapes rdim x cdim in 1..3, square spaces (diagonal
    entries added) or rectangular ones, map entries sometimes -1 (ignored by
    the pattern and by insertion).  Element matrices are integer-valued, so
    the assembled values and the product with an integer x are exact."""
    rng = np.random.default_rng(20_000 + seed)
    extruded = bool(rng.random() < 0.5)
    square = bool(rng.random() < 0.5)
    rdim = int(rng.integers(1, 4))
    cdim = rdim if square else int(rng.integers(1, 4))
    nit = int(rng.integers(0, 16 if extruded else 120))
    nr = int(rng.integers(1, 12 if extruded else 60))
    nc = nr if square else int(rng.integers(1, 12 if extruded else 60))
    spec = {"seed": 20_000 + seed, "extruded": extruded, "square": square, "rdim": rdim,
            "cdim": cdim, "nit": nit, "nr": nr, "nc": nc,
            "block_sparse": bool(rng.random() < 0.5)}
    if extruded:
        kind = rng.choice(["constant", "variable", "periodic"])
        if kind == "variable":
            bottom = rng.integers(0, 3, nit)
            layers = np.stack([bottom, bottom + rng.integers(2, LTOP - 1, nit)], axis=1)
            spec["layers"] = np.minimum(layers, LTOP).astype(np.int32)
        else:
            spec["layers"] = int(rng.integers(2, LTOP + 1))
            if kind == "periodic":
                # at least 2 cell layers: with one, the reference's wrappers
                # (a remainder by one conditional subtraction,
                # pyop2/codegen/builder.py:27-30) and its sparsity (a true
                # modulo, pyop2/sparsity.pyx:376-384) place interior-facet
                # entries with offset quotients differently
                spec["layers"] = max(spec["layers"], 3)
        spec["periodic"] = kind == "periodic"

    def a_map(n_to):
        a = int(rng.integers(1, 5))
        v = rng.integers(0, n_to, (nit, a))
        if extruded:
            v = v * LNODES + 1
        elif rng.random() < 0.25 and v.size:
            # negative entries (flat maps only: a layer offset would move
            # them back into range)
            v[rng.random(v.shape) < 0.2] = -1
        m = {"arity": a, "values": v.astype(np.int32)}
        if extruded:
            m["offset"] = rng.integers(0, 2, a).astype(np.int32)
            if spec["periodic"]:
                m["offset_quotient"] = rng.integers(0, 2, a).astype(np.int32)
        return m

    rmaps = [a_map(nr) for _ in range(int(rng.integers(1, 3)))]
    cmaps = rmaps if square and rng.random() < 0.5 else \
        [a_map(nc) for _ in range(int(rng.integers(1, 3)))]
    pairs = []
    for _ in range(int(rng.integers(1, 4))):
        ri, ci = int(rng.integers(0, len(rmaps))), int(rng.integers(0, len(cmaps)))
        if extruded:
            k = int(rng.integers(1, 3))
            regions = sorted(set(str(r) for r in rng.choice(REGIONS, k)))
        else:
            regions = ["ALL"]
        pairs.append((ri, ci, regions))
    # Per-entity layers with a bottom above 0: the reference's sparsity
    # offsets by the absolute layer modulo the entity's layer count
    # (pyop2/sparsity.pyx:362-384) while its wrappers offset from the
    # entity's bottom (pyop2/codegen/builder.py:100-103).  Both are restated
    # as they are, so only ALL-region loops (whose couplings agree as sets)
    # are assembled there; the pattern itself is compared for every region.
    spec["assemble_all_only"] = bool(extruded and not isinstance(spec["layers"], int)
                                     and np.any(spec["layers"][:, 0] > 0))
    ncols = nc * (LNODES if extruded else 1)
    spec.update(rmaps=rmaps, cmaps=cmaps, shared_maps=cmaps is rmaps, pairs=pairs,
                w=rng.integers(-3, 4, nit), x=rng.integers(-3, 4, (ncols, cdim)))
    return spec


def _mat_kernel(nrow, ncol, name):
    return ("static void %s(double A[%d][%d], const double *w)\n{\n"
            "  for (int i = 0; i < %d; ++i)\n    for (int j = 0; j < %d; ++j)\n"
            "      A[i][j] += (double)((i + 1) * 3 - (j + 2) * (i %% 3)) + w[0];\n}\n"
            % (name, nrow, ncol, nrow, ncol))


def run_mat(op2, spec):
    """Build the sparsity, assemble every (pair, region) with an INC
    par_loop, and return the pattern, the row counts, the values and
    A x (the GPU package's Mat.mult; scipy on the oracle's matrix)."""
    nit = spec["nit"]
    if spec["extruded"]:
        base = op2.Set(nit, "base")
        it = op2.ExtrudedSet(base, spec["layers"], extruded_periodic=True) \
            if spec["periodic"] else op2.ExtrudedSet(base, spec["layers"])
        rset = op2.Set(spec["nr"] * LNODES, "rows")
        cset = rset if spec["square"] else op2.Set(spec["nc"] * LNODES, "cols")
        wset = base
    else:
        it = op2.Set(nit, "it")
        rset = op2.Set(spec["nr"], "rows")
        cset = rset if spec["square"] else op2.Set(spec["nc"], "cols")
        wset = it
    rds = rset ** spec["rdim"]
    cds = rds if spec["square"] else cset ** spec["cdim"]

    def mk(m, to, name):
        kw = {}
        if spec["extruded"]:
            kw["offset"] = m["offset"]
            if "offset_quotient" in m:
                kw["offset_quotient"] = m["offset_quotient"]
        return op2.Map(it, to, m["arity"], m["values"], name, **kw)

    rmaps = [mk(m, rset, "r%d" % i) for i, m in enumerate(spec["rmaps"])]
    cmaps = rmaps if spec["shared_maps"] else \
        [mk(m, cset, "c%d" % i) for i, m in enumerate(spec["cmaps"])]
    triples = [(rmaps[ri], cmaps[ci], tuple(getattr(op2, r) for r in regs))
               for ri, ci, regs in spec["pairs"]]
    sp = op2.Sparsity((rds, cds), triples, block_sparse=spec["block_sparse"])
    A = op2.Mat(sp)
    w = op2.Dat(wset, spec["w"].astype(np.float64))
    for ri, ci, regs in spec["pairs"]:
        rm, cm = rmaps[ri], cmaps[ci]
        for r in regs:
            if spec["assemble_all_only"] and r != "ALL":
                continue
            nf = 2 if r == "ON_INTERIOR_FACETS" else 1
            name = "am%d_%d_%d_%d" % (nf * rm.arity * spec["rdim"], nf * cm.arity * spec["cdim"],
                                      spec["rdim"], spec["cdim"])
            k = op2.Kernel(_mat_kernel(nf * rm.arity * spec["rdim"],
                                       nf * cm.arity * spec["cdim"], name), name)
            kw = {"iteration_region": getattr(op2, r)} if spec["extruded"] else {}
            op2.par_loop(k, it, A(op2.INC, (rm, cm)), w(op2.READ), **kw)
    A.assemble()
    if hasattr(sp, "csr"):
        rowptr, colidx = sp.csr()
        values = A.csr()[2]
        x = op2.Dat(cds, spec["x"].astype(np.float64))
        y = op2.Dat(rds)
        A.mult(x, y)
        yv = np.array(y.data_ro_with_halos).reshape(-1)
        nnz = np.array(sp.nnz)
    else:
        rowptr, colidx, values = sp.rowptr, sp.colidx, A.values_bcsr
        yv = A.to_scipy() @ spec["x"].astype(np.float64).reshape(-1)
        nnz = np.array(sp.nnz)
    return {"rowptr": np.asarray(rowptr, dtype=np.int64), "colidx": np.asarray(colidx),
            "nnz": nnz.astype(np.int64),
            "values": np.asarray(values, dtype=np.float64).reshape(-1), "y": yv}


def _layer_range(spec, e, region, for_sparsity):
    """Cell layers an extruded loop (or the sparsity) visits on entity e:
    pyop2/sparsity.pyx:344-361 and pyop2/codegen/builder.py:768-788."""
    lay = spec["layers"]
    if isinstance(lay, int):
        start, end = 0, lay - 1
    else:
        start, end = int(lay[e, 0]), int(lay[e, 1]) - 1
    bottom, nl = start, end - start
    if region == "ON_BOTTOM":
        end = start + 1
    elif region == "ON_TOP":
        start = end - 1
    elif region == "ON_INTERIOR_FACETS" and not spec["periodic"]:
        end = end - 1
    return range(start, end), bottom, nl


def _rem(a, b):
    return a if a < b else a - b


def _entries(spec, m, e, region, layer, bottom, nl, for_sparsity):
    """Indices of map m on entity e at `layer` (both facets for interior
    facets): the sparsity offsets by the absolute layer modulo the layer
    count (pyop2/sparsity.pyx:371-384), a wrapper from the entity's bottom
    (pyop2/codegen/builder.py:100-122)."""
    a = m["arity"]
    nf = 2 if region == "ON_INTERIOR_FACETS" else 1
    out = []
    for i in range(nf * a):
        k, irem = divmod(i, a)
        v = int(m["values"][e, irem])
        if spec.get("extruded", True):
            q = int(m["offset_quotient"][irem]) if "offset_quotient" in m else 0
            off = int(m["offset"][irem])
            if for_sparsity:
                v += off * ((layer + k + q) % nl - q % nl)
            elif spec["periodic"]:
                # the wrappers' remainder is one conditional subtraction
                # (pyop2/codegen/builder.py:27-30)
                v += off * (_rem(layer - bottom + k + q, nl) - _rem(q, nl))
            else:
                v += off * (layer - bottom + k)
        out.append(v)
    return out


def _visits(spec, ri, ci, region, for_sparsity):
    for e in range(spec["nit"]):
        if not spec["extruded"]:
            yield e, (_entries(spec, spec["rmaps"][ri], e, region, 0, 0, 1, for_sparsity),
                      _entries(spec, spec["cmaps"][ci], e, region, 0, 0, 1, for_sparsity))
            continue
        layers, bottom, nl = _layer_range(spec, e, region, for_sparsity)
        for layer in layers:
            yield e, (_entries(spec, spec["rmaps"][ri], e, region, layer, bottom, nl,
                               for_sparsity),
                      _entries(spec, spec["cmaps"][ci], e, region, layer, bottom, nl,
                               for_sparsity))


def mat_model(spec):
    """The pattern (sorted distinct columns per block row, the diagonal on a
    square space, negative indices ignored), the row counts, the assembled
    values and A x of a make_mat_spec spec, in plain Python."""
    L = LNODES if spec["extruded"] else 1
    nrows, ncols = spec["nr"] * L, spec["nc"] * L
    rdim, cdim = spec["rdim"], spec["cdim"]
    pattern = [set() for _ in range(nrows)]
    for ri, ci, regions in spec["pairs"]:
        for region in regions:
            for _, (rows, cols) in _visits(spec, ri, ci, region, True):
                for r in rows:
                    if r >= 0:
                        pattern[r].update(c for c in cols if c >= 0)
    if spec["square"]:
        for i in range(min(nrows, ncols)):
            pattern[i].add(i)
    rowptr = np.zeros(nrows + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum([len(p) for p in pattern])
    colidx = np.array([c for p in pattern for c in sorted(p)], dtype=np.int32)
    where = [{c: k for k, c in enumerate(sorted(p))} for p in pattern]
    values = np.zeros((len(colidx), rdim, cdim))
    for ri, ci, regions in spec["pairs"]:
        for region in regions:
            if spec["assemble_all_only"] and region != "ALL":
                continue
            for e, (rows, cols) in _visits(spec, ri, ci, region, False):
                w = float(spec["w"][e])
                for i in range(len(rows) * rdim):
                    r = rows[i // rdim]
                    if r < 0:
                        continue
                    for j in range(len(cols) * cdim):
                        c = cols[j // cdim]
                        if c < 0:
                            continue
                        v = (i + 1) * 3 - (j + 2) * (i % 3) + w
                        values[rowptr[r] + where[r][c], i % rdim, j % cdim] += v
    counts = np.diff(rowptr)
    if not (spec["block_sparse"] and rdim == cdim):
        counts = np.repeat(counts * cdim, rdim)
    x = spec["x"].astype(np.float64).reshape(ncols, cdim)
    y = np.zeros((nrows, rdim))
    for r in range(nrows):
        for k in range(rowptr[r], rowptr[r + 1]):
            y[r] += values[k] @ x[colidx[k]]
    return {"rowptr": rowptr, "colidx": colidx, "nnz": counts.astype(np.int64),
            "values": values.reshape(-1), "y": y.reshape(-1)}


def model_extruded(spec):
    """The access semantics of a make_extruded_spec loop in plain Python:
    columns (or the Subset's columns) in order, the layers the iteration
    region visits (pyop2/codegen/builder.py:768-788), map entries offset
    from the column's bottom (both facets for interior facets), direct
    arguments indexed by the column, the layer argument added as 3 * layer."""
    data = [a["init"].astype(a["dtype"]).copy() for a in spec["args"]]
    ents = range(spec["nb"]) if spec.get("subset") is None else spec["subset"]
    for e in ents:
        e = int(e)
        layers, bottom, nl = _layer_range(spec, e, spec["region"], False)
        for layer in layers:
            rows = []
            for a in spec["args"]:
                if a["kind"] == "global":
                    rows.append(None)
                elif a["map"] is None:
                    rows.append([e])
                else:
                    rows.append(_entries(spec, spec["maps"][a["map"]], e, spec["region"],
                                         layer, bottom, nl, False))
            packs = []
            for k, a in enumerate(spec["args"]):
                if a["kind"] == "global":
                    p = data[k].astype(np.float64).copy()
                else:
                    p = np.concatenate([data[k][r] for r in rows[k]]).astype(np.float64)
                if a["access"] == "INC" and a["map"] is not None:
                    p[:] = 0
                packs.append(p)
            s = 0.0
            for k, a in enumerate(spec["args"]):
                if a["access"] in ("READ", "RW"):
                    s += sum(float(i + 1 + k) * packs[k][i] for i in range(len(packs[k])))
            if spec["layer_arg"]:
                s += 3.0 * layer
            for k, a in enumerate(spec["args"]):
                acc, p = a["access"], packs[k]
                if acc == "READ":
                    continue
                cast = (lambda v: float(v)) if a["dtype"].startswith("float") else \
                    (lambda v: float(int(v)))
                for i in range(len(p)):
                    if acc == "INC":
                        p[i] = p[i] + cast(s + i + k)
                    elif acc == "MIN":
                        p[i] = min(p[i], cast(s + i - k))
                    elif acc == "MAX":
                        p[i] = max(p[i], cast(s - i + k))
                if a["kind"] == "global":
                    if acc == "INC":
                        data[k] += (p - data[k].astype(np.float64)).astype(data[k].dtype)
                    else:
                        data[k][:] = p.astype(data[k].dtype)
                    continue
                d = a["dim"]
                for j, r in enumerate(rows[k]):
                    chunk = p[j * d:(j + 1) * d].astype(data[k].dtype)
                    if acc == "INC" and a["map"] is not None:
                        data[k][r] += chunk
                    elif acc == "INC":             # direct: the pack is the entity
                        data[k][r] = chunk
                    elif acc == "MIN":
                        data[k][r] = np.minimum(data[k][r], chunk)
                    else:
                        data[k][r] = np.maximum(data[k][r], chunk)
    return [x.reshape(-1) if a["kind"] == "global" else x.reshape(a["init"].shape)
            for x, a in zip(data, spec["args"])]
