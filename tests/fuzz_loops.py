"""Random par_loop signatures for differential tests.

``make_spec(seed)`` draws one loop: an iteration set with random
core/owned/total sizes (or a Subset of one), up to three target sets, maps of
arity 1-4 (one of them, sometimes, a bijection onto a set as large as the
iteration set), and one to six arguments -- direct Dats (READ, WRITE, RW,
INC), indirect Dats (READ, INC, MIN, MAX; WRITE and RW only through the
bijection, where the result does not depend on the order of iteration) and
Globals (READ, INC, MIN, MAX) -- of dimension 1-3 and dtype float64 or int32.
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
periodic), an iteration region, maps with per-entry layer offsets (and
offset quotients when periodic), the layer argument or not, and arguments
whose results do not depend on the order of iteration (indirect READ, INC,
MIN, MAX; direct READ and INC on the base set; Globals).  They are compared
between implementations only.
"""
import numpy as np

DIRECT_ACCESS = ["READ", "WRITE", "RW", "INC"]
INDIRECT_ACCESS = ["READ", "INC", "MIN", "MAX"]
BIJECTION_ACCESS = ["READ", "INC", "MIN", "MAX", "WRITE", "RW"]
GLOBAL_ACCESS = ["READ", "INC", "MIN", "MAX"]


def make_spec(seed):
    rng = np.random.default_rng(seed)
    total = int(rng.integers(0, 160))
    owned = int(rng.integers(0, total + 1))
    core = int(rng.integers(0, owned + 1))
    subset = None
    if rng.random() < 0.25:
        # a Subset iterates its own indices, all of them owned
        core = owned = total
        subset = np.sort(rng.choice(total, int(rng.integers(0, total + 1)), replace=False))
    targets = [int(rng.integers(1, 60)) for _ in range(int(rng.integers(1, 4)))]
    maps = []
    for _ in range(int(rng.integers(1, 4))):
        t = int(rng.integers(0, len(targets)))
        a = int(rng.integers(1, 5))
        maps.append({"target": t, "arity": a,
                     "values": rng.integers(0, targets[t], (total, a)).astype(np.int32)})
    bij = None
    if total > 0 and rng.random() < 0.35:
        targets.append(total)
        bij = len(maps)
        maps.append({"target": len(targets) - 1, "arity": 1,
                     "values": rng.permutation(total).astype(np.int32).reshape(total, 1)})
    args = []
    for _ in range(int(rng.integers(1, 7))):
        kind = rng.choice(["direct", "indirect", "global"], p=[0.3, 0.45, 0.25])
        dtype = "float64" if rng.random() < 0.75 else "int32"
        dim = int(rng.integers(1, 4))
        if kind == "direct":
            acc = str(rng.choice(DIRECT_ACCESS))
            mp = None
        elif kind == "indirect":
            mp = int(rng.integers(0, len(maps)))
            acc = str(rng.choice(BIJECTION_ACCESS if mp == bij else INDIRECT_ACCESS))
        else:
            acc = str(rng.choice(GLOBAL_ACCESS))
            mp = None
        if kind == "global":
            shape = (dim,)
        else:
            size = total if mp is None else targets[maps[mp]["target"]]
            shape = (size, dim)
        init = rng.integers(-4, 5, shape)
        if kind == "global" and acc in ("MIN", "MAX"):
            init = init * 1000
        args.append({"kind": kind, "dtype": dtype, "dim": dim, "access": acc, "map": mp,
                     "init": init})
    spec = {"seed": seed, "sizes": (core, owned, total), "subset": subset, "targets": targets,
            "maps": maps, "args": args}
    spec["code"], spec["name"] = kernel_code(spec)
    return spec


def _width(spec, a):
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
        t = "double" if a["dtype"] == "float64" else "int"
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
    core, owned, total = spec["sizes"]
    iterset = op2.Set((core, owned, total), "it")
    targets = [op2.Set(n, "t%d" % i) for i, n in enumerate(spec["targets"])]
    maps = [op2.Map(iterset, targets[m["target"]], m["arity"], m["values"], "m%d" % i)
            for i, m in enumerate(spec["maps"])]
    objs, largs = [], []
    for a in spec["args"]:
        dt = np.dtype(a["dtype"])
        acc = getattr(op2, a["access"])
        if a["kind"] == "global":
            g = op2.Global(a["dim"], a["init"].astype(dt), dt)
            objs.append(g)
            largs.append(g(acc))
            continue
        s = iterset if a["map"] is None else targets[spec["maps"][a["map"]]["target"]]
        d = op2.Dat(s ** a["dim"], a["init"].astype(dt), dt)
        objs.append(d)
        largs.append(d(acc) if a["map"] is None else d(acc, maps[a["map"]]))
    it = iterset if spec["subset"] is None else op2.Subset(iterset, spec["subset"])
    op2.par_loop(op2.Kernel(spec["code"], spec["name"]), it, *largs)
    return _results(objs, spec)


def _results(objs, spec):
    # every entry, ghosts included (the reference's data_ro stops at the
    # owned entries; the oracle keeps no such distinction)
    return [np.array(o.data_ro).reshape(-1) if a["kind"] == "global"
            else np.array(getattr(o, "data_ro_with_halos", o.data_ro)).reshape(a["init"].shape)
            for o, a in zip(objs, spec["args"])]


def model(spec):
    core, owned, total = spec["sizes"]
    data = [a["init"].astype(a["dtype"]).copy() for a in spec["args"]]
    ents = range(owned) if spec["subset"] is None else spec["subset"]
    for e in ents:
        e = int(e)
        rows = []
        for a in spec["args"]:
            if a["kind"] == "global":
                rows.append(None)
            elif a["map"] is None:
                rows.append([e])
            else:
                rows.append([int(v) for v in spec["maps"][a["map"]]["values"][e]])
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
        for k, a in enumerate(spec["args"]):
            acc, p = a["access"], packs[k]
            cast = (lambda v: float(v)) if a["dtype"] == "float64" else (lambda v: float(int(v)))
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
    return [x.reshape(-1) if a["kind"] == "global" else x.reshape(a["init"].shape)
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
        dtype = "float64" if rng.random() < 0.75 else "int32"
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
    spec = {"seed": 10_000 + seed, "nb": nb, "layers": layers, "periodic": kind == "periodic",
            "region": region, "nfacets": nf, "layer_arg": bool(rng.random() < 0.5),
            "targets": targets, "maps": maps, "args": args}
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
    op2.par_loop(op2.Kernel(spec["code"], spec["name"]), ext, *largs,
                 iteration_region=getattr(op2, spec["region"]),
                 pass_layer_arg=spec["layer_arg"])
    return _results(objs, spec)
