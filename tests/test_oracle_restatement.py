"""A second, independent restatement of the reference's gather in pure-Python loops, checked bit for bit
against the C oracle on small seeded grids: 1D/2D/3D stencils (named shapes, Annulus, Rectangle,
Positional) x boundaries (Remove, Wrap, Reflect, Use) x paddings (Conditional, Halo{:out}, Halo{:in}) x
reductions (mean, sum, minimum, maximum, kernelproduct, Life, diffusion) in Float64, Float32, UInt8 and
Int64, single maps and SwitchingStencilArray runs; scatterstencil! through the reference's pass schedule;
maps over several arrays (sums of centre / sum / mean / kernelproduct / value terms).  The reference's
own goldens use integer-valued data; this pins the oracle's boundary handling and fold order on random
floats as well.

Semantics restated here (reference file:line):
* neighbour J = I + o: Conditional Remove reads padval outside the array (src/array.jl:133-135);
  Conditional Wrap / Reflect read the per-axis bounded index (src/array.jl:150-175: Wrap i +- s,
  Reflect 2 - i and 2s - i in 1-based indices); Halo reads parent[J + R] (src/array.jl:347-349, 368-373).
* update_boundary! before each map (src/array.jl:195-239): a ring cell of logical index J gets padval
  (Remove) or the interior value at the per-axis bounded index of J (Wrap / Reflect, `halo_val`);
  Use and Conditional leave the parent alone.
* sum / mean / minimum / maximum fold left in offset order from the first value; mean divides by L;
  kernelproduct starts from zero and adds v * w per offset (src/stencils/kernel.jl:37-43); Life counts
  nonzero neighbours against the birth / survive sets; diffusion is c + alpha (s - L c), each operation
  rounded.
"""
import zlib

import numpy as np
import pytest

from _backends import OracleBackend


# ------------------------------------------------------------------ the restatement
def _bound(kind, i, n):
    if kind == "wrap":
        return i + n if i < 0 else (i - n if i >= n else i)
    return -i if i < 0 else (2 * n - 2 - i if i >= n else i)   # reflect, 0-based


def _update_ring(parent, shape, R, kind, padval):
    interior = parent[tuple(slice(R, R + n) for n in shape)].copy()
    for P in np.ndindex(*parent.shape):
        J = tuple(p - R for p in P)
        if all(0 <= j < n for j, n in zip(J, shape)):
            continue
        parent[P] = padval if kind == "remove" else interior[tuple(_bound(kind, j, n) for j, n in zip(J, shape))]


def _fold(red, vals, centre, T, L, weights, rule, alpha):
    if red in ("mean", "sum", "diffusion"):
        acc = T(vals[0])
        for v in vals[1:]:
            acc = T(acc + T(v))
        if red == "mean":
            return T(acc / T(L))
        if red == "sum":
            return acc
        c = T(centre)
        t = T(T(L) * c)
        t = T(acc - t)
        t = T(T(alpha) * t)
        return T(c + t)
    if red in ("minimum", "maximum"):
        acc = T(vals[0])
        for v in vals[1:]:
            v = T(v)
            if (v < acc) if red == "minimum" else (v > acc):
                acc = v
        return acc
    if red == "kernelproduct":
        acc = 0.0
        for v, w in zip(vals, weights):
            acc = acc + float(v) * w
        return acc
    if red == "life":
        cnt = sum(1 for v in vals if v != 0)
        birth, survive = rule
        return int(cnt in (survive if centre != 0 else birth))
    raise ValueError(red)


def restated_map(parent, shape, R, offsets, bname, padval, halo, red, T, weights=None, rule=None, alpha=None,
                 out_dtype=None):
    """One map of the logical array held by `parent` (ring of width R when halo); updates the ring first
    like the reference's gatherstencil! (update_boundary!) and returns the logical result."""
    if halo and bname != "use":
        _update_ring(parent, shape, R, bname, padval)
    out = np.empty(shape, dtype=out_dtype or parent.dtype, order="F")
    L = len(offsets)
    for I in np.ndindex(*shape):
        vals = _hood(parent, shape, R, offsets, bname, padval, halo, I)
        centre = parent[tuple(i + R for i in I)] if halo else parent[I]
        out[I] = _fold(red, vals, centre, T, L, weights, rule, alpha)
    return out


def _hood(parent, shape, R, offsets, bname, padval, halo, I):
    """The neighbour values of logical cell I in offset order."""
    vals = []
    for o in offsets:
        J = tuple(I[d] + (o[d] if d < len(o) else 0) for d in range(parent.ndim))
        if halo:
            vals.append(parent[tuple(j + R for j in J)])
        elif all(0 <= j < n for j, n in zip(J, shape)):
            vals.append(parent[J])
        elif bname == "remove":
            vals.append(padval)
        else:
            vals.append(parent[tuple(_bound(bname, j, n) for j, n in zip(J, shape))])
    return vals


# ------------------------------------------------------------------ the matrix
def _stencils(st):
    return {
        "Window1": (st.Window(1), 2), "Window2": (st.Window(2), 2), "Moore1": (st.Moore(1), 2),
        "VonNeumann2": (st.VonNeumann(2), 2), "Circle2": (st.Circle(2), 2), "Cross1": (st.Cross(1), 2),
        "Annulus2": (st.Annulus(2), 2), "Diamond1": (st.Diamond(1), 2), "Cardinal1": (st.Cardinal(1), 2),
        "Ordinal1": (st.Ordinal(1), 2), "Rectangle": (st.Rectangle((-1, 2), (0, 1)), 2),
        "Positional": (st.Positional((-1, 0), (1, 1), (0, -1)), 2),
        "Moore1_3d": (st.Moore(1, 3), 3), "VonNeumann1_3d": (st.VonNeumann(1, 3), 3), "Cross1_3d": (st.Cross(1, 3), 3),
        "Window2_1d": (st.Window(2, 1), 1),
    }


STENCILS = ["Window1", "Window2", "Moore1", "VonNeumann2", "Circle2", "Cross1", "Annulus2", "Diamond1", "Cardinal1",
            "Ordinal1", "Rectangle", "Positional", "Moore1_3d", "VonNeumann1_3d", "Cross1_3d", "Window2_1d"]
OPS = [("mean", "F64"), ("sum", "F32"), ("minimum", "F64"), ("maximum", "F32"), ("kernelproduct", "F64"),
       ("diffusion", "F32"), ("life", "U8"), ("sum", "I64"), ("mean", "I64")]
BCPADS = [(b, p) for p in ("cond", "halo_out", "halo_in") for b in ("remove", "wrap", "reflect", "use")
          if not (b == "use" and p == "cond")]
SIZES = {1: (11,), 2: (9, 8), 3: (6, 5, 5)}


def _case_setup(st, abi, name, op, dt, rng):
    stencil, nd = _stencils(st)[name]
    npdt = {"F64": np.float64, "F32": np.float32, "U8": np.uint8, "I64": np.int64}[dt]
    shape = SIZES[nd]
    if dt in ("F64", "F32"):
        a = (rng.random(shape) * 2 - 1).astype(npdt)
    elif op == "life":
        a = (rng.random(shape) < 0.4).astype(npdt)
    else:
        a = rng.integers(-5, 9, size=shape).astype(npdt)
    T = {"F64": float, "F32": np.float32, "U8": int, "I64": int}[dt]
    if op == "mean" and dt == "I64":
        T = float
    red = {"mean": st.mean, "sum": st.sum, "minimum": st.minimum, "maximum": st.maximum,
           "kernelproduct": st.kernelproduct, "diffusion": st.Diffusion(0.1), "life": st.life}[op]
    weights = None
    if op == "kernelproduct":
        weights = [float(x) for x in rng.standard_normal(len(stencil))]
        stencil = st.Kernel(stencil, np.array(weights))
    return np.asfortranarray(a), stencil, red, T, weights, getattr(abi, dt)


def _padval(dt):
    return 0.5 if dt in ("F64", "F32") else 3


def _boundary(st, bname, dt):
    return {"remove": st.Remove(_padval(dt)), "wrap": st.Wrap(), "reflect": st.Reflect(), "use": st.Use()}[bname]


def _padding(st, pname):
    return {"cond": st.Conditional(), "halo_out": st.Halo("out"), "halo_in": st.Halo("in")}[pname]


def _restated(a, stencil, op, dt, bname, pname, T, weights, steps, out_dtype):
    R = stencil.radius
    offsets = (stencil.stencil if hasattr(stencil, "stencil") else stencil).offsets()
    padval = T(_padval(dt)) if dt in ("F64", "F32") else _padval(dt)
    halo = pname != "cond"
    if pname == "halo_out":
        parent = np.zeros(tuple(s + 2 * R for s in a.shape), dtype=a.dtype, order="F")
        parent[tuple(slice(R, R + s) for s in a.shape)] = a
    else:
        parent = a.copy(order="F")
    shape = tuple(s - 2 * R for s in parent.shape) if halo else parent.shape
    kw = dict(weights=weights, rule=((3,), (2, 3)), alpha=0.1, out_dtype=out_dtype)
    if steps == 0:
        return restated_map(parent, shape, R, offsets, bname, padval, halo, op, T, **kw)
    dest = parent.copy(order="F")
    for _ in range(steps):
        res = restated_map(parent, shape, R, offsets, bname, padval, halo, op, T, **kw)
        dest[tuple(slice(R, R + n) for n in shape) if halo else ...] = res
        parent, dest = dest, parent
    return np.asfortranarray(parent[tuple(slice(R, R + n) for n in shape)] if halo else parent)


@pytest.mark.parametrize("op,dt", OPS, ids=[f"{o}-{d}" for o, d in OPS])
@pytest.mark.parametrize("name", STENCILS)
def test_oracle_matches_restatement(st, orc, abi, name, op, dt):
    ora = OracleBackend(st, orc, abi)
    for bname, pname in BCPADS:
        rng = np.random.default_rng(zlib.crc32(repr((name, op, dt, bname, pname)).encode()))
        a, stencil, red, T, weights, code = _case_setup(st, abi, name, op, dt, rng)
        if op == "life" and len(stencil) > 31:
            continue
        out_dtype = np.float64 if (op == "kernelproduct" or (op == "mean" and dt == "I64")) else None
        want = _restated(a, stencil, op, dt, bname, pname, T, weights, 0, out_dtype)
        got = ora.map(a, stencil, red, _boundary(st, bname, dt), _padding(st, pname), code=code)
        assert got.dtype == want.dtype and got.shape == want.shape, (bname, pname, got.dtype, want.dtype)
        assert got.tobytes(order="F") == want.tobytes(order="F"), (bname, pname)


SWITCH_CASES = [("Moore1", "life", "U8"), ("VonNeumann1_3d", "diffusion", "F32"), ("Window1", "mean", "F64"),
                ("Circle2", "sum", "F32"), ("Annulus2", "maximum", "F32")]


@pytest.mark.parametrize("name,op,dt", SWITCH_CASES, ids=["-".join(c) for c in SWITCH_CASES])
def test_oracle_switching_matches_restatement(st, orc, abi, name, op, dt):
    """Three steps of A = mapstencil!(f, A) on a SwitchingStencilArray (src/gatherstencil.jl:77-83): each
    step refreshes the source's ring (Halo) and writes the other parent's interior."""
    ora = OracleBackend(st, orc, abi)
    for bname, pname in BCPADS:
        if pname == "halo_in":
            continue      # a Halo{:in} switching pair shrinks nothing further; covered by halo_out
        rng = np.random.default_rng(zlib.crc32(repr(("switch", name, op, dt, bname, pname)).encode()))
        a, stencil, red, T, weights, code = _case_setup(st, abi, name, op, dt, rng)
        want = _restated(a, stencil, op, dt, bname, pname, T, weights, 3, None)
        got = ora.switch_map(a, stencil, red, _boundary(st, bname, dt), _padding(st, pname), steps=3, code=code)
        assert got.tobytes(order="F") == want.tobytes(order="F"), (bname, pname)


# ------------------------------------------------------------------ scatterstencil!
def restated_scatter(value, combine, dest, src, offsets, bname, T, c=None, weights=None):
    """scatterstencil!(f, op, dest, source) run as the reference's pass schedule on one thread
    (src/scatterstencil.jl:48-112): passes over columns j = pass, pass + (2R+1), ...; rows in order;
    each source cell sends f(hood)[k] to (i + o0, j + o1) with Wrap mod1, Reflect 2 - i / 2n - i,
    Remove / Use skipping targets outside."""
    ny, nx = src.shape
    R = max(max(abs(x) for x in o) for o in offsets)
    stride = 2 * R + 1
    out = dest.copy(order="F")
    for pas in range(stride):
        for j in range(pas, nx, stride):
            for i in range(ny):
                centre = T(src[i, j])
                for k, o in enumerate(offsets):
                    val = T(c) if value == "const" else (centre if value == "center" else T(centre * T(weights[k])))
                    ti, tj = i + o[0], j + o[1]
                    if bname == "wrap":
                        ti, tj = ti % ny, tj % nx
                    elif bname == "reflect":
                        ti = -ti if ti < 0 else (2 * ny - 2 - ti if ti >= ny else ti)
                        tj = -tj if tj < 0 else (2 * nx - 2 - tj if tj >= nx else tj)
                    elif not (0 <= ti < ny and 0 <= tj < nx):
                        continue
                    cur = T(out[ti, tj])
                    if combine == "add":
                        out[ti, tj] = T(cur + val)
                    elif combine == "max":
                        out[ti, tj] = val if val > cur else cur
                    else:
                        out[ti, tj] = val if val < cur else cur
    return out


SCATTER_STENCILS = ["Moore1", "Moore2", "VonNeumann1", "Positional"]


@pytest.mark.parametrize("dt", ["F64", "F32"])
@pytest.mark.parametrize("sname", SCATTER_STENCILS)
def test_oracle_scatter_matches_restatement(st, orc, abi, sname, dt):
    import builtins
    import operator
    npdt = np.float64 if dt == "F64" else np.float32
    T = float if dt == "F64" else np.float32
    combines = {"add": operator.add, "max": builtins.max, "min": builtins.min}
    for value in ("const", "center", "weighted"):
        for cname, cop in combines.items():
            for bname, pname in [(b, p) for b in ("remove", "wrap", "reflect", "use") for p in ("cond", "halo")
                                 if not (b == "use" and p == "cond")]:
                rng = np.random.default_rng(zlib.crc32(repr(("scatter", sname, dt, value, cname, bname, pname)).encode()))
                stencil = {"Moore1": st.Moore(1), "Moore2": st.Moore(2), "VonNeumann1": st.VonNeumann(1),
                           "Positional": st.Positional((-1, 0), (1, 1), (0, -1), (1, -1))}[sname]
                shape = (7, 8) if sname != "Moore2" else (9, 11)
                src = np.asfortranarray((rng.random(shape) * 2 - 1).astype(npdt))
                dest0 = np.asfortranarray((rng.random(shape) * 2 - 1).astype(npdt))
                weights = None
                if value == "weighted":
                    weights = rng.standard_normal(len(stencil))
                    if dt == "F32":
                        weights = weights.astype(np.float32)
                    stencil = st.Kernel(stencil, weights, weight_dtype="f32" if dt == "F32" else "f64")
                f = {"const": st.ScatterConst(0.3), "center": st.scatter_center, "weighted": st.scatter_weighted}[value]
                bnd = _boundary(st, bname, dt)
                R = stencil.radius
                parent = src
                pad = st.Conditional()
                if pname == "halo":
                    pad = st.Halo("out")
                    parent = np.zeros((shape[0] + 2 * R, shape[1] + 2 * R), dtype=npdt, order="F")
                    parent[R:-R, R:-R] = src
                got = orc.scatter(f, cop, dest0.copy(order="F"), np.asfortranarray(parent), getattr(abi, dt), stencil,
                                  bnd, pad)
                offs = (stencil.stencil if hasattr(stencil, "stencil") else stencil).offsets()
                want = restated_scatter(value, cname, dest0, src, offs, bname, T, c=0.3,
                                        weights=None if weights is None else [float(w) for w in weights])
                assert got.tobytes(order="F") == want.tobytes(order="F"), (value, cname, bname, pname)


# ------------------------------------------------------------------ maps over several arrays
def restated_terms(terms, args, T):
    """dest[I] = t_1 + t_2 + ... (left to right), t_m = [alpha *] g_m with g_m the argument's centre,
    neighbour sum / mean (fold from the first value), kernelproduct (from zero) or plain value at I; each
    StencilArray argument's ring is refreshed first, as gatherstencil! does for every argument
    (src/gatherstencil.jl:89-113)."""
    prepared = []
    shape = None
    for (kind, alpha), arg in zip(terms, args):
        if kind == "value":
            prepared.append((kind, alpha, arg, None))
            shape = shape or arg.shape
            continue
        parent, stencil, bname, padval, halo, weights = arg
        R = stencil.radius
        sh = tuple(n - 2 * R for n in parent.shape) if halo else parent.shape
        if halo and bname != "use":
            _update_ring(parent, sh, R, bname, padval)
        shape = shape or sh
        prepared.append((kind, alpha, arg, (sh, R, stencil.offsets())))
    out = np.empty(shape, dtype=np.float64 if T is float else np.float32, order="F")
    for I in np.ndindex(*shape):
        acc = None
        for kind, alpha, arg, geo in prepared:
            if kind == "value":
                g = T(arg[I])
            else:
                parent, _, bname, padval, halo, weights = arg
                sh, R, offs = geo
                if kind == "center":
                    g = T(parent[tuple(i + R for i in I)] if halo else parent[I])
                else:
                    vals = [T(v) for v in _hood(parent, sh, R, offs, bname, padval, halo, I)]
                    if kind == "kernelproduct":
                        g = T(0)
                        for v, w in zip(vals, weights):
                            g = T(g + T(v * T(w)))
                    else:
                        g = vals[0]
                        for v in vals[1:]:
                            g = T(g + v)
                        if kind == "mean":
                            g = T(g / T(len(vals)))
            if alpha is not None:
                g = T(T(alpha) * g)
            acc = g if acc is None else T(acc + g)
        out[I] = acc
    return out


TERM_CASES = [
    ("center+0.1sum", [("center", None), ("sum", 0.1)], ["Moore1", "Moore1"]),
    ("mean+kdot", [("mean", None), ("kernelproduct", None)], ["Window2", "Cross1"]),
    ("0.5center+sum+value", [("center", 0.5), ("sum", None), ("value", None)], ["Window1", "VonNeumann2", None]),
    ("2mean-0.25mean", [("mean", 2.0), ("mean", -0.25)], ["Circle2", "Positional"]),
]


@pytest.mark.parametrize("dt", ["F64", "F32"])
@pytest.mark.parametrize("cname,terms,snames", TERM_CASES, ids=[c[0] for c in TERM_CASES])
def test_oracle_terms_match_restatement(st, orc, abi, cname, terms, snames, dt):
    npdt = np.float64 if dt == "F64" else np.float32
    T = float if dt == "F64" else np.float32
    stencils = _stencils(st)
    red = {"center": st.center, "sum": st.sum, "mean": st.mean, "kernelproduct": st.kernelproduct, "value": st.value}
    f = st.Terms(*[red[k] if a is None else st.scaled(a, red[k]) for k, a in terms])
    for combo in [("remove", "cond"), ("wrap", "cond"), ("reflect", "halo_out"), ("use", "halo_out"),
                  ("wrap", "halo_out")]:
        rng = np.random.default_rng(zlib.crc32(repr(("terms", cname, dt, combo)).encode()))
        shape = (9, 8)
        items, rargs = [], []
        for (kind, _), sname in zip(terms, snames):
            a = np.asfortranarray((rng.random(shape) * 2 - 1).astype(npdt))
            if sname is None:
                items.append(a)
                rargs.append(a.copy(order="F"))
                continue
            stencil = stencils[sname][0]
            weights = None
            if kind == "kernelproduct":
                weights = [float(x) for x in rng.standard_normal(len(stencil))]
                if dt == "F32":
                    weights = [float(np.float32(x)) for x in weights]
                stencil = st.Kernel(stencil, np.array(weights, dtype=npdt), weight_dtype="f32" if dt == "F32" else "f64")
            bname, pname = combo
            R = stencil.radius
            parent = a
            if pname == "halo_out":
                parent = np.zeros((shape[0] + 2 * R, shape[1] + 2 * R), dtype=npdt, order="F")
                parent[R:-R, R:-R] = a
            items.append((parent.copy(order="F"), stencil, _boundary(st, bname, dt), _padding(st, pname)))
            base = stencil.stencil if hasattr(stencil, "stencil") else stencil
            rargs.append((parent.copy(order="F"), base, bname, T(_padval(dt)), pname != "cond", weights))
        got = orc.map_terms(f, items, getattr(abi, dt))
        want = restated_terms(terms, rargs, T)
        assert got.tobytes(order="F") == want.tobytes(order="F"), combo


# ------------------------------------------------------------------ the oracle's specialised Life path
@pytest.mark.parametrize("bname,pname", [("wrap", "halo_out"), ("remove", "halo_out"), ("reflect", "halo_in"),
                                         ("use", "halo_in"), ("wrap", "halo_in")])
def test_oracle_life_fast_path_equals_generic(st, orc, abi, bname, pname):
    """Moore(1) Life on UInt8 / Bool Halo parents runs a specialised loop in the oracle (the CPU baseline);
    it equals the generic gather bit for bit for several rules, sizes and step counts."""
    ora = OracleBackend(st, orc, abi)
    rules = [st.life, st.LifeRule((3, 6), (2, 3)), st.LifeRule((1,), (0, 8)), st.LifeRule((), (1, 2, 3, 4))]
    for shape, steps in (((37, 29), 5), ((8, 70), 3), ((64, 64), 12)):
        for rule in rules:
            for dt in ("U8", "BOOL"):
                rng = np.random.default_rng(zlib.crc32(repr((bname, pname, shape, rule.name, dt)).encode()))
                a = np.asfortranarray((rng.random(shape) < 0.35).astype(np.uint8))
                bnd = st.Remove(0) if bname == "remove" else _boundary(st, bname, "U8")
                code = getattr(abi, dt)
                try:
                    orc.set_fast_paths(False)
                    want = ora.switch_map(a, st.Moore(1), rule, bnd, _padding(st, pname), steps=steps, code=code)
                    want1 = ora.map(a, st.Moore(1), rule, bnd, _padding(st, pname), code=code)
                finally:
                    orc.set_fast_paths(True)
                got = ora.switch_map(a, st.Moore(1), rule, bnd, _padding(st, pname), steps=steps, code=code)
                got1 = ora.map(a, st.Moore(1), rule, bnd, _padding(st, pname), code=code)
                assert got.tobytes(order="F") == want.tobytes(order="F"), (shape, rule.name, dt)
                assert got1.tobytes(order="F") == want1.tobytes(order="F"), (shape, rule.name, dt)


@pytest.mark.parametrize("name", ["Window1", "Circle2", "Annulus2", "Rectangle", "Positional", "Moore1_3d",
                                  "Cross1_3d", "Window2_1d"])
@pytest.mark.parametrize("op,dt", [("mean", "F64"), ("sum", "F64"), ("mean", "F32"), ("sum", "F32")])
def test_oracle_float_fast_path_equals_generic(st, orc, abi, name, op, dt):
    """Float sum / mean fold the interior (Conditional) or every cell (Halo) from constant offsets in the
    oracle; that equals the generic gather bit for bit, including grids too small to have an interior."""
    ora = OracleBackend(st, orc, abi)
    stencil, nd = _stencils(st)[name]
    sizes = {1: [(11,), (3,)], 2: [(9, 8), (3, 40), (40, 3)], 3: [(6, 5, 5), (3, 9, 4)]}[nd]
    red = st.mean if op == "mean" else st.sum
    npdt = np.float64 if dt == "F64" else np.float32
    for shape in sizes:
        if min(shape) <= stencil.radius:
            continue
        for bname, pname in BCPADS:
            if pname == "halo_in" and min(shape) <= 3 * stencil.radius:
                continue
            rng = np.random.default_rng(zlib.crc32(repr(("ffast", name, op, dt, shape, bname, pname)).encode()))
            a = np.asfortranarray((rng.random(shape) * 2 - 1).astype(npdt))
            bnd, pad = _boundary(st, bname, dt), _padding(st, pname)
            try:
                orc.set_fast_paths(False)
                want = ora.map(a, stencil, red, bnd, pad, code=getattr(abi, dt))
            finally:
                orc.set_fast_paths(True)
            got = ora.map(a, stencil, red, bnd, pad, code=getattr(abi, dt))
            assert got.tobytes(order="F") == want.tobytes(order="F"), (shape, bname, pname)
