"""Generate the golden fixtures in this folder from the reference sources.

Run here (where the reference checkout exists) as

    python tests/golden/make_golden.py [/path/to/isosurface]

It reads, as text only:

* ``src/marching_cubes_tables.rs`` -> ``mc_tables.json`` (CORNERS, REMAP_CUBE,
  EDGE_CONNECTION, EDGE_CROSSING_MASK, TRIANGLE_CONNECTION and EDGE_LOOPS
  exactly as the reference declares them, marching_cubes_tables.rs:16-594).
* the inline ``#[cfg(test)]`` known-answer tests of the implicit primitives
  (sphere.rs:65-109, rectangular_prism.rs:82-130, cylinder.rs:87-140,
  torus.rs:110-171, csg.rs:108-167) -> ``kats.json``: the ``sample_scalar``,
  ``sample_normal(..).normalised()`` and ``sample_vector`` (the Directed
  metric of ExtendedMarchingCubes) assertions.  Expected values written as
  expressions (``Vec2::from_scalar(1.0 - (4.0f32 - 1.0f32).sqrt())
  .extend(-3.0)``) are evaluated here in float32, as Rust evaluates them.

The fixtures are committed so that nothing at test time reads the reference.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _ints(text):
    out = []
    for tok in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", text):
        out.append(int(tok, 16) if "x" in tok.lower() else int(tok))
    return out


def parse_tables(ref):
    src = open(os.path.join(ref, "src", "marching_cubes_tables.rs")).read()
    tables = {}
    for name in ["CORNERS", "REMAP_CUBE", "EDGE_CONNECTION", "EDGE_CROSSING_MASK",
                 "TRIANGLE_CONNECTION", "EDGE_LOOPS"]:
        m = re.search(r"pub const %s: ([^=]+)= \[(.*?)\];" % name, src, re.S)
        body = m.group(2)
        # strip the type's own array sizes from the count: the body only holds values
        vals = _ints(body)
        line = src[: m.start()].count("\n") + 1
        tables[name] = {"values": vals, "line": line}
    t = tables
    out = {
        "CORNERS": [t["CORNERS"]["values"][3 * i: 3 * i + 3] for i in range(8)],
        "REMAP_CUBE": t["REMAP_CUBE"]["values"],
        "EDGE_CONNECTION": [t["EDGE_CONNECTION"]["values"][2 * i: 2 * i + 2] for i in range(12)],
        "EDGE_CROSSING_MASK": t["EDGE_CROSSING_MASK"]["values"],
        "TRIANGLE_CONNECTION": [t["TRIANGLE_CONNECTION"]["values"][16 * i: 16 * i + 16]
                                for i in range(256)],
        "EDGE_LOOPS": [t["EDGE_LOOPS"]["values"][17 * i: 17 * i + 17] for i in range(256)],
        "source_lines": {k: v["line"] for k, v in t.items()},
    }
    assert len(out["EDGE_CROSSING_MASK"]) == 256
    assert len(t["TRIANGLE_CONNECTION"]["values"]) == 256 * 16
    assert len(t["EDGE_LOOPS"]["values"]) == 256 * 17
    return out


_NUM = r"-?\d+(?:\.\d*)?(?:f32)?"


def _num(s):
    return float(s.replace("f32", ""))


def _vec(expr):
    expr = expr.strip()
    if expr == "Vec3::zero()":
        return [0.0, 0.0, 0.0]
    m = re.fullmatch(r"Vec3::from_scalar\((%s)\)" % _NUM, expr)
    if m:
        v = _num(m.group(1))
        return [v, v, v]
    m = re.fullmatch(r"Vec3::new\((%s),\s*(%s),\s*(%s)\)" % (_NUM, _NUM, _NUM), expr)
    if m:
        return [_num(m.group(i)) for i in (1, 2, 3)]
    return None


F32_MAX = 3.4028234663852886e38  # std::f32::MAX, exactly representable


def _f32_eval(expr):
    """A scalar Rust f32 expression (literals, MAX, + - * /, parentheses,
    ``(..).sqrt()``) evaluated in float32, operation by operation."""
    import numpy as np
    e = re.sub(r"(\d+(?:\.\d*)?)(?:f32)?", r"F(\1)", expr)
    e = e.replace("MAX", "F(%r)" % F32_MAX)
    # innermost `( ... ).sqrt()` first
    while ".sqrt()" in e:
        e2 = re.sub(r"\(([^()]*(?:\([^()]*\)[^()]*)*)\)\.sqrt\(\)", r"np.sqrt(\1)", e, count=1)
        assert e2 != e, expr
        e = e2
    v = eval(e, {"F": np.float32, "np": np})
    assert isinstance(v, np.float32), (expr, type(v))
    return float(v)


def _split_args(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
            continue
        depth += (ch == "(") - (ch == ")")
        cur += ch
    out.append(cur)
    return [a.strip() for a in out if a.strip()]


def _vec_expr(expr):
    """Expected Directed values: Vec3::zero / from_scalar / new, or
    Vec2::from_scalar(x).extend(z), with f32 expressions as components."""
    expr = expr.strip().rstrip(",").strip()
    if expr == "Vec3::zero()":
        return [0.0, 0.0, 0.0]
    m = re.fullmatch(r"Vec3::from_scalar\((.*)\)", expr)
    if m:
        v = _f32_eval(m.group(1))
        return [v, v, v]
    m = re.fullmatch(r"Vec3::new\((.*)\)", expr)
    if m:
        args = _split_args(m.group(1))
        assert len(args) == 3, expr
        return [_f32_eval(a) for a in args]
    m = re.fullmatch(r"Vec2::from_scalar\((.*)\)\.extend\((.*)\)", expr)
    if m:
        v = _f32_eval(m.group(1))
        return [v, v, _f32_eval(m.group(2))]
    raise ValueError("unparsed vector: " + expr)


def _ctor(expr, env):
    expr = expr.strip()
    m = re.fullmatch(r"Sphere::new\((%s)\)" % _NUM, expr)
    if m:
        return {"type": "sphere", "radius": _num(m.group(1))}
    m = re.fullmatch(r"RectangularPrism::new\((.*)\)", expr)
    if m:
        return {"type": "box", "half_extent": _vec(m.group(1))}
    m = re.fullmatch(r"Cylinder::new\((%s),\s*(%s)\)" % (_NUM, _NUM), expr)
    if m:
        return {"type": "cylinder", "radius": _num(m.group(1)), "half_length": _num(m.group(2))}
    m = re.fullmatch(r"Torus::new\((%s),\s*(%s)\)" % (_NUM, _NUM), expr)
    if m:
        return {"type": "torus", "radius": _num(m.group(1)), "tube_radius": _num(m.group(2))}
    m = re.fullmatch(r"(Union|Intersection|Difference)::new\((\w+)\.clone\(\),\s*(\w+)\.clone\(\)\)", expr)
    if m:
        return {"type": m.group(1).lower(), "a": env[m.group(2)], "b": env[m.group(3)]}
    raise ValueError("unparsed constructor: " + expr)


def parse_kats(ref):
    kats = []
    for fname in ["sphere.rs", "rectangular_prism.rs", "cylinder.rs", "torus.rs", "csg.rs"]:
        path = os.path.join(ref, "src", "implicit", fname)
        text = open(path).read()
        start = text.index("#[cfg(test)]")
        body = text[start:]
        base_line = text[:start].count("\n") + 1
        env = {}
        # statements end with ';' — walk them in order, tracking line numbers
        pos = 0
        for stmt_m in re.finditer(r"[^;{}]*;", body):
            stmt = stmt_m.group(0)
            line = base_line + body[: stmt_m.start() + len(stmt) - len(stmt.lstrip())].count("\n")
            flat = " ".join(stmt.split())
            m = re.match(r"let (\w+) = (.*);$", flat)
            if m:
                env[m.group(1)] = _ctor(m.group(2), env)
                continue
            m = re.match(r"assert_eq!\(\s*(\w+)\s*\.sample_scalar\((.*)\)\s*\.0,\s*(%s)\s*\);$" % _NUM, flat)
            if m:
                kats.append({"file": "src/implicit/" + fname, "line": line,
                             "source": env[m.group(1)], "kind": "scalar",
                             "point": _vec(m.group(2)), "expected": _num(m.group(3))})
                continue
            m = re.match(r"assert_eq!\(\s*(\w+)\s*\.sample_vector\((.*?)\)\s*\.0,\s*(.*?)\s*\);$", flat)
            if m:
                kats.append({"file": "src/implicit/" + fname, "line": line,
                             "source": env[m.group(1)], "kind": "vector",
                             "point": _vec(m.group(2)), "expected": _vec_expr(m.group(3))})
                continue
            m = re.match(r"assert_eq!\(\s*(\w+)\s*\.sample_normal\((.*?)\)\s*\.normalised\(\)\s*\.unwrap\(\),\s*(.*)\s*\);$", flat)
            if m:
                kats.append({"file": "src/implicit/" + fname, "line": line,
                             "source": env[m.group(1)], "kind": "normal",
                             "point": _vec(m.group(2)), "expected": _vec(m.group(3))})
                continue
    return kats


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ISO_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout>  (or set ISO_REFERENCE_DIR)")
    tables = parse_tables(ref)
    with open(os.path.join(HERE, "mc_tables.json"), "w") as f:
        json.dump(tables, f, indent=0)
    kats = parse_kats(ref)
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump(kats, f, indent=1)
    print("tables ok; %d KATs" % len(kats))


if __name__ == "__main__":
    main()
