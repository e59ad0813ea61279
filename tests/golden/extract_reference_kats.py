"""Extract the known-answer values of MarineHydro.jl's own tests into reference_kats.json.

The reference cannot run here (no Julia), so its test files are read as text and
their hard-coded expected values are transcribed mechanically:

  test/rankine_vectorized.jl      Birk (2021) tables: square, twisted quad, triangle
                                  (area, frame T, centroid, local corners, phi, v, Hessian)
  test/greens_function.jl         Capytaine Delhommeau point values, the canonical
                                  element pair, Wu-vs-Delhommeau tolerance
  test/consistency_with_analytical_solutions.jl
                                  Hulme (1982) heaving-hemisphere added mass / damping
  src/green_functions/wu.jl       every numeric constant of the Liang-Wu-Noblesse fits
                                  GF_FuncA-D, GF_dFuncA-C, the Struve fits StruveH0/H1
                                  and Euler's constant of GF_Func_L0, as written there
  every .jl / .toml / .ipynb file the line count (so that file:line citations in this
                                  repository can be checked without the reference tree)

Usage:  python tests/golden/extract_reference_kats.py REFERENCE_ROOT
where REFERENCE_ROOT is the root of a MarineHydro.jl checkout.  Writes
tests/golden/reference_kats.json.
"""
from __future__ import annotations

import ast
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _julia_to_py(text: str) -> str:
    """Convert the literal subset used in the test tables to Python syntax."""
    t = text.replace("SVector", "").replace("@SMatrix", "")
    t = re.sub(r"#[^\n]*", "", t)

    def mat(m):
        body = m.group(1)
        if ";" not in body:
            return "[" + body + "]"
        rows = [r.strip() for r in body.split(";") if r.strip()]
        return "[" + ", ".join("[" + ", ".join(r.split()) + "]" for r in rows) + "]"

    # innermost brackets first
    prev = None
    while prev != t:
        prev = t
        t = re.sub(r"\[([^\[\]]*)\]", lambda m: mat(m).replace("[", "⟦").replace("]", "⟧"), t)
    t = t.replace("⟦", "[").replace("⟧", "]")
    t = re.sub(r"(\d)im\b", r"\1j", t)
    return t


def _block(src: str, start_pat: str) -> str:
    """Text of a parenthesised Julia expression starting at the first match of start_pat."""
    m = re.search(start_pat, src)
    if not m:
        raise ValueError(f"pattern not found: {start_pat}")
    i = src.index("(", m.end() - 1)
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "(":
            depth += 1
        elif src[j] == ")":
            depth -= 1
            if depth == 0:
                return src[i:j + 1]
    raise ValueError("unbalanced")


def _eval(text: str):
    return ast.literal_eval(_julia_to_py(text))


def _testset(src: str, title: str) -> str:
    i = src.index(f'@testset "{title}')
    j = src.find("@testset", i + 10)
    return src[i:j if j > 0 else len(src)]


def _after(src: str, pat: str, conv=float):
    m = re.search(pat, src)
    if not m:
        raise ValueError(f"pattern not found: {pat}")
    return conv(m.group(1))


def extract(root: str) -> dict:
    out = {"source": "MarineHydro.jl test files (read as text)", "birk": {}}
    rv = open(os.path.join(root, "test", "rankine_vectorized.jl")).read()
    for key, title in (("square", "Square panel"), ("twisted", "Twisted quadrilateral"), ("triangle", "Triangle panel")):
        blk = _testset(rv, title)
        case = {"corners": _eval(_block(blk, r"corners\s*=\s*\(")),
                "area": _after(blk, r"@test A ≈ ([-\d.eE]+)")}
        m = re.search(r"T_exp\s*=\s*(\[[^\]]*\])", blk)
        case["T"] = _eval(m.group(1)) if m else [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
        m = re.search(r"@test qgc ≈ (\[[^\]]*\])", blk)
        case["qgc"] = _eval(m.group(1))
        lcs = re.findall(r"@test local_corners\[(\d)\] ≈ SVector\(([^)]*)\)", blk)
        case["local_corners"] = [[float(x) for x in c.split(",")] for _, c in sorted(lcs)]
        case["tol_geometry"] = 1e-6
        cases = _eval(_block(blk, r"cases\s*=\s*\("))
        rows = []
        for c in cases:
            row = {"point": list(c[0]), "phi": c[1], "v": list(c[2])}
            if len(c) > 3:
                if isinstance(c[3][0], list):
                    row["H"] = c[3]
                else:
                    row["point_local"] = list(c[3])
            rows.append(row)
        case["cases"] = rows
        m = re.search(r"hessian_cases\s*=\s*\(", blk)
        if m:
            case["hessian_cases"] = [{"point": list(p), "H": H} for p, H in _eval(_block(blk, r"hessian_cases\s*=\s*\("))]
        case["tol_phi"] = 1e-6
        case["tol_v"] = 1e-5 if key == "twisted" else 1e-6
        case["tol_H"] = 1e-6
        case["tol_laplace"] = 1e-8
        out["birk"][key] = case
    gf = open(os.path.join(root, "test", "greens_function.jl")).read()
    ref = _eval(re.search(r"capy_ref = (\[[^\]]*\])", gf).group(1))
    out["delhommeau_dimless"] = {"r": 1.0, "z": -1.0, "G": [ref[0], ref[1]], "dG_dr": [ref[2], ref[3]], "atol": 1e-4}
    g = re.search(r"capy_g = (-?[\d.]+(?:[eE][-+]?\d+)?)([+-][\d.]+(?:[eE][-+]?\d+)?)im", gf)
    gg = _eval(re.search(r"capy_gradg = (\[[^\]]*\])", gf).group(1))
    out["delhommeau_pair"] = {
        "e1_center": [0.0, 0.0, -1.0], "e2_center": [1.0, 1.0, -2.0], "k": 1.0,
        "G": [float(g.group(1)), float(g.group(2))],
        "grad_wrt_first": [[z.real, z.imag] for z in gg], "atol": 1e-4,
    }
    out["canonical_pair"] = {
        "e1_center": [0.0, 0.0, -1.0],
        "e2": {"center": [1.0, 1.0, -2.0],
               "vertices": [[-0.5 + 1, -0.5 + 1, -2.0], [0.5 + 1, -0.5 + 1, -2.0], [0.5 + 1, 0.5 + 1, -2.0],
                            [-0.5 + 1, 0.5 + 1, -2.0]],
               "normal": [0.0, 0.0, 1.0], "area": 1.0, "radius": 2 ** 0.5 / 2},
        "wu_vs_delhommeau_k": [float(x) for x in re.search(r'"GFWu, k=\$k" for k in \[([^\]]*)\]', gf).group(1).split(",")],
        "wu_vs_delhommeau_atol": 2e-2,
        "rankine_vs_delhommeau_rtol": 1e-4,
    }
    ca = open(os.path.join(root, "test", "consistency_with_analytical_solutions.jl")).read()
    blk = ca[ca.index("using Wu gf  rtol=1e-1"):]
    out["hulme_heave"] = {
        "K": _eval(re.search(r"K_heave = (\[[^\]]*\])", blk).group(1)),
        "A": _eval(re.search(r"A_heave = (\[[^\]]*\])", blk).group(1)),
        "B": _eval(re.search(r"B_heave = (\[[^\]]*\])", blk).group(1)),
        "g_for_omega": 9.8, "rho": 1025.0, "radius": 1.0, "rtol": 0.1,
        "citation": "Hulme 1982, J. Fluid Mech. 121:443-463 (test/consistency_with_analytical_solutions.jl:52-76)",
    }
    return out


WU_FUNCTIONS = ("GF_dFuncC", "GF_dFuncB", "GF_dFuncA", "GF_FuncD", "GF_FuncC", "GF_FuncB", "GF_FuncA",
                "StruveH0", "StruveH1", "GF_Func_L0")


def _julia_function(src: str, name: str) -> str:
    """Body of `@inline function name(...)` up to its matching `end` (keywords counted per line)."""
    m = re.search(r"^[ \t]*(?:@inline[ \t]+)?function[ \t]+" + re.escape(name) + r"\(", src, re.M)
    if not m:
        raise ValueError(f"function {name} not found")
    lines = src[m.start():].split("\n")
    depth, out = 0, []
    for line in lines:
        code = re.sub(r"#.*", "", line)
        depth += len(re.findall(r"\b(?:function|if|for|while|begin|let)\b", code))
        depth -= len(re.findall(r"\bend\b", code))
        out.append(line)
        if depth <= 0:
            return "\n".join(out)
    raise ValueError(f"unterminated function {name}")


def extract_wu_constants(root: str) -> dict:
    """Every `NAME = literal` assignment of the fit functions of wu.jl, in source order,
    with the literal kept as written (the tests parse it to the same double)."""
    src = open(os.path.join(root, "src", "green_functions", "wu.jl")).read()
    lit = re.compile(r"^\s*([A-Za-z]\w*)\s*=\s*([-+]?\d+\.\d*(?:[eE][-+]?\d+)?)\s*$")
    out = {}
    for name in WU_FUNCTIONS:
        body = _julia_function(src, name)
        out[name] = [[m.group(1), m.group(2)] for m in map(lit.match, body.split("\n")) if m]
        if not out[name]:
            raise ValueError(f"no constants found in {name}")
    return out


def reference_line_counts(root: str) -> dict:
    counts = {}
    for d, _, files in os.walk(root):
        if os.path.basename(d).startswith("."):
            continue
        for f in files:
            if f.endswith((".jl", ".toml", ".ipynb")):
                p = os.path.join(d, f)
                with open(p, errors="replace") as fh:
                    counts[os.path.relpath(p, root)] = sum(1 for _ in fh)
    return dict(sorted(counts.items()))


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: extract_reference_kats.py REFERENCE_ROOT")
    root = sys.argv[1]
    data = extract(root)
    data["wu_constants"] = extract_wu_constants(root)
    data["reference_files"] = reference_line_counts(root)
    path = os.path.join(HERE, "reference_kats.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
