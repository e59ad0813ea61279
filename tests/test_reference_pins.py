"""Pins of this repository to the MarineHydro.jl source text (CPU only).

* Every `file.jl:a-b` citation in the docs, the C-ABI header, the CUDA sources, the
  oracle, the package and the tests names lines that exist in the cited reference
  file.  The line counts come from tests/golden/reference_kats.json, written by
  tests/golden/extract_reference_kats.py from a MarineHydro.jl checkout, so the check
  runs without the reference tree; with MH_REFERENCE_ROOT set to a checkout the index
  itself is checked against it.
* Every constant of the Liang-Wu-Noblesse fits (GF_FuncA-D, GF_dFuncA-C), of the Struve
  fits (StruveH0/H1) and Euler's constant of GF_Func_L0, as extracted from wu.jl, appears
  bit for bit in the oracle, in the FP64 kernels (primal and dual-number adjoint), in the
  FP32 surrogate base and in the generator of the Chebyshev tables -- each polynomial as
  one contiguous run of literals in the order its Horner form uses them (the FP64 kernel's
  fixed-point tables list them lowest degree first).  A mistyped or
  reordered coefficient in any copy fails here, below the 2e-2 level at which the
  reference's own tests compare Wu with the exact Green function.
"""
from __future__ import annotations

import json
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KATS = os.path.join(REPO, "tests", "golden", "reference_kats.json")
CSRC = os.path.join(REPO, "marinehydro.jl_gb300", "csrc")

# files of this build that describe the state of the build rather than cite the reference
_SKIP_DOCS = {"VERDICT.md", "ADVICE.md", "SURVEY.md", "BASELINE.md"}
_CITE = re.compile(r"((?:[\w.-]+/)*[\w-]+\.(?:jl|ipynb|toml)):(\d+)(?:-(\d+))?((?:,\s*:?\d+(?:-\d+)?)*)")
_BARE = re.compile(r"(?<![\w.])[(, ]:(\d+)(?:-(\d+))?")


def _kats():
    with open(KATS) as f:
        return json.load(f)


def _resolve(name, counts):
    """Reference path of a cited file name: exact relative path, else the unique file with that
    suffix, else the one under src/ (src/ and test/ both hold a matrix_assembly.jl)."""
    name = name.lstrip("./")
    if name in counts:
        return name
    cands = [p for p in counts if p.endswith("/" + name)]
    if len(cands) == 1:
        return cands[0]
    src = [p for p in cands if p.startswith("src/")]
    return src[0] if len(src) == 1 else None


def _citing_files():
    out = []
    for root, dirs, files in os.walk(REPO):
        rel = os.path.relpath(root, REPO)
        dirs[:] = [d for d in dirs if not d.startswith((".", "_")) and d not in ("gpurun_out", "baseline")]
        if rel.startswith(("_work", "gpurun_out")):
            continue
        for f in files:
            if f.endswith((".md", ".h", ".cu", ".cuh", ".py", ".c")) and f not in _SKIP_DOCS:
                out.append(os.path.join(root, f))
    return sorted(out)


def citation_errors(counts):
    errors, seen = [], 0
    for path in _citing_files():
        last = None
        with open(path, errors="replace") as fh:
            for ln, line in enumerate(fh, 1):
                events = [(m.start(), 0, m) for m in _CITE.finditer(line)]
                events += [(m.start(), 1, m) for m in _BARE.finditer(line)]
                for _, kind, m in sorted(events, key=lambda e: e[0]):
                    where = f"{os.path.relpath(path, REPO)}:{ln}: {m.group(0).strip()}"
                    if kind == 0:
                        ref = _resolve(m.group(1), counts)
                        if ref is None:
                            errors.append(f"{where}: no such reference file")
                            last = None
                            continue
                        last = ref
                        ranges = [(int(m.group(2)), int(m.group(3) or m.group(2)))]
                        ranges += [(int(a), int(b or a)) for a, b in re.findall(r":?(\d+)(?:-(\d+))?", m.group(4) or "")]
                    elif last is not None:
                        ref = last
                        ranges = [(int(m.group(1)), int(m.group(2) or m.group(1)))]
                    else:
                        continue
                    for a, b in ranges:
                        seen += 1
                        if not (1 <= a <= b <= counts[ref]):
                            errors.append(f"{where}: {ref} has {counts[ref]} lines")
    return errors, seen


def test_citations_name_existing_reference_lines():
    counts = _kats()["reference_files"]
    errors, seen = citation_errors(counts)
    assert seen > 300, seen  # the scan found the citations
    assert not errors, "\n".join(errors)


def test_citation_check_catches_a_bad_range():
    counts = {"src/bodies.jl": 226, "src/matrix_assembly.jl": 450, "test/matrix_assembly.jl": 126}
    assert _resolve("bodies.jl", counts) == "src/bodies.jl"
    assert _resolve("matrix_assembly.jl", counts) == "src/matrix_assembly.jl"
    assert _resolve("test/matrix_assembly.jl", counts) == "test/matrix_assembly.jl"
    m = _CITE.search("combine_floatingbodies (bodies" + ".jl:165-225, 446-469)")  # split: not a citation
    assert m and m.group(4).strip(", ") == "446-469"


def test_reference_index_matches_checkout():
    root = os.environ.get("MH_REFERENCE_ROOT")
    if not root or not os.path.isdir(root):
        pytest.skip("MH_REFERENCE_ROOT not set to a MarineHydro.jl checkout")
    counts = _kats()["reference_files"]
    for rel, n in counts.items():
        with open(os.path.join(root, rel), errors="replace") as fh:
            assert sum(1 for _ in fh) == n, rel


# ---------------------------------------------------------------------------
# Wu fit constants
# ---------------------------------------------------------------------------
_LIT = re.compile(r"(?<![\w.])-?\d+\.\d*(?:[eE][-+]?\d+)?f?")


def _literals(path):
    with open(path) as fh:
        text = fh.read()
    text = re.sub(r"//[^\n]*|/\*.*?\*/|#[^\n]*", " ", text, flags=re.S) if not path.endswith(".py") else \
        re.sub(r"#[^\n]*", " ", text)
    return [float(t.rstrip("f")) for t in _LIT.findall(text)]


def _contains_run(seq, run):
    n = len(run)
    return any(seq[i:i + n] == run for i in range(len(seq) - n + 1))


def _horner_run(coeffs):
    """Literal order of c0 + (c1 + (... (c_{n-1} + c_n t) t ...) t) written innermost-first as
    v = (c_{n-1} + c_n t) t; v = (c_{n-2} + v) t; ...; c0 + v."""
    return [coeffs[-2], coeffs[-1]] + coeffs[-3::-1]


def _wu():
    return {k: [(n, float(v)) for n, v in vals] for k, vals in _kats()["wu_constants"].items()}


def _struve_runs(vals):
    d = dict(vals)
    p = sorted(n for n in d if n.startswith("P"))
    return [[d[n] for n in p], [d[f"a{i}"] for i in range(4)], [d[f"b{i}"] for i in (1, 2, 3)]]


POLYS = ("GF_FuncA", "GF_FuncB", "GF_FuncC", "GF_FuncD", "GF_dFuncA", "GF_dFuncB", "GF_dFuncC")


@pytest.mark.parametrize("path", ["oracle/mh_oracle.c", "marinehydro.jl_gb300/csrc/mh_greens.cuh",
                                  "marinehydro.jl_gb300/csrc/mh_adjoint.cu"])
def test_wu_fit_constants_match_wu_jl(path):
    wu = _wu()
    lits = _literals(os.path.join(REPO, path))
    for name in POLYS:
        coeffs = [v for _, v in wu[name]]
        # the reference's nested order, or lowest degree first (the fixed-point tables)
        assert _contains_run(lits, _horner_run(coeffs)) or _contains_run(lits, coeffs), (path, name)
    for name in ("StruveH0", "StruveH1"):
        for run in _struve_runs(wu[name]):
            assert _contains_run(lits, run), (path, name, run)
    assert wu["GF_Func_L0"][0][1] in lits, (path, "gama")


def test_fp32_base_and_table_generator_use_the_same_constants():
    wu = _wu()
    lits = _literals(os.path.join(CSRC, "mh_wu_f32.cuh"))
    for name in ("StruveH0", "StruveH1"):
        for run in _struve_runs(wu[name]):
            assert _contains_run(lits, run), ("mh_wu_f32.cuh", name, run)
    assert wu["GF_Func_L0"][0][1] in lits
    gen = _literals(os.path.join(CSRC, "gen_special_tables.py"))
    for name in POLYS:
        coeffs = [v for _, v in wu[name]]  # the generator lists them lowest degree first
        assert _contains_run(gen, coeffs), ("gen_special_tables.py", name)


def test_wu_constant_check_catches_a_changed_digit():
    wu = _wu()
    coeffs = [v for _, v in wu["GF_FuncA"]]
    lits = _literals(os.path.join(REPO, "oracle", "mh_oracle.c"))
    bad = list(coeffs)
    bad[4] = bad[4] + 0.01  # 8418.94 -> 8418.95
    assert _contains_run(lits, _horner_run(coeffs))
    assert not _contains_run(lits, _horner_run(bad))
    swapped = list(coeffs)
    swapped[2], swapped[3] = swapped[3], swapped[2]
    assert not _contains_run(lits, _horner_run(swapped))
