"""Green-function types and BEM formulations (formulations.jl:1-37, green_functions/*.jl).

A formulation carries its Green-function tuple; the tuple becomes the bit set the
C-ABI takes (MH_GF_*).  `precision` selects the linear-solve arithmetic of the
GPU path: "fp64" (the reference's arithmetic), "mixed" (FP32 LU factors with
FP64 iterative refinement to FP64 accuracy) or "fp64_tc" (the FP64 LU with its
trailing update on the BF16 tensor cores by Ozaki splitting).
"""
from __future__ import annotations

from . import _lib


class GreensFunction:
    flag = 0
    wavenumber_independent = False

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self))

    def __repr__(self):
        return f"{type(self).__name__}()"


class Rankine(GreensFunction):
    """Birk (2021) vectorized constant-source panel (rankine_vectorized.jl:21)."""
    flag = _lib.GF_RANKINE
    wavenumber_independent = True


class RankineReflected(GreensFunction):
    """Free-surface image of Rankine (rankine_reflected.jl:1)."""
    flag = _lib.GF_RANKINE_REFLECTED
    wavenumber_independent = True


class RankineReflectedNegative(GreensFunction):
    """Minus the free-surface image (rankine_reflected_negative.jl:1)."""
    flag = _lib.GF_RANKINE_REFLECTED_NEGATIVE
    wavenumber_independent = True


class DelhommeauRankine(GreensFunction):
    """Capytaine-style Rankine panel integral (rankine.jl:9)."""
    flag = _lib.GF_DELHOMMEAU_RANKINE
    wavenumber_independent = True


class DelhommeauRankineReflected(GreensFunction):
    """Image of DelhommeauRankine (rankine_reflected.jl:10)."""
    flag = _lib.GF_DELHOMMEAU_RANKINE_REFLECTED
    wavenumber_independent = True


class GFWu(GreensFunction):
    """Liang-Wu-Noblesse infinite-depth wave term (wu.jl:3)."""
    flag = _lib.GF_WU


class ExactGuevelDelhommeau(GreensFunction):
    """Exact Guevel-Delhommeau wave term by adaptive quadrature (exact_Guevel_Delhommeau.jl:3)."""
    flag = _lib.GF_EXACT_DELHOMMEAU


class SurrogateDelhommeau(GreensFunction):
    """Learned approximation of ExactGuevelDelhommeau: the Wu fits plus a BF16 MLP
    correction, exact kernel outside the training box (no counterpart in the
    reference; train with ``train_surrogate`` or install parameters with
    ``set_surrogate`` first)."""
    flag = _lib.GF_SURROGATE


def partition_greens_functions(gfs):
    """partition_greens_functions (abstract_greens_function.jl:8-22)."""
    gfs = tuple(gfs)
    return (tuple(g for g in gfs if g.wavenumber_independent), tuple(g for g in gfs if not g.wavenumber_independent))


def gf_flags(gfs) -> int:
    if isinstance(gfs, GreensFunction):
        gfs = (gfs,)
    flags = 0
    for g in gfs:
        if not isinstance(g, GreensFunction):
            raise ValueError(f"not a Green function: {g!r}")
        if flags & g.flag:
            raise ValueError(f"{g!r} appears twice in the Green-function tuple")
        flags |= g.flag
    if not flags:
        raise ValueError("empty Green-function tuple")
    return flags


def default_greens_functions(gf: str = "Wu"):
    """default_greens_functions (formulations.jl:22-30)."""
    if gf == "Wu":
        wave = GFWu()
    elif gf == "ExactGuevelDelhommeau":
        wave = ExactGuevelDelhommeau()
    elif gf == "Surrogate":
        wave = SurrogateDelhommeau()
    else:
        raise ValueError(f'unknown Green\'s function "{gf}"; use "Wu" or "ExactGuevelDelhommeau"')
    return (Rankine(), RankineReflected(), wave)


class BEMFormulation:
    direct = True

    def __init__(self, greens=None, precision: str = "fp64"):
        if greens is None:
            greens = default_greens_functions("Wu")
        elif isinstance(greens, str):
            greens = default_greens_functions(greens)
        self.greens = tuple(greens) if not isinstance(greens, GreensFunction) else (greens,)
        gf_flags(self.greens)
        if precision not in ("fp64", "mixed", "fp64_tc"):
            raise ValueError('precision must be "fp64", "mixed" or "fp64_tc"')
        self.precision = precision

    @property
    def precision_code(self) -> int:
        return {"fp64": _lib.MH_PREC_FP64, "mixed": _lib.MH_PREC_MIXED, "fp64_tc": _lib.MH_PREC_FP64_TC}[self.precision]

    def __repr__(self):
        return f"{type(self).__name__}({self.greens!r}, precision={self.precision!r})"


class DirectBEM(BEMFormulation):
    """DirectBEM{G} (formulations.jl:7-11)."""
    direct = True


class IndirectBEM(BEMFormulation):
    """IndirectBEM{G} (formulations.jl:13-17)."""
    direct = False


def is_direct(f: BEMFormulation) -> bool:
    return bool(f.direct)


def bem_formulation(formulation=None, direct=True, gf="Wu", greens_functions=None):
    """bem_formulation (formulations.jl:33-37)."""
    if formulation is not None:
        return formulation
    gfs = default_greens_functions(gf) if greens_functions is None else greens_functions
    return DirectBEM(gfs) if direct else IndirectBEM(gfs)
