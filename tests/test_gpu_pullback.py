"""Matrix-level pullback of solve(D, S, bc; direct) on the device (mh_solve_pullback)
against the oracle's restatement of the reference's _mulvec / _linearsolve rules
(ad_rules.jl:300-414), itself pinned to central differences in test_pullback_oracle.py.
Bar: 1e-11 relative (Frobenius) on every output."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-11


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
@pytest.mark.parametrize("direct", [True, False])
def test_pullback_of_bem_solve_matches_oracle(mh, oracle, ctx, direct, precision):
    mesh = mh.hemisphere_mesh(1.0, 6, 14)
    k = 1.2 ** 2 / 9.81
    S, D = mh.assemble_matrices(mh.default_greens_functions("Wu"), mesh, k, direct=direct, ctx=ctx)
    rng = np.random.default_rng(9)
    n = mesh.nfaces
    for nrhs in (1, 3):
        shape = (n,) if nrhs == 1 else (n, nrhs)
        b = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        pb = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        sb = None if direct else rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        got = mh.solve_pullback(D, S, b, pb, direct=direct, sources_bar=sb, precision=precision, ctx=ctx)
        ref = oracle.solve_pullback(D, S, b, pb, direct=direct, sources_bar=sb)
        for name, g_, r_ in zip(("phi", "sources", "D_bar", "S_bar", "bc_bar"), got, ref):
            if r_ is None:
                assert g_ is None
                continue
            assert np.shape(g_) == np.shape(r_), name
            assert rel(g_, r_) < REL, (name, rel(g_, r_))


def test_pullback_rejects_sources_cotangent_for_direct(mh, ctx):
    A = np.eye(4, dtype=complex)
    with pytest.raises(Exception):
        mh.solve_pullback(A, A, np.ones(4), np.ones(4), direct=True, sources_bar=np.ones(4), ctx=ctx)
