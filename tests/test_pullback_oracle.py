"""The oracle's restatement of the solve pullback (ad_rules.jl:300-414 applied to
solve(D, S, bc; direct), matrix_assembly.jl:436-449) against central differences of the
oracle's own solve, on the CPU.  This pins the adjoint oracle that the GPU pullback and
the GPU gradients are compared with."""
import numpy as np
import pytest


def _rand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _objective(oracle, D, S, b, pb, sb, direct):
    phi, src = oracle.solve(D, S, b, direct=direct)
    J = np.real(np.sum(np.conj(pb) * phi))
    if sb is not None:
        J += np.real(np.sum(np.conj(sb) * src))
    return J


@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_pullback_matches_central_differences(oracle, direct, nrhs):
    rng = np.random.default_rng(3 + nrhs + 10 * direct)
    n = 14
    D = _rand(rng, n, n) + 4 * n ** 0.5 * np.eye(n)
    S = _rand(rng, n, n)
    b = _rand(rng, n, nrhs) if nrhs > 1 else _rand(rng, n)
    pb = _rand(rng, *b.shape)
    sb = None if direct else _rand(rng, *b.shape)
    phi, src, Db, Sb, bb = oracle.solve_pullback(D, S, b, pb, direct=direct, sources_bar=sb)
    phi0, src0 = oracle.solve(D, S, b, direct=direct)
    assert np.allclose(phi, phi0, rtol=0, atol=1e-13 * np.abs(phi0).max())
    h = 1e-6
    for _ in range(3):
        ED, ES, Eb = _rand(rng, n, n), _rand(rng, n, n), _rand(rng, *b.shape)
        jp = _objective(oracle, D + h * ED, S + h * ES, b + h * Eb, pb, sb, direct)
        jm = _objective(oracle, D - h * ED, S - h * ES, b - h * Eb, pb, sb, direct)
        fd = (jp - jm) / (2 * h)
        ad = np.real(np.sum(np.conj(Db) * ED) + np.sum(np.conj(Sb) * ES) + np.sum(np.conj(bb) * Eb))
        assert abs(ad - fd) <= 1e-7 * max(abs(fd), 1.0), (ad, fd)
