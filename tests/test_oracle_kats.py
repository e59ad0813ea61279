"""Pin the CPU oracle to the known-answer values of the reference's own tests.

Golden values: tests/golden/reference_kats.json, extracted from
test/rankine_vectorized.jl, test/greens_function.jl and
test/consistency_with_analytical_solutions.jl by tests/golden/extract_reference_kats.py.
Tolerances are the reference's own.
"""
import numpy as np
import pytest


@pytest.mark.parametrize("panel", ["square", "twisted", "triangle"])
def test_birk_geometry(oracle, kats, panel):
    c = kats["birk"][panel]
    T, qgc, lc, A = oracle.birk_panel_geometry(c["corners"])
    tol = c["tol_geometry"]
    assert A == pytest.approx(c["area"], abs=tol)
    np.testing.assert_allclose(T, np.array(c["T"]), atol=tol)
    np.testing.assert_allclose(qgc, c["qgc"], atol=tol)
    if c["local_corners"]:
        np.testing.assert_allclose(lc, np.array(c["local_corners"])[:, :2], atol=tol)


@pytest.mark.parametrize("panel", ["square", "twisted", "triangle"])
def test_birk_phi_velocity_hessian(oracle, kats, panel):
    """rankine_vectorized.jl:44-62, 86-109, 129-151: phi, v, H tables + Laplace."""
    c = kats["birk"][panel]
    T, qgc, lc, _ = oracle.birk_panel_geometry(c["corners"])
    for row in c["cases"]:
        p = T.T @ (np.array(row["point"]) - qgc)
        if "point_local" in row:
            np.testing.assert_allclose(p, row["point_local"], atol=c["tol_geometry"])
        phi = oracle.birk_velocity_potential(*p, lc)
        v = T @ oracle.birk_velocity_derivatives(*p, lc)
        H = T @ oracle.birk_velocity_hessian(*p, lc) @ T.T
        assert phi == pytest.approx(row["phi"], abs=c["tol_phi"])
        np.testing.assert_allclose(v, row["v"], atol=c["tol_v"])
        if "H" in row:
            np.testing.assert_allclose(H, np.array(row["H"]), atol=c["tol_H"])
        assert abs(np.trace(H)) < c["tol_laplace"]
        # fused eq. (46)+(47)-(49) equals the separate loops (rankine_vectorized.jl:155-175)
        phi2, v2 = oracle.birk_phi_and_velocity(*p, lc)
        assert phi2 == pytest.approx(phi, abs=1e-14, rel=1e-14)
        np.testing.assert_allclose(T @ v2, v, atol=1e-14, rtol=1e-14)
    for row in c.get("hessian_cases", []):
        p = T.T @ (np.array(row["point"]) - qgc)
        H = T @ oracle.birk_velocity_hessian(*p, lc) @ T.T
        np.testing.assert_allclose(H, np.array(row["H"]), atol=c["tol_H"])


def test_fused_matches_separate_degenerate(oracle):
    """rankine_vectorized.jl:155-175 incl. the z=0 and degenerate-edge (triangle) cases."""
    lc = np.array([[-0.5, -0.5], [0.5, -0.5], [0.5, 0.5], [-0.5, 0.5]])
    for x, y, z in ((0.1, 0.2, 0.4), (0.0, 0.0, 0.0), (0.5, 1.0, 0.0), (-0.25, 0.25, 0.5)):
        phi1 = oracle.birk_velocity_potential(x, y, z, lc)
        v1 = oracle.birk_velocity_derivatives(x, y, z, lc)
        phi2, v2 = oracle.birk_phi_and_velocity(x, y, z, lc)
        assert phi2 == pytest.approx(phi1, abs=1e-14, rel=1e-14)
        np.testing.assert_allclose(v2, v1, atol=1e-14, rtol=1e-14)
    tri = np.array([[-0.5, -0.5], [0.5, -0.5], [0.5, 0.5], [0.5, 0.5]])
    phi1 = oracle.birk_velocity_potential(0.1, 0.2, 0.3, tri)
    phi2, v2 = oracle.birk_phi_and_velocity(0.1, 0.2, 0.3, tri)
    assert phi2 == pytest.approx(phi1, abs=1e-14, rel=1e-14)
    np.testing.assert_allclose(v2, oracle.birk_velocity_derivatives(0.1, 0.2, 0.3, tri), atol=1e-14, rtol=1e-14)


def test_delhommeau_dimensionless_term(oracle, kats):
    """greens_function.jl:81-89 (Capytaine Fortran core values, atol 1e-4)."""
    d = kats["delhommeau_dimless"]
    G = oracle.egd_dimless(d["r"], d["z"])
    dG = oracle.egd_dimless_dr(d["r"], d["z"])
    assert abs(G - complex(*d["G"])) < d["atol"]
    assert abs(dG - complex(*d["dG_dr"])) < d["atol"]
    # the reference integrates at Integrals.jl's default tolerance (1e-8); same answer within it
    G8 = oracle.egd_dimless(d["r"], d["z"], rtol=1e-8, atol=1e-8)
    assert abs(G8 - G) < 1e-7


def test_delhommeau_green_function_pair(oracle, kats):
    """greens_function.jl:91-98: G and grad_x G for the canonical element pair at k=1."""
    d = kats["delhommeau_pair"]
    g, grad = oracle.point_greens(oracle.GF_EXACT_DELHOMMEAU, d["e1_center"], d["e2_center"], d["k"],
                                  wrt_first=True)
    assert abs(g - complex(*d["G"])) < d["atol"]
    np.testing.assert_allclose(grad, [complex(*z) for z in d["grad_wrt_first"]], atol=d["atol"])


def test_wu_matches_delhommeau(oracle, kats):
    """greens_function.jl:96-99: Wu approximates the exact term within 2e-2."""
    cp = kats["canonical_pair"]
    for k in cp["wu_vs_delhommeau_k"]:
        for wrt in (False,):
            gw, gw_grad = oracle.point_greens(oracle.GF_WU, cp["e1_center"], cp["e2"]["center"], k, wrt)
            ge, ge_grad = oracle.point_greens(oracle.GF_EXACT_DELHOMMEAU, cp["e1_center"], cp["e2"]["center"], k, wrt)
            assert abs(gw - ge) < cp["wu_vs_delhommeau_atol"]
            np.testing.assert_allclose(gw_grad, ge_grad, atol=cp["wu_vs_delhommeau_atol"])


def test_rankine_closed_forms(oracle, kats):
    """greens_function.jl:44-52, 74-79: point Rankine and its image."""
    cp = kats["canonical_pair"]
    e1, e2 = np.array(cp["e1_center"]), np.array(cp["e2"]["center"])
    g, gr = oracle.point_greens(oracle.GF_RANKINE, e1, e2, 1.0, True)
    assert g.real == pytest.approx(1 / np.sqrt(3), abs=1e-8)
    np.testing.assert_allclose(gr.real, (e2 - e1) / np.sqrt(3) ** 3, atol=1e-8)
    g, gr = oracle.point_greens(oracle.GF_RANKINE, e1, e2, 1.0, False)
    np.testing.assert_allclose(gr.real, (e1 - e2) / np.sqrt(3) ** 3, atol=1e-8)
    refl = lambda v: np.array([v[0], v[1], -v[2]])
    g, gr = oracle.point_greens(oracle.GF_RANKINE_REFLECTED, e1, e2, 1.0, True)
    assert g.real == pytest.approx(1 / np.sqrt(11), abs=1e-8)
    np.testing.assert_allclose(gr.real, (refl(e2) - e1) / np.sqrt(11) ** 3, atol=1e-8)
    g, gr = oracle.point_greens(oracle.GF_RANKINE_REFLECTED, e1, e2, 1.0, False)
    np.testing.assert_allclose(gr.real, refl(e1 - refl(e2)) / np.sqrt(11) ** 3, atol=1e-8)


def test_rankine_matches_delhommeau_rankine(oracle, kats):
    """rankine_vectorized.jl:177-200: Birk vs Delhommeau panel integrals, canonical pair, rtol 1e-4."""
    cp = kats["canonical_pair"]
    e2 = cp["e2"]
    tol = cp["rankine_vs_delhommeau_rtol"]
    for kb, kd in ((oracle.GF_RANKINE, oracle.GF_DELHOMMEAU_RANKINE),
                   (oracle.GF_RANKINE_REFLECTED, oracle.GF_DELHOMMEAU_RANKINE_REFLECTED)):
        for wrt in (True, False):
            ib, gb = oracle.pair_integrals(kb, cp["e1_center"], e2["vertices"], e2["center"], e2["normal"],
                                           e2["area"], e2["radius"], 1.0, wrt)
            idd, gd = oracle.pair_integrals(kd, cp["e1_center"], e2["vertices"], e2["center"], e2["normal"],
                                            e2["area"], e2["radius"], 1.0, wrt)
            assert abs(ib - idd) <= tol + tol * abs(idd)
            np.testing.assert_allclose(gb, gd, rtol=tol, atol=tol)


def test_exp_e1_against_mpmath(oracle):
    """The restated complex E1 (DLMF 6.6.2 / 6.9.1) against mpmath on the quadrature's domain."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    rng = np.random.default_rng(1)
    worst = 0.0
    zs = [complex(-x, y) for x in (1e-3, 0.5, 3.0, 12.0, 40.0, 60.0) for y in (0.0, 1e-3, 0.7, 5.0, 30.0, 900.0)]
    zs += [complex(-rng.uniform(0, 60), rng.uniform(0, 1000) * rng.uniform(0, 1) ** 3) for _ in range(300)]
    for z in zs:
        ref = complex(mp.exp(mp.mpc(z.real, z.imag)) * mp.e1(mp.mpc(z.real, z.imag)))
        worst = max(worst, abs(oracle.exp_e1(z) - ref) / abs(ref))
    assert worst < 1e-13
