"""CUDA path vs the CPU oracle, through the C-ABI (libmarinehydro_cuda.so).

Tolerances (the parity bar of the plain FP64 path): S, D relative error <= 1e-10 (Frobenius
norm over the matrix); added mass, damping and excitation force <= 1e-8.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_SD = 1e-10
REL_COEF = 1e-8


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300)


GF_SETS = {
    "default_wu": ("RANKINE", "RANKINE_REFLECTED", "WU"),
    "rankine": ("RANKINE",),
    "rankine_image": ("RANKINE", "RANKINE_REFLECTED"),
    "negative_image": ("RANKINE", "RANKINE_REFLECTED_NEGATIVE"),
    "wu_only": ("WU",),
    "delhommeau_rankine_wu": ("DELHOMMEAU_RANKINE", "DELHOMMEAU_RANKINE_REFLECTED", "WU"),
    "mixed_static": ("RANKINE", "DELHOMMEAU_RANKINE_REFLECTED", "WU"),
}


def flags(oracle, names):
    return sum(getattr(oracle, "GF_" + n) for n in names)


def gf_tuple(mh, names):
    m = {"RANKINE": mh.Rankine, "RANKINE_REFLECTED": mh.RankineReflected,
         "RANKINE_REFLECTED_NEGATIVE": mh.RankineReflectedNegative, "DELHOMMEAU_RANKINE": mh.DelhommeauRankine,
         "DELHOMMEAU_RANKINE_REFLECTED": mh.DelhommeauRankineReflected, "WU": mh.GFWu,
         "EXACT_DELHOMMEAU": mh.ExactGuevelDelhommeau}
    return tuple(m[n]() for n in names)


def test_bessel01_points(mh, ctx):
    # the joint J0/J1/Y0/Y1 evaluator of the Wu kernels against scipy's (Cephes) Bessel
    # functions: absolute error, dense over the polynomial intervals and the Hankel region
    special = pytest.importorskip("scipy.special")
    rng = np.random.default_rng(3)
    x = np.concatenate([[0.0, 1e-12, 2.9999999, 3.0, 7.9999999999, 8.0, 8.0000000001, 1e3, 3.3e4],
                        np.linspace(0, 8, 1601), rng.uniform(0, 40, 2000), 10 ** rng.uniform(1, 3, 500)])
    got = mh._device.bessel01_points(ctx, x)
    ref = np.stack([special.j0(x), special.j1(x), special.y0(x), special.y1(x)], axis=1)
    for c in range(2):
        assert np.abs(got[:, c] - ref[:, c]).max() < 4e-15, (c, np.abs(got[:, c] - ref[:, c]).max())
    ok = x >= 3.0
    assert np.isnan(got[~ok, 2:]).all()
    for c in (2, 3):
        assert np.abs(got[ok, c] - ref[ok, c]).max() < 4e-15, (c, np.abs(got[ok, c] - ref[ok, c]).max())


def test_fixpoint_functions(mh, ctx):
    # exp, log, reciprocal and square root of the Wu term, evaluated in 64-bit fixed point on
    # the integer pipe, against numpy's FP64 functions: reciprocal and square root within an
    # ulp of the correctly rounded result, exp and log within two ulps of numpy's (log: ulps
    # of max(|log x|, 1/2), the absolute error the Wu term sees)
    rng = np.random.default_rng(11)
    x = np.concatenate([[1.0, 2.0, 0.5, 1 + 2.0 ** -52, 2 - 2.0 ** -52, 3.0, 7.999999999999, 8.0, 744.0, 1e-300,
                         2.0 ** -40],
                        rng.uniform(0, 2, 4000), 10 ** rng.uniform(-12, 2.85, 4000), 10 ** rng.uniform(-300, 300, 2000)])
    got = mh._device.fixpoint_points(ctx, x)
    ulp = lambda v: np.spacing(np.abs(v))
    e = np.exp(-x)
    ok = e > 2.3e-308  # below the normal range the integer path flushes to zero
    assert np.all(np.abs(got[ok, 0] - e[ok]) <= 2.0 * ulp(e[ok])), np.max(np.abs(got[ok, 0] - e[ok]) / ulp(e[ok]))
    assert np.all(np.abs(got[~ok, 0]) < 2.3e-308)
    lg = np.log(x)
    assert np.all(np.abs(got[:, 1] - lg) <= 2.0 * ulp(np.maximum(np.abs(lg), 0.5)))
    r = 1.0 / x
    assert np.all(np.abs(got[:, 2] - r) <= ulp(r))
    q = np.sqrt(x)
    assert np.all(np.abs(got[:, 3] - q) <= ulp(q))


def test_wu_wave_terms(mh, oracle, ctx):
    rng = np.random.default_rng(0)
    hh = np.concatenate([[0.0, 1e-7, 2.999, 3.0, 3.001], rng.uniform(0, 20, 300), 10 ** rng.uniform(-3, 2, 200)])
    vv = -np.concatenate([[0.5, 1.0, 2.0, 0.1, 5.0], rng.uniform(1e-3, 30, 300), 10 ** rng.uniform(-3, 1.3, 200)])
    got = mh._device.wu_wave_terms(ctx, hh, vv)
    ref = np.array([oracle.wu_wave_term_and_derivs(h, v) for h, v in zip(hh, vv)])
    # The polynomial fits A-D of wu.jl:131-329 have coefficients up to 2e5 with
    # alternating signs evaluated at rho in (0, 1): the reference's FP64 rounding of the
    # partial sums (the oracle follows it) is amplified to ~3e-11 absolute, while the GPU
    # evaluates them in 64-bit fixed point (error ~4e-13).
    for c in range(3):
        err = np.abs(got[:, c] - ref[:, c]) / np.maximum(np.abs(ref[:, c]), 1.0)
        assert err.max() < 1e-10, (c, err.max())
        assert np.median(err) < 1e-14, (c, np.median(err))


def test_exact_wave_terms(mh, oracle, ctx):
    # includes large r with small |z|: hundreds of oscillations of the integrand
    rs = np.array([0.0, 1e-4, 0.3, 1.0, 2.5, 7.0, 40.0, 300.0, 300.0, 950.0, 120.0])
    zs = -np.array([1.0, 0.05, 0.8, 1.0, 3.0, 0.4, 20.0, 49.0, 0.5, 2.0, 0.02])
    got = mh._device.exact_wave_terms(ctx, rs, zs, rtol=1e-12, atol=1e-14)
    for i, (r, z) in enumerate(zip(rs, zs)):
        G = oracle.egd_dimless(r, z, 1e-12, 1e-14)
        dG = oracle.egd_dimless_dr(r, z, 1e-12, 1e-14)
        assert abs(got[i, 0] - G) <= 1e-10 * max(1.0, abs(G)), (r, z, got[i, 0], G)
        assert abs(got[i, 1] - dG) <= 1e-10 * max(1.0, abs(dG)), (r, z, got[i, 1], dG)


@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("gfs", list(GF_SETS))
def test_assembly_hemisphere(mh, oracle, ctx, gfs, direct):
    mesh = mh.config1_hemisphere()
    k = 1.03 ** 2 / 9.81
    names = GF_SETS[gfs]
    S, D = mh.assemble_matrices(gf_tuple(mh, names), mesh, k, direct=direct, ctx=ctx)
    So, Do = oracle.assemble_matrices(mesh, k, gfs=flags(oracle, names), direct=direct)
    assert rel(S, So) < REL_SD
    assert rel(D, Do) < REL_SD


def test_assembly_fixed_normal_no_identity(mh, oracle, ctx):
    mesh = mh.hemisphere_mesh(1.0, 6, 12)
    k = 0.7
    for include_identity in (True, False):
        for fixed in (None, [1.0, 0.0, 0.0]):
            S, D = mh.assemble_matrices(mh.default_greens_functions("Wu"), mesh, k, direct=False,
                                        include_identity=include_identity, all_normals=fixed, ctx=ctx)
            So, Do = oracle.assemble_matrices(mesh, k, gfs=oracle.DEFAULT_WU, direct=False,
                                              include_identity=include_identity, fixed_normal=fixed)
            assert rel(S, So) < REL_SD
            assert rel(D, Do) < REL_SD


def test_assembly_tiny_mesh_and_static_reuse(mh, oracle, ctx):
    """Two-panel fixture (test/gpu.jl:36-57) and static+wave decomposition
    (test/matrix_assembly.jl:37-68): the cached Rankine part is reused across k."""
    mesh = mh.tiny_static_mesh()
    gfs = mh.default_greens_functions("Wu")
    for k in (1.0, 0.7, 1.5):
        S, D = mh.assemble_matrices(gfs, mesh, k, ctx=ctx)
        So, Do = oracle.assemble_matrices(mesh, k, gfs=oracle.DEFAULT_WU)
        assert rel(S, So) < REL_SD and rel(D, Do) < REL_SD
    big = mh.config1_hemisphere()
    static, wave = mh.partition_greens_functions(gfs)
    Ss1, Ds1 = mh.assemble_matrices(static, big, 1.0, ctx=ctx)
    Ss2, Ds2 = mh.assemble_matrices(static, big, 2.0, ctx=ctx)
    np.testing.assert_array_equal(Ss1, Ss2)
    for k in (0.7, 1.5):
        Sf, Df = mh.assemble_matrices(gfs, big, k, ctx=ctx)
        Sw, Dw = mh.assemble_matrices(wave, big, k, include_identity=False, ctx=ctx)
        assert rel(Sf, Ss1 + Sw) < 1e-14
        assert rel(Df, Ds1 + Dw) < 1e-14


def test_assembly_exact_delhommeau_small(mh, oracle, ctx):
    mesh = mh.hemisphere_mesh(1.0, 4, 8)
    k = 1.2
    ctx.set_quadrature_tolerance(1e-12, 1e-14)
    oracle.set_egd_tolerance(1e-12, 1e-14)
    for direct in (True, False):
        S, D = mh.assemble_matrices(mh.default_greens_functions("ExactGuevelDelhommeau"), mesh, k, direct=direct,
                                    ctx=ctx)
        So, Do = oracle.assemble_matrices(mesh, k, gfs=oracle.DEFAULT_EGD, direct=direct)
        assert rel(S, So) < REL_SD
        assert rel(D, Do) < REL_SD


def _well_conditioned(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = A / np.sqrt(n) + 2.0 * np.eye(n)
    B = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    return np.asfortranarray(A), np.asfortranarray(B)


@pytest.mark.parametrize("n,nrhs", [(1, 1), (7, 3), (33, 1), (64, 2), (200, 7), (531, 9)])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
def test_linsolve(mh, ctx, n, nrhs, precision):
    A, B = _well_conditioned(n, nrhs, n)
    X = mh.linsolve(A, B, precision=precision, ctx=ctx)
    Xr = np.linalg.solve(A, B)
    assert rel(X, Xr) < 1e-12
    x = mh.linsolve(A, B[:, 0], precision=precision, ctx=ctx)
    assert x.shape == (n,) and rel(x, Xr[:, 0]) < 1e-12
    L = mh.linsolve_adjoint(A, B, precision=precision, ctx=ctx)
    assert rel(L, np.linalg.solve(A.conj().T, B)) < 1e-12


def test_linsolve_needs_pivoting_and_singular(mh, ctx):
    A = np.array([[0.0, 1.0, 2.0], [1.0, 0.0, 3.0], [4.0, -3.0, 8.0]], dtype=complex)
    b = np.array([1.0, 2.0, 3.0], dtype=complex)
    assert rel(mh.linsolve(A, b, ctx=ctx), np.linalg.solve(A, b)) < 1e-14
    with pytest.raises(np.linalg.LinAlgError):
        mh.linsolve(np.zeros((4, 4), dtype=complex), np.ones(4, dtype=complex), ctx=ctx)
    with pytest.raises(ValueError):
        mh.linsolve(np.eye(3, dtype=complex), np.ones(4, dtype=complex), ctx=ctx)


@pytest.mark.parametrize("direct", [True, False])
def test_solve_matrix_level(mh, oracle, ctx, direct):
    mesh = mh.config1_hemisphere()
    k = 1.03 ** 2 / 9.81
    So, Do = oracle.assemble_matrices(mesh, k, gfs=oracle.DEFAULT_WU, direct=direct)
    bc = -1j * 1.03 * mesh.normals[:, 2]
    phi, src = mh.solve_linear(Do, So, bc, direct=direct, ctx=ctx)
    phio, srco = oracle.solve(Do, So, bc, direct=direct)
    assert rel(phi, phio) < 1e-11
    if not direct:
        assert rel(src, srco) < 1e-11


@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
def test_hydro_config1(mh, oracle, ctx, direct, precision):
    """200-panel hemisphere, omega = 1.03, rho = 1025, Heave radiation + beta = 0 diffraction."""
    mesh = mh.config1_hemisphere()
    body = mh.FloatingBody(mesh, ["Heave"], body_name="hemisphere")
    params = {"wave_frequencies": [1.03], "radiating_dofs": ["Heave"], "influenced_dofs": ["Heave"],
              "wave_directions": [0.0]}
    F = mh.DirectBEM(precision=precision) if direct else mh.IndirectBEM(precision=precision)
    res = mh.hydrodynamic_coefficients(body, params, F, ctx=ctx, rho=1025.0)
    A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(mesh, body.dofs, 1.03, rho=1025.0, direct=direct, betas=[0.0])
    assert abs(res["added_mass"].ravel()[0] - A[0, 0]) <= REL_COEF * abs(A[0, 0])
    assert abs(res["radiation_damping"].ravel()[0] - B[0, 0]) <= REL_COEF * abs(B[0, 0])
    assert abs(res["diffraction_force"].ravel()[0] - Fd[0, 0]) <= REL_COEF * abs(Fd[0, 0])
    assert abs(res["Froude_Krylov_force"].ravel()[0] - Fk[0, 0]) <= REL_COEF * abs(Fk[0, 0])
    assert abs(res["excitation_force"].ravel()[0] - Fe[0, 0]) <= REL_COEF * abs(Fe[0, 0])


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
@pytest.mark.parametrize("direct", [True, False])
def test_hydro_sweep_six_dofs(mh, oracle, ctx, precision, direct):
    """Several frequencies, 6 rigid dofs radiating + 2 headings, against the oracle per frequency,
    for each precision of the LU (FP64 CUDA-core update, FP32 factors refined in FP64, FP64 with
    the tensor-core update)."""
    mesh = mh.vertical_cylinder_mesh(2.0, 3.0, 16, 6, 4)
    dofs = ["Surge", "Sway", "Heave", "Roll", "Pitch", "Yaw"]
    body = mh.FloatingBody(mesh, dofs, rotation_center=(0.0, 0.0, -1.0), body_name="cyl")
    oms = [0.4, 1.1, 2.3]
    betas = [0.0, np.pi / 3]
    F = (mh.DirectBEM if direct else mh.IndirectBEM)(precision=precision)
    res = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": dofs,
                                              "influenced_dofs": dofs, "wave_directions": betas},
                                       F, ctx=ctx, rho=1025.0)
    assert res["added_mass"].shape == (6, 6, 3, 1)
    assert res["excitation_force"].shape == (6, 3, 2, 1)
    for w, om in enumerate(oms):
        A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(mesh, body.dofs, om, rho=1025.0, betas=betas,
                                                      direct=direct)
        scale_a = np.abs(A).max()
        scale_b = np.abs(B).max()
        assert np.abs(res["added_mass"][:, :, w, 0] - A).max() <= REL_COEF * scale_a
        assert np.abs(res["radiation_damping"][:, :, w, 0] - B).max() <= REL_COEF * scale_b
        assert np.abs(res["excitation_force"][:, w, :, 0] - Fe).max() <= REL_COEF * np.abs(Fe).max()


def test_problem_level_solve_matches_sweep(mh, ctx):
    mesh = mh.hemisphere_mesh(1.0, 6, 12)
    body = mh.FloatingBody(mesh, ["Heave", "Surge"], body_name="sphere")
    r = mh.solve(mh.RadiationProblem(body, 1.3, "Heave", ["Heave", "Surge"], rho=1025.0), mh.DirectBEM(), ctx=ctx)
    d = mh.solve(mh.DiffractionProblem(body, 1.3, 0.0, ["Heave", "Surge"], rho=1025.0), mh.DirectBEM(), ctx=ctx)
    res = mh.hydrodynamic_coefficients(body, {"wave_frequencies": [1.3], "radiating_dofs": ["Heave"],
                                              "influenced_dofs": ["Heave", "Surge"], "wave_directions": [0.0]},
                                       ctx=ctx, rho=1025.0)
    a = mh.added_mass(r)
    assert a["Heave"] == pytest.approx(res["added_mass"][0, 0, 0, 0], rel=1e-10)
    assert a["Surge"] == pytest.approx(res["added_mass"][1, 0, 0, 0], rel=1e-8, abs=1e-8 * abs(a["Heave"]))
    fe = mh.excitation_force(d)
    assert abs(fe["Heave"] - res["excitation_force"][0, 0, 0, 0]) <= 1e-10 * abs(fe["Heave"])


def test_hulme_heaving_hemisphere(mh, kats, ctx):
    """Hulme (1982) table, rtol 0.1 (consistency_with_analytical_solutions.jl:52-76)."""
    h = kats["hulme_heave"]
    mesh = mh.hemisphere_mesh(1.0, 10, 20)
    body = mh.FloatingBody(mesh, ["Heave"], body_name="hemisphere")
    K = np.array(h["K"])
    oms = np.sqrt(K * h["g_for_omega"])
    res = mh.hydrodynamic_coefficients(body, {"wave_frequencies": oms, "radiating_dofs": ["Heave"],
                                              "influenced_dofs": ["Heave"]}, ctx=ctx, rho=h["rho"], g=9.81)
    m = 2 / 3 * np.pi * h["radius"] * h["rho"]
    A = res["added_mass"][0, 0, :, 0] / m
    B = res["radiation_damping"][0, 0, :, 0] / m / oms
    np.testing.assert_allclose(A, h["A"], rtol=h["rtol"])
    np.testing.assert_allclose(B, h["B"], rtol=h["rtol"], atol=2e-3)


def test_config2_scale_properties(mh, oracle, ctx):
    """2000-panel cylinder: full-matrix parity of S, D and an FP64 residual check of the LU."""
    mesh = mh.config2_cylinder()
    k = 1.5 ** 2 / 9.81
    S, D = mh.assemble_matrices(mh.default_greens_functions("Wu"), mesh, k, ctx=ctx)
    So, Do = oracle.assemble_matrices(mesh, k, gfs=oracle.DEFAULT_WU)
    assert rel(S, So) < REL_SD and rel(D, Do) < REL_SD
    rng = np.random.default_rng(3)
    B = rng.standard_normal((mesh.nfaces, 7)) + 1j * rng.standard_normal((mesh.nfaces, 7))
    for precision in ("fp64", "mixed"):
        X = mh.linsolve(D, B, precision=precision, ctx=ctx)
        r = np.linalg.norm(D @ X - B) / (np.linalg.norm(D) * np.linalg.norm(X))
        assert r < 1e-15


@pytest.mark.parametrize("direct", [True, False])
def test_sweep_tensor_core_fp64_update(mh, ctx, direct):
    """The FP64 LU with its trailing update on the BF16 tensor cores (Ozaki splitting) gives
    the FP64 path's coefficients to FP64 rounding (two panel steps and ragged tiles: N = 300)."""
    body = mh.FloatingBody(mh.vertical_cylinder_mesh(2.0, 3.0, 20, 10, 5), ["Heave", "Surge", "Pitch"],
                           rotation_center=(0.0, 0.0, 0.0))
    p = {"wave_frequencies": [0.5, 1.1, 2.3], "radiating_dofs": ["Heave", "Surge", "Pitch"],
         "wave_directions": [0.0, 0.4]}
    F = mh.DirectBEM if direct else mh.IndirectBEM
    r64 = mh.hydrodynamic_coefficients(body, p, F(precision="fp64"), ctx=ctx, rho=1025.0)
    rtc = mh.hydrodynamic_coefficients(body, p, F(precision="fp64_tc"), ctx=ctx, rho=1025.0)
    for key in ("added_mass", "radiation_damping", "excitation_force"):
        a, b = rtc[key], r64[key]
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), key
