"""Many-body batch (one CUDA graph over several streams) vs the CPU oracle and vs per-body sweeps.

The batch is checked directly against the oracle (per body and per frequency, at the
1e-8 coefficient bar) for bodies of uneven panel counts, one of them a two-body array,
in each precision of the LU; the batched schedule must also reproduce the per-body
sweep for uneven frequency counts, on the first call (capture) and on a second call
with new frequencies (cached graph, new parameters).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-10


def _bodies(mh):
    meshes = [mh.hemisphere_mesh(1.0, 6, 12), mh.vertical_cylinder_mesh(2.0, 3.0, 16, 4, 3),
              mh.barge_mesh(12.0, 4.0, 2.0, 8, 3, 2)]
    return [mh.FloatingBody(m, ["Heave", "Pitch"], rotation_center=(0.0, 0.0, 0.0), body_name=f"b{i}")
            for i, m in enumerate(meshes)]


def _check(res, ref):
    for key in ("added_mass", "radiation_damping", "excitation_force", "diffraction_force", "Froude_Krylov_force"):
        a, b = np.asarray(res[key]), np.asarray(ref[key])
        assert a.shape == b.shape, key
        assert np.abs(a - b).max() <= REL * max(np.abs(b).max(), 1e-30), key


@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
def test_batch_matches_per_body(mh, ctx, direct, precision):
    bodies = _bodies(mh)
    F = (mh.DirectBEM if direct else mh.IndirectBEM)(precision=precision)
    rng = np.random.default_rng(5)
    for call in range(2):  # second call: cached graph, new frequencies
        params = [{"wave_frequencies": np.sort(rng.uniform(0.3, 2.5, nw)), "radiating_dofs": ["Heave", "Pitch"],
                   "influenced_dofs": ["Heave", "Pitch"], "wave_directions": [0.0, 0.7]} for nw in (3, 2, 4)]
        out = mh.batch_hydrodynamic_coefficients(bodies, params, F, ctx=ctx, rho=1025.0, n_streams=2)
        for body, p, res in zip(bodies, params, out):
            ref = mh.hydrodynamic_coefficients(body, p, F, ctx=ctx, rho=1025.0)
            _check(res, ref)


REL_COEF = 1e-8


def _oracle_batches(mh):
    """Bodies of 100-300 panels: three single bodies in one batch, and two two-cylinder arrays
    (interaction terms) in another -- a batch takes bodies with the same dof names."""
    single = [mh.hemisphere_mesh(1.0, 8, 16), mh.vertical_cylinder_mesh(2.0, 3.0, 20, 8, 3),
              mh.barge_mesh(12.0, 4.0, 2.0, 12, 4, 3)]
    singles = [mh.FloatingBody(m, ["Heave", "Pitch"], rotation_center=(0.0, 0.0, 0.0), body_name=f"s{i}")
               for i, m in enumerate(single)]
    arrays = []
    for sep, nth in ((4.0, 10), (6.0, 14)):
        m1 = mh.vertical_cylinder_mesh(1.0, 1.5, nth, 4, 2)
        m2 = mh.vertical_cylinder_mesh(1.0, 1.5, nth, 4, 2, center=(sep, 1.0))
        arrays.append(mh.FloatingBody(m1, ["Heave", "Pitch"], rotation_center=(0.0, 0.0, 0.0), body_name="a") +
                      mh.FloatingBody(m2, ["Heave", "Pitch"], rotation_center=(sep, 1.0, 0.0), body_name="b"))
    return [singles, arrays]


@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
def test_batch_matches_oracle(mh, oracle, ctx, direct, precision):
    F = (mh.DirectBEM if direct else mh.IndirectBEM)(precision=precision)
    rng = np.random.default_rng(17)
    for bodies in _oracle_batches(mh):
        sizes = [b.mesh.nfaces for b in bodies]
        assert min(sizes) >= 100 and max(sizes) <= 300 and len(set(sizes)) == len(sizes), sizes
        params = []
        for i, b in enumerate(bodies):
            names = list(b.dofs)
            params.append({"wave_frequencies": np.sort(rng.uniform(0.3, 2.5, 3 - i % 2)), "radiating_dofs": names,
                           "influenced_dofs": names, "wave_directions": [0.0, 0.9]})
        out = mh.batch_hydrodynamic_coefficients(bodies, params, F, ctx=ctx, rho=1025.0, n_streams=2)
        for b, p, res in zip(bodies, params, out):
            for w, om in enumerate(p["wave_frequencies"]):
                A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(b.mesh, b.dofs, float(om), rho=1025.0,
                                                              direct=direct, betas=[0.0, 0.9])
                for got, ref in ((res["added_mass"][:, :, w, 0], A), (res["radiation_damping"][:, :, w, 0], B),
                                 (res["diffraction_force"][:, w, :, 0], Fd),
                                 (res["Froude_Krylov_force"][:, w, :, 0], Fk),
                                 (res["excitation_force"][:, w, :, 0], Fe)):
                    assert np.abs(got - ref).max() <= REL_COEF * np.abs(ref).max(), (b.body_name, om)


def test_batch_rejects_mixed_dof_names(mh, ctx):
    b = _bodies(mh)
    b[1] = mh.FloatingBody(b[1].mesh, ["Heave"], body_name="other")
    with pytest.raises(ValueError):
        mh.batch_hydrodynamic_coefficients(b, [{"wave_frequencies": [1.0], "radiating_dofs": ["Heave"]}] * 3,
                                           ctx=ctx)


def test_batch_after_a_mesh_is_destroyed(mh, ctx):
    """The cached batch graph is keyed by mesh addresses; destroying a mesh drops the graph,
    so a new mesh (possibly at the same address) is never served the old one's buffers."""
    p = {"wave_frequencies": [0.8, 1.5], "radiating_dofs": ["Heave"]}
    for q in range(4):
        body = mh.FloatingBody(mh.hemisphere_mesh(1.0 + 0.3 * q, 5, 10), ["Heave"])
        out = mh.batch_hydrodynamic_coefficients([body], [p], ctx=ctx, rho=1025.0)
        ref = mh.hydrodynamic_coefficients(body, p, ctx=ctx, rho=1025.0)
        assert np.abs(out[0]["added_mass"] - ref["added_mass"]).max() <= 1e-12 * np.abs(ref["added_mass"]).max()
        for h in list(body.mesh._handles.values()):
            h.close()
        body.mesh._handles.clear()
