"""Edge cases of the sweep through the C-ABI: the smallest meshes, one-sided problem sets,
a one-body one-frequency batch, and orders beyond the supported maximum.  Bars as in the
parity tests (coefficients 1e-8 of the oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def close(a, b, rel=1e-8):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() <= rel * max(np.abs(b).max(), 1e-300)


def _one_panel(mh):
    V = np.array([(-0.5, -0.5, -1.0), (0.5, -0.5, -1.0), (0.5, 0.5, -1.0), (-0.5, 0.5, -1.0)])
    return mh.StaticArraysMesh(V, [(1, 4, 3, 2)])  # normal -z


@pytest.mark.parametrize("direct", [True, False])
def test_one_and_two_panel_meshes(mh, oracle, ctx, direct):
    for mesh in (_one_panel(mh), mh.tiny_static_mesh()):
        body = mh.FloatingBody(mesh, ["Heave", "Surge"])
        F = mh.DirectBEM() if direct else mh.IndirectBEM()
        res = mh.hydrodynamic_coefficients(body, {"wave_frequencies": [0.7, 2.0], "radiating_dofs": ["Heave"],
                                                  "wave_directions": [0.0]}, F, ctx=ctx, rho=1025.0)
        for w, om in enumerate((0.7, 2.0)):
            A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(mesh, body.dofs, om, rho=1025.0, direct=direct,
                                                          radiating=["Heave"], betas=[0.0])
            assert close(res["added_mass"][:, :, w, 0], A)
            assert close(res["radiation_damping"][:, :, w, 0], B)
            assert close(res["excitation_force"][:, w, :, 0], Fe)


def test_one_sided_problem_sets(mh, oracle, ctx):
    mesh = mh.hemisphere_mesh(1.0, 5, 10)
    body = mh.FloatingBody(mesh, ["Heave", "Pitch"])
    only_dif = mh.hydrodynamic_coefficients(body, {"wave_frequencies": [1.2], "wave_directions": [0.0, 1.0]},
                                            ctx=ctx, rho=1025.0)
    assert only_dif["added_mass"].size == 0 and only_dif["excitation_force"].shape == (2, 1, 2, 1)
    only_rad = mh.hydrodynamic_coefficients(body, {"wave_frequencies": [1.2], "radiating_dofs": ["Pitch"]},
                                            ctx=ctx, rho=1025.0)
    assert only_rad["excitation_force"].size == 0 and only_rad["added_mass"].shape == (2, 1, 1, 1)
    A, B, Fd, Fk, Fe = oracle.hydro_one_frequency(mesh, body.dofs, 1.2, rho=1025.0, radiating=["Pitch"],
                                                  betas=[0.0, 1.0])
    assert close(only_rad["added_mass"][..., 0, 0], A)
    assert close(only_dif["excitation_force"][:, 0, :, 0], Fe)
    with pytest.raises(ValueError, match="nothing to solve"):
        mh.hydrodynamic_coefficients(body, {"wave_frequencies": [1.2]}, ctx=ctx)


def test_one_body_one_frequency_batch(mh, ctx):
    body = mh.FloatingBody(mh.hemisphere_mesh(1.0, 5, 10), ["Heave"])
    p = {"wave_frequencies": [0.9], "radiating_dofs": ["Heave"], "wave_directions": [0.0]}
    out = mh.batch_hydrodynamic_coefficients([body], [p], ctx=ctx, rho=1025.0)
    ref = mh.hydrodynamic_coefficients(body, p, ctx=ctx, rho=1025.0)
    for key in ("added_mass", "radiation_damping", "excitation_force"):
        assert close(out[0][key], ref[key], 1e-12)


def test_orders_beyond_the_maximum_are_rejected_before_device_work(mh, ctx):
    # a 12001-panel mesh uploads, but its sweep is refused as unsupported
    k = 12001
    V = np.zeros((4 * k, 3))
    V[0::4] = np.c_[np.arange(k), np.zeros(k), -np.ones(k)]
    V[1::4] = V[0::4] + [1.0, 0.0, 0.0]
    V[2::4] = V[0::4] + [1.0, 1.0, 0.0]
    V[3::4] = V[0::4] + [0.0, 1.0, 0.0]
    mesh = mh.StaticArraysMesh(V, np.arange(4 * k).reshape(k, 4) + 1)
    body = mh.FloatingBody(mesh, ["Heave"])
    with pytest.raises(ValueError, match="exceeds the supported"):
        mh.hydrodynamic_coefficients(body, {"wave_frequencies": [1.0], "radiating_dofs": ["Heave"]}, ctx=ctx)
