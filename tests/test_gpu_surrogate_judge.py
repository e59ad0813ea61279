"""The exact path judges every surrogate result (mh_surrogate_set_judge).

Each frequency's surrogate-assembled S and D are checked against the exact
Guevel-Delhommeau term on sampled panel pairs; a frequency whose sampled relative error
exceeds the tolerance is solved with the exact term.  Checked: a tolerance above every
estimate leaves the surrogate results, a zero tolerance re-runs every frequency and
reproduces the exact-term sweep, an intermediate one re-runs exactly the flagged
frequencies, the batch does the same, and the estimate tracks the coefficients' actual
error against the exact term.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OMS = [0.5, 1.2, 2.4, 3.3]
KEYS = ("added_mass", "radiation_damping", "excitation_force")


def _setup(mh, ctx):
    mh.load_surrogate(ctx=ctx)
    mesh = mh.barge_mesh(8.0, 3.0, 1.5, 12, 4, 3)
    body = mh.FloatingBody(mesh, ["Heave", "Pitch"], rotation_center=(0.0, 0.0, 0.0), body_name="barge")
    params = {"wave_frequencies": OMS, "radiating_dofs": ["Heave", "Pitch"], "wave_directions": [0.0, 0.8]}
    return body, params


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def _per_omega(res, key, w):
    a = res[key]
    return a[:, :, w] if key != "excitation_force" else a[:, w]


def test_judge_keeps_or_reruns_each_frequency(mh, ctx):
    body, params = _setup(mh, ctx)
    FS = mh.DirectBEM("Surrogate", precision="fp64")
    FE = mh.DirectBEM("ExactGuevelDelhommeau", precision="fp64")
    try:
        mh.set_surrogate_judge(0, ctx=ctx)
        plain = mh.hydrodynamic_coefficients(body, params, FS, ctx=ctx, rho=1025.0)
        assert "surrogate_judge" not in plain
        exact = mh.hydrodynamic_coefficients(body, params, FE, ctx=ctx, rho=1025.0)
        # a tolerance above every estimate: the surrogate results stand
        mh.set_surrogate_judge(2048, tolerance=1.0, ctx=ctx)
        kept = mh.hydrodynamic_coefficients(body, params, FS, ctx=ctx, rho=1025.0)
        est = kept["surrogate_judge"]["estimate"]
        assert not kept["surrogate_judge"]["rerun"].any()
        assert np.all(est > 0) and np.all(est < 0.1), est
        for k in KEYS:
            assert _rel(kept[k], plain[k]) < 1e-12, k
        # the estimate follows the actual error of the coefficients against the exact term
        for w in range(len(OMS)):
            actual = max(_rel(_per_omega(plain, k, w), _per_omega(exact, k, w)) for k in KEYS)
            print(f"omega {OMS[w]}: estimate {est[w]:.2e}, actual coefficient error {actual:.2e}")
            assert actual <= 30 * est[w], (w, actual, est[w])
        # zero tolerance: every frequency goes through the exact term
        mh.set_surrogate_judge(2048, tolerance=0.0, ctx=ctx)
        redo = mh.hydrodynamic_coefficients(body, params, FS, ctx=ctx, rho=1025.0)
        assert redo["surrogate_judge"]["rerun"].all()
        for k in KEYS:
            assert _rel(redo[k], exact[k]) < 1e-10, k
        # in between: exactly the flagged frequencies are re-run
        tol = float(np.sort(est)[len(est) // 2 - 1]) * (1 + 1e-9)
        mh.set_surrogate_judge(2048, tolerance=tol, ctx=ctx)
        mix = mh.hydrodynamic_coefficients(body, params, FS, ctx=ctx, rho=1025.0)
        flags = mix["surrogate_judge"]["rerun"]
        assert np.array_equal(flags, est > tol) and 0 < flags.sum() < len(OMS)
        for w in range(len(OMS)):
            ref = exact if flags[w] else plain
            for k in KEYS:
                assert _rel(_per_omega(mix, k, w), _per_omega(ref, k, w)) < 1e-10, (w, k)
    finally:
        mh.set_surrogate_judge(0, ctx=ctx)


def test_batch_judge_reruns_flagged_frequency_solves(mh, ctx):
    body, params = _setup(mh, ctx)
    other = mh.FloatingBody(mh.vertical_cylinder_mesh(1.5, 2.0, 14, 5, 3), ["Heave", "Pitch"],
                            rotation_center=(0.0, 0.0, 0.0), body_name="cyl")
    bodies = [body, other]
    plist = [params, dict(params, wave_frequencies=[0.9, 2.0])]
    FS = mh.DirectBEM("Surrogate", precision="fp64")
    FE = mh.DirectBEM("ExactGuevelDelhommeau", precision="fp64")
    try:
        mh.set_surrogate_judge(1024, tolerance=0.0, ctx=ctx)
        out = mh.batch_hydrodynamic_coefficients(bodies, plist, FS, ctx=ctx, rho=1025.0)
        ctx._L.mh_batch_release(ctx.handle)
        mh.set_surrogate_judge(0, ctx=ctx)
        for b, p, o in zip(bodies, plist, out):
            assert o["surrogate_judge"]["rerun"].all()
            assert o["surrogate_judge"]["estimate"].shape == (len(p["wave_frequencies"]),)
            ref = mh.hydrodynamic_coefficients(b, p, FE, ctx=ctx, rho=1025.0)
            for k in KEYS:
                assert _rel(o[k], ref[k]) < 1e-10, k
        mh.set_surrogate_judge(1024, tolerance=1.0, ctx=ctx)
        kept = mh.batch_hydrodynamic_coefficients(bodies, plist, FS, ctx=ctx, rho=1025.0)
        ctx._L.mh_batch_release(ctx.handle)
        assert not any(o["surrogate_judge"]["rerun"].any() for o in kept)
    finally:
        mh.set_surrogate_judge(0, ctx=ctx)
