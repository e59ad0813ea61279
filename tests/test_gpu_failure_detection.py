"""Failure detection without a GPU fault.

Every completion wait of the tensor-core kernels polls an mbarrier a bounded number of
times; when it gives up the kernel records a timeout, drains what it has in flight, frees
its tensor memory and returns, and the host reports MH_ERR_TIMEOUT.  The probe runs that
path on purpose (a wait that nothing satisfies); the context must stay usable after it.
Bad inputs (NaN meshes, singular matrices) come back as status codes, never as faults.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives(mh, ctx):
    for polls in (1, 64, 1024):
        with pytest.raises(mh.MarineHydroError, match="gave up after"):
            ctx.check(ctx._L.mh_probe_wait_timeout(ctx.handle, polls), "wait probe")
    with pytest.raises(ValueError, match="polls"):
        ctx.check(ctx._L.mh_probe_wait_timeout(ctx.handle, 0), "wait probe")
    # the context and the tensor cores still work: a tensor-core factorization afterwards
    rng = np.random.default_rng(3)
    A = rng.standard_normal((300, 300)) + 1j * rng.standard_normal((300, 300))
    b = rng.standard_normal(300) + 0j
    x = mh.linsolve(A, b, precision="fp64_tc", ctx=ctx)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)


def test_non_finite_mesh_is_rejected(mh, ctx):
    mesh = mh.hemisphere_mesh(1.0, 4, 8)
    for field in ("centers", "areas", "radii"):
        bad = mh.StaticArraysMesh(mesh.vertices, mesh.faces, mesh.centers.copy(), mesh.normals, mesh.areas.copy(),
                                  mesh.radii.copy())
        getattr(bad, field).reshape(-1)[3] = np.nan if field != "areas" else np.inf
        with pytest.raises(ValueError, match="not finite"):
            mh.assemble_matrix_wu(bad, 1.0, ctx=ctx)


def test_singular_system_is_a_status(mh, ctx):
    A = np.ones((40, 40), dtype=complex)
    with pytest.raises(np.linalg.LinAlgError):
        mh.linsolve(A, np.ones(40, dtype=complex), ctx=ctx)
    # and the context goes on
    x = mh.linsolve(np.eye(40, dtype=complex) * 2, np.ones(40, dtype=complex), ctx=ctx)
    assert np.allclose(x, 0.5)
