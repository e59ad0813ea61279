"""Device-memory buffers through the C-ABI (MH_MEM_DEVICE) -- the reference's
`arrtype = CuArray` path (matrix_assembly.jl:167-175, 418-434; test/gpu.jl): meshes built
from device arrays, matrices, solves and the sweep written to device buffers (torch CUDA
tensors here), compared with the host-buffer calls of the same entry points."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def test_mesh_assembly_and_solves_in_device_memory(mh, ctx):
    L = ctx._L
    MEM_DEV = 1
    mesh = mh.hemisphere_mesh(1.0, 6, 12)
    n = mesh.nfaces
    V, C, N, A, R = (_dev(x) for x in (mesh.panel_vertices, mesh.centers, mesh.normals, mesh.areas, mesh.radii))
    dm = mh.api._device.DeviceMesh.from_device_arrays(ctx, n, V, C, N, A, R)
    k = 1.3 ** 2 / 9.81
    gfs = mh.gf_flags(mh.default_greens_functions("Wu"))
    S_ref, D_ref = mh.assemble_matrices(mh.default_greens_functions("Wu"), mesh, k, ctx=ctx)
    S = torch.empty((n, n, 2), dtype=torch.float64, device="cuda")  # column-major complex: transpose below
    D = torch.empty_like(S)
    ctx.check(L.mh_assemble_matrices(ctx.handle, dm.handle, k, gfs, 1, 1, None, S.data_ptr(), D.data_ptr(), MEM_DEV),
              "assemble (device)")
    to_np = lambda t: (t[..., 0] + 1j * t[..., 1]).cpu().numpy().T  # (j, i) storage -> (i, j)
    assert np.array_equal(to_np(S), S_ref) and np.array_equal(to_np(D), D_ref)

    # linsolve and solve(D, S, bc) with device operands
    rng = np.random.default_rng(4)
    B = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    X_ref = mh.linsolve(D_ref, B, ctx=ctx)
    cm = lambda M: torch.view_as_real(torch.from_numpy(np.asfortranarray(M).T.copy())).to("cuda")  # column-major
    X = torch.empty((3, n, 2), dtype=torch.float64, device="cuda")
    ctx.check(L.mh_linsolve(ctx.handle, n, 3, D.data_ptr(), cm(B).data_ptr(), X.data_ptr(), 0, MEM_DEV), "linsolve")
    assert np.abs(to_np(X) - X_ref).max() <= 1e-13 * np.abs(X_ref).max()
    phi_ref, _ = mh.solve_linear(D_ref, S_ref, B, ctx=ctx)
    phi = torch.empty((3, n, 2), dtype=torch.float64, device="cuda")
    ctx.check(L.mh_solve(ctx.handle, n, 3, D.data_ptr(), S.data_ptr(), cm(B).data_ptr(), 1, phi.data_ptr(), None, 0,
                         MEM_DEV), "solve")
    assert np.abs(to_np(phi) - phi_ref).max() <= 1e-13 * np.abs(phi_ref).max()


def test_sweep_with_device_dofs_and_outputs(mh, ctx):
    L = ctx._L
    mesh = mh.hemisphere_mesh(1.0, 6, 12)
    body = mh.FloatingBody(mesh, ["Heave", "Surge"])
    oms = np.array([0.6, 1.4, 2.2])
    betas = np.array([0.0, 0.8])
    params = {"wave_frequencies": oms, "radiating_dofs": ["Heave", "Surge"], "wave_directions": betas}
    ref = mh.hydrodynamic_coefficients(body, params, ctx=ctx, rho=1025.0)
    dofs = _dev(body.dof_array(["Heave", "Surge"]))
    idx = np.array([0, 1], dtype=np.int32)
    outs = [torch.empty(2 * 2 * 3, dtype=torch.float64, device="cuda") for _ in range(2)] + \
           [torch.empty(2 * 3 * 2 * 2, dtype=torch.float64, device="cuda") for _ in range(3)]
    gfs = mh.gf_flags(mh.default_greens_functions("Wu"))
    ctx.check(L.mh_hydrodynamic_coefficients(ctx.handle, mesh.device_mesh(ctx).handle, 3, oms.ctypes.data, 1025.0,
                                             9.81, gfs, 1, 2, dofs.data_ptr(), 2, idx.ctypes.data, 2, idx.ctypes.data,
                                             2, betas.ctypes.data, 0, *[o.data_ptr() for o in outs], 1), "sweep")
    A = outs[0].cpu().numpy().reshape((2, 2, 3), order="F")
    Fe = outs[4].cpu().numpy().view(np.complex128).reshape((2, 3, 2), order="F")
    assert np.array_equal(A, ref["added_mass"][..., 0])
    assert np.array_equal(Fe, ref["excitation_force"][..., 0])
