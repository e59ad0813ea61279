"""The assembly entry point that allocates no device memory.

Some callers cannot call cudaMalloc -- code running under a device-memory pool
that already owns the GPU (a Julia CUDA.jl session, a framework's caching
allocator) or code that must not allocate after start-up.  For them
mh_assemble_matrices_noalloc keeps its per-panel scratch in a fixed device array
(8192 panels) instead of allocating a workspace.  This checks it, called through
the C-ABI, against the allocating mh_assemble_matrices on calls in a row that
share that array: each case's mesh has fewer panels than the one before, so
records of the previous mesh lie right past the current mesh's records, and a
call that read past its own panels, or skipped rewriting them, would give S and
D that differ from the allocating path's.  The cases cover the direct and
indirect forms, with and without a fixed normal and the identity jump, and the
static-only, wave-only and mixed Green-function sets.

Kept in a file of its own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_SD = 1e-10  # the S, D parity bar of the other GPU tests


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _noalloc(mh, torch, mesh, k, gfs, direct, include_identity=True, fixed=None):
    L = mh.load_library()
    n = mesh.nfaces
    V, C, N = _dev(torch, mesh.panel_vertices), _dev(torch, mesh.centers), _dev(torch, mesh.normals)
    A, R = _dev(torch, mesh.areas), _dev(torch, mesh.radii)
    S = torch.empty((n * n * 2,), dtype=torch.float64, device="cuda")
    D = torch.empty_like(S)
    fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.float64)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.mh_assemble_matrices_noalloc(stream, n, V.data_ptr(), C.data_ptr(), N.data_ptr(), A.data_ptr(),
                                        R.data_ptr(), float(k), int(gfs), int(direct), int(include_identity),
                                        fx.ctypes.data if fx is not None else None, S.data_ptr(), D.data_ptr())
    assert rc == 0, rc
    torch.cuda.current_stream().synchronize()
    to_c = lambda t: t.cpu().numpy().view(np.complex128).reshape((n, n), order="F")
    return to_c(S), to_c(D)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_noalloc_matches_allocating_entry_point_twice(mh, ctx):
    torch = pytest.importorskip("torch")
    wu = mh.default_greens_functions("Wu")
    rankine_neg = (mh.Rankine(), mh.RankineReflectedNegative())
    wave_only = (mh.GFWu(),)
    # (mesh, k, gfs, direct, include_identity, fixed normal); panel counts decrease
    cases = [(mh.config1_hemisphere(), 1.03 ** 2 / 9.81, wu, True, True, None),                       # 200
             (mh.vertical_cylinder_mesh(2.0, 3.0, 12, 5, 3), 0.8, wu, False, True, [1.0, 0.0, 0.0]),  # 96
             (mh.hemisphere_mesh(1.5, 5, 16), 0.5, wu, False, True, None),                             # 80
             (mh.vertical_cylinder_mesh(1.0, 2.0, 10, 4, 2), 1.7, rankine_neg, True, False, None),    # 60
             (mh.hemisphere_mesh(0.8, 3, 12), 2.2, wave_only, False, True, None),                      # 36
             (mh.hemisphere_mesh(0.8, 2, 10), 0.9, wave_only, True, False, [0.0, 0.0, 1.0])]          # 20
    sizes = [c[0].nfaces for c in cases]
    assert sizes == sorted(sizes, reverse=True) and len(set(sizes)) == len(sizes), sizes
    for mesh, k, gfs, direct, ident, fixed in cases:
        S, D = _noalloc(mh, torch, mesh, k, mh.gf_flags(gfs), direct, ident, fixed)
        S0, D0 = mh.assemble_matrices(gfs, mesh, k, direct=direct, include_identity=ident, all_normals=fixed,
                                      ctx=ctx)
        assert rel(S, S0) < REL_SD, (mesh.nfaces, direct)
        assert rel(D, D0) < REL_SD, (mesh.nfaces, direct)


def test_noalloc_rejects_oversize_and_unsupported(mh):
    L = mh.load_library()
    p = ctypes.c_void_p(8)  # never dereferenced: the size check comes first
    assert L.mh_assemble_matrices_noalloc(None, 8193, p, p, p, p, p, 1.0, 35, 1, 1, None, p, p) == 1
    assert L.mh_assemble_matrices_noalloc(None, 10, p, p, p, p, p, 1.0, 64 | 3, 1, 1, None, p, p) == 2
