"""The batched LU's launch-shape table and its autotuner (mh_tile_table_*, mh_autotune).

Launch shapes change the schedule, not the arithmetic: every output entry of the
trailing updates is computed the same way whatever the column tiles per CTA, and the
panel's rows are updated by the same operations whatever the cluster size, so solves
under any table agree with the default table to rounding (1e-13 here).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    B = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    return np.asfortranarray(A), np.asfortranarray(B)


def test_autotune_installs_a_table(mh, ctx):
    saved = ctx.tile_table()
    try:
        rep = mh.autotune(sizes=(160, 400), batch=4, precisions=("mixed", "fp64_tc"), reps=1, ctx=ctx)
        t = rep["table"]
        assert len(t) == 2
        assert t[0]["n_max"] == int(np.sqrt(160 * 400)) and t[1]["n_max"] is None
        for e in t:
            for k in ("ozaki_column_tiles", "bf16x3_column_tiles", "panel_cluster_fp64", "panel_cluster_fp32"):
                assert 1 <= e[k] <= 8
        for p in ("mixed", "fp64_tc"):
            tuned, dflt = np.array(rep["ms"][p]["tuned"]), np.array(rep["ms"][p]["default"])
            assert (tuned > 0).all() and (tuned <= dflt).all()
    finally:
        ctx.set_tile_table(saved)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_tc"])
def test_launch_shapes_do_not_change_results(mh, ctx, precision):
    saved = ctx.tile_table()
    A, B = _system(700, 3, 11)
    try:
        ctx.set_tile_table([])
        x0 = mh.linsolve(A, B, precision=precision, ctx=ctx)
        for shape in ((1, 1, 2, 2), (8, 8, 8, 8), (2, 2, 4, 4)):
            ctx.set_tile_table([(500,) + shape, (2 ** 63 - 1,) + shape])
            x = mh.linsolve(A, B, precision=precision, ctx=ctx)
            assert np.linalg.norm(x - x0) <= 1e-13 * np.linalg.norm(x0)
    finally:
        ctx.set_tile_table(saved)


def test_batch_graph_recaptures_under_a_new_table(mh, ctx):
    saved = ctx.tile_table()
    bodies = [mh.FloatingBody(mh.vertical_cylinder_mesh(1.0 + 0.5 * q, 2.0, 16 + 4 * q, 6, 4), ["Heave", "Pitch"])
              for q in range(3)]
    params = [{"wave_frequencies": [0.5, 1.0, 1.7], "radiating_dofs": ["Heave", "Pitch"]}] * 3
    try:
        F = mh.DirectBEM(precision="fp64_tc")
        ctx.set_tile_table([])
        r0 = mh.batch_hydrodynamic_coefficients(bodies, params, F, ctx=ctx)
        ctx.set_tile_table([(2 ** 63 - 1, 1, 1, 2, 2)])
        r1 = mh.batch_hydrodynamic_coefficients(bodies, params, F, ctx=ctx)
        for a, b in zip(r0, r1):
            assert np.abs(a["added_mass"] - b["added_mass"]).max() <= 1e-12 * np.abs(b["added_mass"]).max()
    finally:
        ctx.set_tile_table(saved)


def test_tile_table_rejects_bad_entries(mh, ctx):
    saved = ctx.tile_table()
    with pytest.raises(ValueError, match="ascending"):
        ctx.set_tile_table([(800, 4, 4, 8, 8), (400, 4, 4, 8, 8)])
    with pytest.raises(ValueError, match="outside 1..8"):
        ctx.set_tile_table([(800, 9, 4, 8, 8)])
    with pytest.raises(ValueError, match="orders must ascend"):
        ctx.autotune(0, [400, 200])
    assert ctx.tile_table() == saved


def test_shipped_tile_table_loads(mh, ctx):
    saved = ctx.tile_table()
    try:
        entries = mh.load_tile_table(ctx=ctx)
        assert ctx.tile_table() == [tuple(e) for e in entries] and len(entries) >= 1
    finally:
        ctx.set_tile_table(saved)
