"""Several scenes in one map (the batched workload, reduced): each view is
confined to its scene's brick box (mrf_add_view_box), so the scenes share
the brick pool, the incidence and pair arrays and the BP launches -- one
Jacobi ray launch runs every ray of every scene -- without seeing one
another.  Checked against the FP64 oracle holding the same boxed views:
bricks and incidence lists bit-exact, every incidence inside its view's box,
beliefs within 1e-3 with >= 99.9 % class agreement (Jacobi and
Gauss-Seidel); and each scene's beliefs equal those of a map that holds
that scene alone."""
import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    b = synthetic.batch_scenes(11, n_scenes=3, views_per_scene=5, sizes=((60, 80), (120, 160)),
                               size_cycle=(0, 1), res=0.04, n_boxes=6, room_range=(3.0, 6.0))
    return b, [synthetic.render_batch_view(b, k) for k in range(len(b.poses))]


def _add(m, b, depths, views, oracle=False):
    for k in views:
        rows, cols, fx, fy, cx, cy = b.cams[k]
        lo, hi = b.boxes[b.scene_of[k]]
        if oracle:
            m.add_view_box(b.poses[k], depths[k], rows, cols, fx, fy, cx, cy, lo, hi, O.ACT_FULL_RAY)
        else:
            m.add_view_box(b.poses[k], depths[k], fx, fy, cx, cy, lo, hi)


def test_boxes_bit_exact_and_isolated(native_lib, oracle_lib, batch):
    b, depths = batch
    gm = L.MRFMap(b.params, activation=L.ACT_FULL_RAY)
    om = O.OracleMap(b.params, threads=8)
    _add(gm, b, depths, range(len(b.poses)))
    _add(om, b, depths, range(len(b.poses)), oracle=True)
    assert gm.num_bricks == om.num_bricks
    coords = gm.brick_coords()
    np.testing.assert_array_equal(coords, om.brick_coords())
    for v in range(len(b.poses)):
        meta, vox, ln, mu = gm.view_incidences(v)
        t = om.view_trace(v)
        ometa = np.zeros((depths[v].size, 5), np.int32)
        ometa[t["pix"]] = t["meta"]
        np.testing.assert_array_equal(meta, ometa)
        np.testing.assert_array_equal(vox.astype(np.int64), t["vox"].astype(np.int64))
        np.testing.assert_array_equal(ln.view(np.uint32), t["len"].view(np.uint32))
        lo, hi = (np.array(x) for x in b.boxes[b.scene_of[v]])
        bc = coords[vox.astype(np.int64) // 512]
        assert np.all((bc >= lo) & (bc < hi)), f"view {v} leaves its scene box"
    # every active brick lies in some scene box
    inside = np.zeros(len(coords), bool)
    for lo, hi in b.boxes:
        inside |= np.all((coords >= np.array(lo)) & (coords < np.array(hi)), axis=1)
    assert inside.all()
    gm.close()
    om.close()


@pytest.mark.parametrize("flags", [L.JACOBI, 0], ids=["jacobi", "gauss-seidel"])
def test_batched_beliefs(native_lib, oracle_lib, batch, flags):
    b, depths = batch
    gm = L.MRFMap(b.params, activation=L.ACT_FULL_RAY)
    om = O.OracleMap(b.params, threads=8)
    _add(gm, b, depths, range(len(b.poses)))
    _add(om, b, depths, range(len(b.poses)), oracle=True)
    gm.infer(iters=10, flags=flags)
    om.infer(iters=10, flags=O.JACOBI if flags else 0)
    gb, ob = gm.beliefs().astype(np.float64), om.beliefs()
    touched = (gb > 0) | (ob > 0)
    assert np.abs(gb - ob).max() <= 1e-3
    assert ((gb > 0.5) == (ob > 0.5))[touched].mean() >= 0.999
    # each scene alone in its own map: the same beliefs
    coords = {tuple(c): i for i, c in enumerate(gm.brick_coords())}
    for s in range(len(b.boxes)):
        views = [k for k in range(len(b.poses)) if b.scene_of[k] == s]
        sm = L.MRFMap(b.params, activation=L.ACT_FULL_RAY)
        _add(sm, b, depths, views)
        sm.infer(iters=10, flags=flags)
        sb = sm.beliefs()
        idx = [coords[tuple(c)] for c in sm.brick_coords()]
        np.testing.assert_allclose(gm.beliefs()[idx], sb, rtol=0, atol=1e-5)
        sm.close()
    gm.close()
    om.close()


def test_box_arguments_checked(native_lib, batch):
    b, depths = batch
    m = L.MRFMap(b.params, activation=L.ACT_FULL_RAY)
    rows, cols, fx, fy, cx, cy = b.cams[0]
    for lo, hi in (([0, 0, 0], [0, 5, 5]), ([-1, 0, 0], [4, 4, 4]), ([0, 0, 0], [10 ** 6, 4, 4])):
        with pytest.raises(L.MrfError) as e:
            m.add_view_box(b.poses[0], depths[0], fx, fy, cx, cy, lo, hi)
        assert e.value.status == 1
    m.close()
