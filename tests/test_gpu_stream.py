"""The bounded keyframe window of a long incremental run (the large-map
workload's mode, scaled down): frames of a seeded random walk stream in, each
is added, the view that leaves the window is retired (mrf_retire_view: its
messages stay in the log-odds, its lists and pairs are dropped) and
MRF_INCREMENTAL iterations run over the live window.  The loop of the
reference's viewer (src/Viewer.cpp:44-61: add_camera, then
perform_inference, for every keyframe) with consistent messages and a
window.

Compared with the FP64 oracle running the same loop (orc_retire_view):
beliefs within 1e-3 with >= 99.9 % class agreement along the stream, the
message-update count of the live window, and the total log-odds rebuilt from
the prior, the retired views' messages and the live ones."""
import ctypes as C

import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic
from oracle import oracle as O

pytestmark = pytest.mark.gpu

WINDOW = 4
ITERS = 5
N_FRAMES = 20


@pytest.fixture(scope="module")
def walk():
    w = synthetic.walk_room(7, n_frames=N_FRAMES, rows=120, cols=160, res=0.04, dims=(8.0, 8.0, 3.0),
                            n_boxes=30, step=0.15)
    return w, [synthetic.render_frame(w, k) for k in range(N_FRAMES)]


def _compare(gb, ob):
    gb = gb.astype(np.float64)
    touched = (gb > 0) | (ob > 0)
    return float(np.abs(gb - ob).max()), float(((gb > 0.5) == (ob > 0.5))[touched].mean())


def test_windowed_incremental_stream_matches_oracle(native_lib, oracle_lib, walk):
    w, depths = walk
    gm = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    om = O.OracleMap(w.params, threads=8)
    for k in range(N_FRAMES):
        gm.add_view(w.poses[k], depths[k])
        om.add_view(w.poses[k], depths[k], O.ACT_FULL_RAY)
        if k >= WINDOW:
            gm.retire_view(k - WINDOW)
            om.retire_view(k - WINDOW)
        gm.infer(iters=ITERS, flags=L.INCREMENTAL)
        om.infer(iters=ITERS, flags=O.INCREMENTAL)
        assert gm.num_bricks == om.num_bricks
        assert gm.stats()["n_inc_post"] * ITERS == om.last_updates  # the live window only
        if k in (WINDOW, N_FRAMES // 2, N_FRAMES - 1):
            emax, agree = _compare(gm.beliefs(), om.beliefs())
            assert emax <= 1e-3, f"frame {k}: max belief error {emax}"
            assert agree >= 0.999, f"frame {k}: class agreement {agree}"
    # the total log-odds is the prior + retired views' messages + live ones
    lo = gm.logodds()
    gm.rebuild_logodds()
    np.testing.assert_allclose(gm.logodds(), lo, rtol=0, atol=2e-4)
    np.testing.assert_allclose(lo, om.logodds(), rtol=1e-3, atol=1e-2)
    gm.close()
    om.close()


def test_retired_views_refuse_per_view_calls(native_lib, walk):
    w, depths = walk
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for k in range(3):
        m.add_view(w.poses[k], depths[k])
    m.infer(iters=2, flags=L.INCREMENTAL)
    m.retire_view(0)
    m.retire_view(0)  # again: nothing to do
    for call in (lambda: m.likelihood_view(0), lambda: m.read_messages(0), lambda: m.view_incidences(0),
                 lambda: m.set_pose(0, w.poses[0])):
        with pytest.raises(L.MrfError) as e:
            call()
        assert e.value.status == 6  # MRF_ERR_STATE
    m.infer(iters=2, flags=L.INCREMENTAL)
    s, img = m.likelihood_view(1)
    assert np.isfinite(s) and img.shape == depths[1].shape
    st = m.stats()
    assert st["n_views"] == 3
    m.close()


def test_appended_lists_equal_a_full_build(native_lib, walk):
    """Frames added one at a time to a full-ray map, each followed by a build,
    append only the new view's lists; they are those a single build of all
    the views gives, bit for bit, and BP from the prior reaches the same
    beliefs within 1e-5 (from the third iteration the ray kernel sums each
    static prefix as a quiet part and a loud part, and an appended view
    whose quiet pair turned loud counts all its pairs as loud until the
    next full build, so the two maps round those sums differently).  After retiring a view and appending more, a Jacobi run (which
    needs the all-view structures: a full build first) matches a map built
    directly from the live views."""
    w, depths = walk
    a = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for k in range(8):
        a.add_view(w.poses[k], depths[k])
        a.infer(iters=1, flags=L.INCREMENTAL)
    st = a.stats()
    assert st["builds_appended"] == 7 and st["builds_full"] == 1
    b = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for k in range(8):
        b.add_view(w.poses[k], depths[k])
    b.infer(iters=1)
    np.testing.assert_array_equal(a.brick_coords(), b.brick_coords())
    for v in range(8):
        for x, y in zip(a.view_incidences(v), b.view_incidences(v)):
            np.testing.assert_array_equal(x, y)
    assert a.stats()["n_inc_post"] == b.stats()["n_inc_post"]
    a.reset_state()
    b.reset_state()
    a.infer(iters=5)
    b.infer(iters=5)
    np.testing.assert_allclose(a.beliefs(), b.beliefs(), rtol=0, atol=1e-5)
    # a window step: retire, append, then Jacobi
    a.retire_view(0)
    for k in (8, 9):
        a.add_view(w.poses[k], depths[k])
        a.infer(iters=1, flags=L.INCREMENTAL)
    assert a.stats()["builds_appended"] == 9
    c = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for k in range(10):
        c.add_view(w.poses[k], depths[k])
    c.retire_view(0)
    a.reset_state()
    c.reset_state()
    a.infer(iters=4, flags=L.JACOBI)
    c.infer(iters=4, flags=L.JACOBI)
    assert a.stats()["builds_full"] == 2
    np.testing.assert_array_equal(a.brick_coords(), c.brick_coords())
    np.testing.assert_allclose(a.beliefs(), c.beliefs(), rtol=0, atol=1e-6)
    for m in (a, b, c):
        m.close()


def test_brick_footprint_covers_every_crossing_ray(native_lib, walk):
    """After bricks are activated, an appended build re-traces only the
    pixels of each old view whose rays may cross one of the new bricks (the
    bricks' projected footprint).  Every pixel whose incidence list holds a
    voxel of a brick in the range must be in that footprint: checked
    against the oracle's own lists for every view, over slices of the
    brick range."""
    w, depths = walk
    nv = 4
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    om = O.OracleMap(w.params, threads=8)
    for k in range(nv):
        m.add_view(w.poses[k], depths[k])
        om.add_view(w.poses[k], depths[k], O.ACT_FULL_RAY)
    m.infer(iters=1)
    om.build_all()
    nb = m.num_bricks
    assert nb == om.num_bricks
    lib = L.load()
    rows, cols = w.params.rows, w.params.cols
    checked = 0
    for v in range(nv):
        tr = om.view_trace(v)
        pix, off, meta, vox = tr["pix"], tr["off"], tr["meta"], tr["vox"]
        for b0, b1 in ((0, nb // 3), (nb // 3, 2 * nb // 3), (2 * nb // 3, nb), (nb - 5, nb)):
            mask = np.zeros(rows * cols, np.uint8)
            allf = C.c_int(0)
            assert lib.mrf_test_brick_footprint(m.handle, v, b0, b1,
                                                mask.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(allf)) == 0
            if allf.value:
                continue
            for r in range(len(pix)):
                n = meta[r, 0]
                if n == 0:
                    continue
                bricks = vox[off[r]:off[r] + n] // 512
                if np.any((bricks >= b0) & (bricks < b1)):
                    assert mask[pix[r]] == 1, (v, r, b0, b1)
                    checked += 1
    assert checked > 0
    m.close()
    om.close()


def test_failed_append_falls_back_to_a_full_build(native_lib, oracle_lib, walk):
    """A build that appends a new view's lists and fails part-way (injected
    on the host, mrf_test_fail_next_append, once the new view's pairs are
    built): out of device memory, the same call makes a full build instead
    (which drops the retired views' lists); any other failure fails the call
    and the next call's build is a full one.  The messages carried into the
    full build are the built views' only, so both streams go on to the
    oracle's beliefs, identical to each other and within 1e-4 of a stream
    that appended throughout (a full and an appended build round the static
    prefixes' sums differently)."""
    w, depths = walk
    lib = L.load()
    n = 14
    # the frames whose build appends (a build is a full one when new bricks
    # change an older view's rays): the same stream, run once beforehand
    # (the stats are read after each frame's infer only: reading them builds
    # the lists of views added since the last build)
    probe = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    appends, count = [], 0
    for k in range(n):
        probe.add_view(w.poses[k], depths[k])
        if k >= WINDOW:
            probe.retire_view(k - WINDOW)
        probe.infer(iters=ITERS, flags=L.INCREMENTAL)
        if probe.stats()["builds_appended"] > count:
            appends.append(k)
        count = probe.stats()["builds_appended"]
    probe.close()
    later = [k for k in appends if k > WINDOW]  # with retired views' lists in the arenas
    assert later, f"no appended build after frame {WINDOW}: {appends}"
    fail_at = later[0]
    om = O.OracleMap(w.params, threads=8)
    maps = {name: L.MRFMap(w.params, activation=L.ACT_FULL_RAY) for name in ("plain", "oom", "cuda")}
    last = {}
    for k in range(n):
        om.add_view(w.poses[k], depths[k], O.ACT_FULL_RAY)
        for m in maps.values():
            m.add_view(w.poses[k], depths[k])
        if k >= WINDOW:
            om.retire_view(k - WINDOW)
            for m in maps.values():
                m.retire_view(k - WINDOW)
        om.infer(iters=ITERS, flags=O.INCREMENTAL)
        if k == fail_at:
            before = last
            assert lib.mrf_test_fail_next_append(maps["oom"].handle, 3) == 0   # MRF_ERR_OOM
            assert lib.mrf_test_fail_next_append(maps["cuda"].handle, 2) == 0  # MRF_ERR_CUDA
            maps["oom"].infer(iters=ITERS, flags=L.INCREMENTAL)
            st = maps["oom"].stats()
            assert st["builds_oom_fallback"] == 1
            assert st["builds_full"] == before["oom"]["builds_full"] + 1
            with pytest.raises(L.MrfError, match="MRF_ERR_CUDA"):
                maps["cuda"].infer(iters=ITERS, flags=L.INCREMENTAL)
            maps["cuda"].infer(iters=ITERS, flags=L.INCREMENTAL)
            st = maps["cuda"].stats()
            assert st["builds_oom_fallback"] == 0
            assert st["builds_full"] == before["cuda"]["builds_full"] + 1
            maps["plain"].infer(iters=ITERS, flags=L.INCREMENTAL)
        else:
            for m in maps.values():
                m.infer(iters=ITERS, flags=L.INCREMENTAL)
        last = {name: m.stats() for name, m in maps.items()}
        if k in (fail_at, n - 1):
            ob = om.beliefs()
            bel = {name: m.beliefs() for name, m in maps.items()}
            for name, gb in bel.items():
                emax, agree = _compare(gb, ob)
                assert emax <= 1e-3, f"{name}, frame {k}: max belief error {emax}"
                assert agree >= 0.999, f"{name}, frame {k}: class agreement {agree}"
            np.testing.assert_array_equal(bel["oom"], bel["cuda"])
            np.testing.assert_allclose(bel["oom"], bel["plain"], rtol=0, atol=1e-4)
    assert maps["plain"].stats()["builds_oom_fallback"] == 0
    for m in maps.values():
        m.close()
    om.close()


def test_quiet_prefix_on_appended_lists(native_lib, oracle_lib, walk):
    """The static prefixes taken from their quiet sums (forced,
    MRF_QUIET_PREFIX) on lists built by appending one view at a time: an
    older view whose quiet pair turned loud when a later view was appended
    counts all its pairs as loud, so the fast path and the full ray path
    (MRF_FULL_RAYS) on the same lists agree to FP32 rounding of the
    regrouped prefix sums (within 5e-5: 1.1e-5 at one voxel of 457,216
    after 6 iterations, the rest within 1e-5), and both agree with the
    oracle within 1e-3 at >= 99.9 % class agreement."""
    w, depths = walk
    n = 8
    om = O.OracleMap(w.params, threads=8)
    for k in range(n):
        om.add_view(w.poses[k], depths[k], O.ACT_FULL_RAY)
    om.infer(iters=ITERS + 1)
    ob = om.beliefs()
    om.close()
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for k in range(n):
        m.add_view(w.poses[k], depths[k])
        m.infer(iters=1, flags=L.INCREMENTAL)  # one build per view: appended
    assert m.stats()["builds_appended"] == n - 1
    out = {}
    for name, extra in (("fast", L.QUIET_PREFIX), ("full", L.FULL_RAYS)):
        m.reset_state()
        m.infer(iters=ITERS + 1, flags=extra)
        st = m.stats()
        assert st["quiet_prefix_used"] == (1 if name == "fast" else 0)
        assert st["builds_appended"] == n - 1 and st["builds_full"] == 1  # the same lists for both
        emax, agree = _compare(m.beliefs(), ob)
        assert emax <= 1e-3, f"{name}: max belief error {emax}"
        assert agree >= 0.999, f"{name}: class agreement {agree}"
        out[name] = m.beliefs()
    np.testing.assert_allclose(out["fast"], out["full"], rtol=0, atol=5e-5)
    assert (np.abs(out["fast"] - out["full"]) > 1e-5).sum() <= 10
    m.close()
