"""The drop-in boundary on the GPU: the reference's Python module names
(GVDBPyModules), the C++ shim behind it, and the C ABI's error behaviour."""
import os
import sys

import numpy as np
import pytest

from mrfmap_gb300 import _build
from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G(native_lib):
    path = _build.build_pymodule()
    sys.path.insert(0, os.path.dirname(path))
    import GVDBPyModules
    return GVDBPyModules


@pytest.fixture(scope="module")
def w():
    return synthetic.small_room(3, n_frames=3, rows=60, cols=80)


def _set_global_params(G, p):
    gp = G.gvdb_params()
    gp.res, gp.prior, gp.rows, gp.cols = p.res, p.prior, p.rows, p.cols
    gp.dims = list(p.dims)
    gp.K = p.K
    gp.max_iters = p.max_iters
    gp.lookup_n = 3
    gp.const_sigmasq_poly = list(p.const_sigmasq_poly)
    gp.populate_lookup_tables()
    gp.set_from_python()
    return gp


def test_python_module_matches_c_abi(G, w):
    _set_global_params(G, w.params)
    inf = G.GVDBInference(True, False)
    for P, D in zip(w.poses, w.depths):
        inf.add_camera_with_depth(P, D)
    inf.perform_inference()
    bricks = inf.get_occupied_bricks(0)
    alphas = np.zeros((len(bricks), 512), np.float32)
    inf.get_indices_and_alphas(alphas)
    img = np.zeros((w.params.rows, w.params.cols), np.float32)
    s = inf.get_likelihood_image(1, img)

    m = L.MRFMap(w.params)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer()
    cen, bel = m.read_bricks()
    np.testing.assert_array_equal(bricks, cen)
    np.testing.assert_array_equal(alphas, bel)
    s2, img2 = m.likelihood_view(1)
    np.testing.assert_array_equal(img, img2)
    assert s == s2
    assert s == pytest.approx(inf.compute_likelihood(1))
    # GVDBImage + add_camera path and likelihood at an arbitrary pose
    im = G.GVDBImage(w.depths[0])
    img3 = np.zeros_like(img)
    s3 = inf.get_likelihood_image_at_pose(w.poses[0], im, img3)
    s4, img4 = m.likelihood(w.poses[0], w.depths[0])
    np.testing.assert_array_equal(img3, img4)
    assert s3 == s4


def test_wrong_readback_shape_raises(G, w):
    _set_global_params(G, w.params)
    inf = G.GVDBInference(True, False)
    inf.add_camera_with_depth(w.poses[0], w.depths[0])
    n = len(inf.get_occupied_bricks(0))
    with pytest.raises(RuntimeError, match="incorrect"):
        inf.get_indices_and_alphas(np.zeros((n + 1, 512), np.float32))
    with pytest.raises(TypeError):
        inf.get_indices_and_alphas(np.zeros((n, 512), np.float64))


def test_upper_level_nodes(G, w):
    _set_global_params(G, w.params)
    inf = G.GVDBInference(True, False)
    for P, D in zip(w.poses, w.depths):
        inf.add_camera_with_depth(P, D)
    b0 = inf.get_occupied_bricks(0)
    b1 = inf.get_occupied_bricks(1)
    assert 0 < len(b1) <= len(b0)
    parents = {tuple(((c - 4) // 64).astype(int)) for c in b0}
    assert parents == {tuple(((c - 32) // 64).astype(int)) for c in b1}


def test_occupied_voxels_mask(G, w):
    _set_global_params(G, w.params)
    inf = G.GVDBInference(True, False)
    for P, D in zip(w.poses, w.depths):
        inf.add_camera_with_depth(P, D)
    inf.perform_inference()
    n = len(inf.get_occupied_bricks(0))
    alphas = np.zeros((n, 512), np.float32)
    inf.get_indices_and_alphas(alphas)
    mask = np.zeros((n, 16), np.int32)
    inf.get_occupied_voxels_mask(mask, 0.5)
    bits = np.unpackbits(mask.view(np.uint8), bitorder="little").reshape(n, 512)
    np.testing.assert_array_equal(bits.astype(bool), alphas >= 0.5)


def test_estimator_load_map_likelihood(G, w):
    """External-map likelihood: loading the inferred beliefs at voxel centres
    reproduces the inference map's likelihood image."""
    gp = _set_global_params(G, w.params)
    m = L.MRFMap(w.params)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer()
    cen, bel = m.read_bricks()
    local = np.stack(np.meshgrid(np.arange(8), np.arange(8), np.arange(8), indexing="ij"), -1).reshape(512, 3)
    pts = ((cen[:, None, :] - 4) + local[None] + 0.5).reshape(-1, 3).astype(np.float32)
    occ = bel.reshape(-1)
    keep = occ > 0
    est = G.GVDBMapLikelihoodEstimator(gp, False)
    assert est.load_map(pts[keep], occ[keep])
    img = np.zeros((w.params.rows, w.params.cols), np.float32)
    s = est.get_likelihood_image_at_pose_with_depth(w.poses[0], w.depths[0], img)
    s_ref, img_ref = m.likelihood(w.poses[0], w.depths[0])
    np.testing.assert_allclose(img, img_ref, atol=2e-3)
    assert s == pytest.approx(s_ref, rel=1e-3)
    est.add_camera(w.poses[0], G.GVDBImage(w.depths[0]))
    assert est.compute_likelihood(0) == pytest.approx(s, rel=1e-6)


def test_c_abi_errors(native_lib, w):
    m = L.MRFMap(w.params)
    with pytest.raises(L.MrfError) as e:
        m.set_pose(5, np.eye(4))
    assert e.value.status == 1
    with pytest.raises(L.MrfError):
        m.likelihood_view(0)
    with pytest.raises(ValueError):
        m.add_view(np.eye(4), np.zeros((3, 3), np.float32))
    # an empty map: likelihood of every valid pixel is log(LIKE_EPS)
    s, img = m.likelihood(w.poses[0], w.depths[0])
    valid = np.isfinite(w.depths[0]) & (w.depths[0] > 0)
    np.testing.assert_allclose(img[valid], np.log(np.float32(1e-3)), rtol=1e-6)
    assert m.num_bricks == 0
    m.infer()  # no views: a no-op


def test_incremental_and_ids(native_lib, w):
    """perform_inference_ids zeroes only the listed cameras; MRF_INCREMENTAL
    keeps every camera's messages (matches the oracle's schedule)."""
    for ids, flags, oflags in (([1], 0, 0), (None, L.INCREMENTAL, O.INCREMENTAL)):
        m = L.MRFMap(w.params)
        om = O.OracleMap(w.params, threads=4)
        for P, D in zip(w.poses[:2], w.depths[:2]):
            m.add_view(P, D)
            om.add_view(P, D)
        m.infer(iters=3)
        om.infer(iters=3)
        m.add_view(w.poses[2], w.depths[2])
        om.add_view(w.poses[2], w.depths[2])
        m.infer(ids=ids, iters=3, flags=flags)
        om.infer(ids=ids, iters=3, flags=oflags)
        err = np.abs(m.beliefs() - om.beliefs()).max()
        assert err <= 1e-3, (ids, flags, err)


def test_set_pose_matches_oracle(native_lib, w):
    m = L.MRFMap(w.params)
    om = O.OracleMap(w.params, threads=4)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
        om.add_view(P, D)
    P2 = w.poses[1].copy()
    P2[0, 3] += 0.1
    m.set_pose(1, P2)
    om.set_pose(1, P2)
    assert m.num_bricks == om.num_bricks
    m.infer()
    om.infer()
    assert np.abs(m.beliefs() - om.beliefs()).max() <= 1e-3


def test_graph_replay_matches_direct_launches(native_lib, w):
    """The captured CUDA graph of one iteration gives bit-identical results to
    launching the kernels one by one (and to a second replay), on the
    call that captures it and on a later call on the same build."""
    out = []
    for flags in (L.NO_GRAPH, 0, 0, L.JACOBI | L.NO_GRAPH, L.JACOBI):
        m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.infer(iters=4, flags=flags)
        m.infer(iters=4, flags=flags)
        out.append(m.beliefs())
        m.close()
    for flags in (L.NO_GRAPH, 0):
        m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.infer(iters=8, flags=flags)
        out.append(m.beliefs())
        m.close()
    np.testing.assert_array_equal(out[5], out[6])
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[1], out[2])
    np.testing.assert_array_equal(out[3], out[4])


def test_runs_are_reproducible(native_lib, w):
    """No atomics in any reduction: two runs give identical bits."""
    res = []
    for _ in range(2):
        m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.infer(iters=5)
        res.append((m.beliefs(), m.logodds()))
        m.close()
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])


def test_infer_converge(native_lib, w):
    """Convergence-checked inference stops once the largest belief change is
    below the tolerance, and its state equals a fixed-count run of the same
    number of iterations (the check reads, never writes, the state)."""
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    n, d = m.infer_converge(1e-4, max_iters=60)
    assert 1 < n < 60 and 0.0 <= d < 1e-4
    b1 = m.beliefs()
    m.reset_state()
    m.infer(iters=n)
    np.testing.assert_array_equal(m.beliefs(), b1)
    # a coarse check interval: stops at a multiple of it
    m.reset_state()
    n2, d2 = m.infer_converge(1e-4, max_iters=60, check_every=4)
    assert n2 % 4 == 0 and d2 < 1e-4
    with pytest.raises(L.MrfError):
        m.infer_converge(0.0)


def test_ray_variants_identical_and_autotune(native_lib, w):
    """Every ray-kernel variant computes the same bits; the autotuner picks
    one of them and leaves the map state untouched."""
    out = []
    for k in range(L.load().mrf_ray_variants()):
        m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.set_ray_variant(k)
        m.infer(iters=3)
        out.append(m.beliefs())
        if k == 0:
            before = (m.beliefs(), m.logodds())
            best, ms = m.autotune(reps=2)
            assert 0 <= best < len(ms) and (ms > 0).all()
            np.testing.assert_array_equal(m.beliefs(), before[0])
            np.testing.assert_array_equal(m.logodds(), before[1])
        m.close()
    # the pair reduction's two variants, Gauss-Seidel and Jacobi
    for flags in (0, L.JACOBI):
        res = []
        for pv in (0, 1):
            m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
            for P, D in zip(w.poses, w.depths):
                m.add_view(P, D)
            m.set_pair_variant(pv)
            m.infer(iters=3, flags=flags)
            assert m.tuning()[2] == pv
            res.append(m.beliefs())
            m.close()
        np.testing.assert_array_equal(res[1], res[0])
        if flags == 0:
            np.testing.assert_array_equal(res[0], out[0])
    for b in out[1:]:
        np.testing.assert_array_equal(b, out[0])
    m = L.MRFMap(w.params)
    with pytest.raises(L.MrfError):
        m.set_ray_variant(99)
    with pytest.raises(L.MrfError):
        m.set_pair_variant(2)


@pytest.mark.parametrize("flags", [0, L.JACOBI, L.FIX_PRE_RESET], ids=["gauss-seidel", "jacobi", "fix-reset"])
def test_quiet_prefix_paths(native_lib, oracle_lib, w, flags):
    """From the third iteration of a call the ray kernel may take each ray's
    static prefix from its quiet sums (formed once per call) plus its loud
    incidences.  Forced on and forced off, both paths agree with the FP64
    oracle at the tests' tolerance and with each other to FP32 rounding of
    the regrouped sums, and the stats say which path ran."""
    om = O.OracleMap(w.params, threads=8)
    for P, D in zip(w.poses, w.depths):
        om.add_view(P, D, O.ACT_FULL_RAY)
    om.infer(iters=10, flags=(O.JACOBI if flags & L.JACOBI else 0) | (O.FIX_PRE_RESET if flags & L.FIX_PRE_RESET else 0))
    ob = om.beliefs()
    om.close()
    out = {}
    for name, extra in (("fast", L.QUIET_PREFIX), ("full", L.FULL_RAYS)):
        m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.infer(iters=10, flags=flags | extra)
        st = m.stats()
        assert st["quiet_prefix_used"] == (1 if name == "fast" else 0)
        assert st["n_loud_prefix"] >= 0
        b = m.beliefs().astype(np.float64)
        touched = (b > 0) | (ob > 0)
        assert np.abs(b - ob).max() <= 1e-3
        assert ((b > 0.5) == (ob > 0.5))[touched].mean() >= 0.999
        out[name] = b
        m.close()
    np.testing.assert_allclose(out["fast"], out["full"], rtol=0, atol=1e-5)


def test_home_share_moves_rays_not_results(native_lib, w):
    """The SM-region schedule's home share only moves rays between warps:
    every share gives the same bits, in Gauss-Seidel and Jacobi; its
    autotuner picks one of the shares it timed and leaves the state as it
    was."""
    for flags in (0, L.JACOBI):
        out = []
        for share in (40, 75, 100):
            m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
            for P, D in zip(w.poses, w.depths):
                m.add_view(P, D)
            m.set_ray_variant(4)
            m.infer(iters=1, flags=flags)
            m.set_home_share(share)
            assert m.tuning()[:2] == (4, share)
            m.infer(iters=3, flags=flags | L.INCREMENTAL)
            out.append(m.beliefs())
            if share == 75:
                before = (m.beliefs(), m.logodds())
                best, ms = m.autotune_home_share((50, 90), reps=2, flags=flags)
                assert best in (50, 90) and (ms > 0).all() and m.tuning()[1] == best
                np.testing.assert_array_equal(m.beliefs(), before[0])
                np.testing.assert_array_equal(m.logodds(), before[1])
            m.close()
        for b in out[1:]:
            np.testing.assert_array_equal(b, out[0])
    m = L.MRFMap(w.params)
    for bad in (0, 101):
        with pytest.raises(L.MrfError):
            m.set_home_share(bad)
    m.close()


def test_ray_variants_identical_jacobi(native_lib, w):
    """The Jacobi schedule runs one ray launch over all views' queues (the
    SM-region schedule then has regions of every view and one leftover
    queue for all): every variant still computes the same bits."""
    out = []
    for k in range(L.load().mrf_ray_variants()):
        m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.set_ray_variant(k)
        m.infer(iters=3, flags=L.JACOBI)
        out.append(m.beliefs())
        m.close()
    for b in out[1:]:
        np.testing.assert_array_equal(b, out[0])


def test_release_cached_memory(native_lib, w):
    """Device memory of destroyed maps stays pooled for the next map;
    mrf_release_cached_memory hands it back, and later maps still work."""
    m = L.MRFMap(w.params)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=2)
    b = m.beliefs()
    m.close()
    assert L.load().mrf_release_cached_memory() == 0
    m = L.MRFMap(w.params)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=2)
    np.testing.assert_array_equal(m.beliefs(), b)
    m.close()


def test_message_checkpoint_resume(native_lib, w):
    """The BP state is the per-camera messages: written back into a fresh map
    (and the total log-odds rebuilt from them) the run resumes where it
    stopped.  The rebuilt log-odds are one sum instead of a running sum, so
    the resumed run agrees to rounding."""
    ref = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        ref.add_view(P, D)
    ref.infer(iters=4)
    msgs = [ref.read_messages(v) for v in range(len(w.poses))]
    L4 = ref.logodds()
    ref.infer(iters=4, flags=L.INCREMENTAL)
    b8 = ref.beliefs()
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=1)
    for v, d in enumerate(msgs):
        m.write_messages(v, d)
    m.rebuild_logodds()
    np.testing.assert_allclose(m.logodds(), L4, atol=1e-4)
    for v, d in enumerate(msgs):
        np.testing.assert_array_equal(m.read_messages(v), d)
    m.infer(iters=4, flags=L.INCREMENTAL)
    assert np.abs(m.beliefs() - b8).max() <= 1e-4
    with pytest.raises(L.MrfError):
        m.read_messages(len(w.poses))


def test_infer_until_a_target_map(native_lib, w):
    """mrf_infer_until stops at the first checked iteration within tol of a
    target field; from the same start it takes no more iterations than the
    plain run to that field, and it equals an mrf_infer of that many
    iterations bit for bit."""
    import torch
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    n_ref, d_ref = m.infer_converge(1e-6, max_iters=400)
    assert d_ref < 1e-6
    ref = m.beliefs()
    target = torch.from_numpy(ref.reshape(-1)).cuda()
    m.reset_state()
    n, dist = m.infer_until(target.data_ptr(), 1e-3, max_iters=400)
    assert 0 < n <= n_ref and dist <= 1e-3
    got = m.beliefs()
    assert np.abs(got - ref).max() <= 1e-3
    m.reset_state()
    m.infer(iters=n)
    np.testing.assert_array_equal(m.beliefs(), got)
    # a target out of reach: runs to the cap and reports the distance
    far = torch.full_like(target, 0.5)
    m.reset_state()
    n2, d2 = m.infer_until(far.data_ptr(), 1e-3, max_iters=7)
    assert n2 == 7 and d2 > 1e-3
    with pytest.raises(L.MrfError):
        m.infer_until(0, 1e-3)
    m.close()
