"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden outputs, so the oracle is pinned by
closed-form single-ray cases restated independently here in plain Python,
an independent float32 DDA, and invariants of the update equations.
"""
import math

import numpy as np
import pytest

from mrfmap_gb300.params import MapParams
from oracle import oracle as O

F_EPS = float(np.float32(1e-4))
LIKE_EPS = float(np.float32(1e-3))


def _params(sigma=0.5, prior=0.1, dims=(32.0, 32.0, 32.0)):
    p = MapParams(res=1.0, dims=dims, rows=1, cols=1, fx=1000.0, fy=1000.0, cx=0.5, cy=0.5,
                  prior=prior, max_iters=1)
    p.set_const_polys([sigma, 0.0, 0.0], [0.0, 0.0, 0.0])
    return p


def _pose_x(o_vox, p):
    """camera looking along world +x with its origin at voxel coords o_vox"""
    P = np.eye(4, dtype=np.float32)
    P[:3, :3] = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]], np.float32)
    off = np.array([p.dims[0] / 2 / p.res, p.dims[1] / 2 / p.res, 0.0])
    P[:3, 3] = (np.asarray(o_vox) - off) * p.res
    return P


def _clamp(x, lo, hi):
    return min(max(x, lo), hi)


def _potential(s, d, sig):
    s3 = 3 * sig
    return 0.398942 / s3 * math.exp(-0.5 * ((d - s) / s3) ** 2)


def _single_ray_messages(q, lens, mus, inf_vis=None):
    """Pre/Post recursions of gvdbkernels.cu:689-1038 for one ray, no reset."""
    A, T = 0.0, 0.0
    for qi, li, mi in zip(q, lens, mus):
        A += li * math.log(qi)
        T += math.exp(A) * (1 - qi) * mi
    if inf_vis is not None:
        T += math.exp(A)
    A, F, out = 0.0, 0.0, []
    for qi, li, mi in zip(q, lens, mus):
        A += li * math.log(qi)
        V = math.exp(A)
        tau = V * (1 - qi) * mi
        R = T - F - tau
        mu1 = F + V * mi
        mu0 = F + R / qi
        out.append(_clamp(mu1 / (mu1 + mu0 + 1e-7), F_EPS, 1 - F_EPS))
        F += tau
    return out


def _belief(L):
    return 1 - _clamp(1 / (1 + math.exp(L)), F_EPS, 1 - F_EPS)


def test_single_ray_closed_form(oracle_lib):
    p = _params(sigma=0.5)
    m = O.OracleMap(p)
    o = (0.5, 16.5, 16.5)
    d = 10.0
    m.add_view(_pose_x(o, p), np.array([[d]], np.float32))
    # endpoint voxel (10,16,16) with halo 9..11 x 15..17 x 15..17 -> bricks x=1, y,z in {1,2}
    assert sorted(map(tuple, m.brick_coords())) == [(1, 1, 1), (1, 1, 2), (1, 2, 1), (1, 2, 2)]
    t = m.view_trace(0)
    assert len(t["pix"]) == 1
    n_pre, n_post, r0, rinf, gate = t["meta"][0]
    # the ray crosses brick (1,2,2) along x: voxels 8..15, unit lengths; the
    # brick exit depth 15.5 > d + 3 sigma = 11.5 stops both passes there
    assert (n_pre, n_post, r0, gate) == (8, 8, 0, 0)
    np.testing.assert_array_equal(t["len"], np.ones(8, np.float32))
    np.testing.assert_array_equal(t["s"], np.arange(8, 16, dtype=np.float32) + 0.5)
    mus = [_potential(8.5 + i, d, 0.5) for i in range(8)]
    np.testing.assert_allclose(t["mu"], mus, rtol=1e-12)
    m.infer(iters=1)
    Lp = math.log(float(np.float32(0.1))) - math.log(1 - float(np.float32(0.1)))
    q = [_clamp(1 / (1 + math.exp(Lp)), F_EPS, 1 - F_EPS)] * 8
    pm = _single_ray_messages(q, [1.0] * 8, mus)
    b = m.beliefs()
    slot = [tuple(c) for c in m.brick_coords()].index((1, 2, 2))
    for i in range(8):
        a = _clamp(pm[i], F_EPS, 1 - F_EPS)
        Lv = Lp + math.log(a) - math.log(1 - a)
        local = (i * 8 + 0) * 8 + 0  # (x=i, y=16%8=0, z=16%8=0)
        assert b[slot, local] == pytest.approx(_belief(Lv), abs=1e-12)
    # the two voxels whose exit depths (9.5, 10.5) straddle d = 10 carry the
    # same, largest occupancy
    col = np.array([b[slot, (i * 8) * 8] for i in range(8)])
    assert col[1] == pytest.approx(col[2], rel=1e-12) and col[1] == col.max()


def test_infinity_term_only(oracle_lib):
    """d beyond every active brick: all potentials vanish and only the
    visibility-at-infinity term remains; every message is F_EPS."""
    p = _params(sigma=0.01)
    m = O.OracleMap(p)
    m.add_view(_pose_x((0.5, 16.5, 16.5), p), np.array([[100.0]], np.float32), O.ACT_FULL_RAY)
    t = m.view_trace(0)
    n_pre, n_post, r0, rinf, gate = t["meta"][0]
    assert gate == 1 and n_pre == n_post == 40  # voxels x = 0..39, the camera inside x = 0
    assert r0 == n_pre and rinf == 32  # no non-zero potential; last brick run starts at x=32
    assert np.all(t["mu"] == 0)
    m.infer(iters=1)
    Lp = math.log(float(np.float32(0.1))) - math.log(1 - float(np.float32(0.1)))
    a = F_EPS
    want = _belief(Lp + math.log(a) - math.log(1 - a))
    b = m.beliefs()
    coords = [tuple(c) for c in m.brick_coords()]
    for x in range(0, 40):
        s = coords.index((x // 8, 2, 2))
        assert b[s, ((x % 8) * 8) * 8] == pytest.approx(want, abs=1e-12)


def test_invalid_pixels_do_nothing(oracle_lib):
    p = _params()
    m = O.OracleMap(p)
    for d in (np.nan, -1.0, 0.0):
        m.add_view(_pose_x((0.5, 16.5, 16.5), p), np.array([[d]], np.float32))
    assert m.num_bricks == 0
    m.infer()
    assert m.last_updates == 0


def test_short_cumulative_length_is_ignored(oracle_lib):
    """A voxel whose total crossing length is <= 0.1 keeps its state
    (gvdbkernels.cu:408, 489-495)."""
    p = _params(sigma=0.5)
    m = O.OracleMap(p)
    m.add_view(_pose_x((7.95, 16.5, 16.5), p), np.array([[0.5]], np.float32))
    coords = [tuple(c) for c in m.brick_coords()]
    assert (0, 2, 2) in coords and (1, 2, 2) in coords
    t = m.view_trace(0)
    assert t["len"][0] == np.float32(np.float32(8.0) - np.float32(7.95))
    m.infer(iters=1)
    b = m.beliefs()
    L = m.logodds()
    s0 = coords.index((0, 2, 2))
    Lp = math.log(float(np.float32(0.1))) - math.log(1 - float(np.float32(0.1)))
    assert b[s0, (7 * 8) * 8] == 0.0
    assert L[s0, (7 * 8) * 8] == pytest.approx(Lp, abs=1e-15)
    s1 = coords.index((1, 2, 2))
    assert b[s1, 0] > 0.0


def test_empty_map_likelihood(oracle_lib):
    p = MapParams(res=0.05, dims=(4.0, 4.0, 3.0), rows=8, cols=10, fx=10, fy=10, cx=5, cy=4, prior=0.1)
    p.set_const_polys([0.01, 0, 0])
    m = O.OracleMap(p)
    rng = np.random.default_rng(3)
    depth = rng.uniform(0.5, 12.0, (8, 10)).astype(np.float32)
    depth[0, :3] = np.nan
    depth[1, 0] = 0.0
    tot, img = m.likelihood(np.eye(4, dtype=np.float32), depth)
    valid = np.isfinite(depth) & (depth > 0)
    want = np.where(depth >= 10.0, math.log(1 - LIKE_EPS), math.log(LIKE_EPS))
    np.testing.assert_allclose(img[valid], want[valid], rtol=1e-6)
    assert np.all(img[~valid] == 0)
    assert tot == pytest.approx(want[valid].sum(), rel=1e-9)


def _f(x):
    return np.float32(x)


def _py_dda(o, d, E):
    """Independent fp32 restatement of the Amanatides-Woo DDA (numpy float32
    scalars, every operation rounded separately)."""
    t0, t1 = _f(0.0), _f(np.inf)
    inv = [_f(0.0)] * 3
    for a in range(3):
        if d[a] != 0:
            inv[a] = _f(1.0) / d[a]
            tA = (_f(0.0) - o[a]) * inv[a]
            tB = (_f(E[a]) - o[a]) * inv[a]
            tn, tf = min(tA, tB), max(tA, tB)
        else:
            if o[a] < 0 or o[a] >= E[a]:
                return []
            tn, tf = _f(-np.inf), _f(np.inf)
        t0, t1 = max(t0, tn), min(t1, tf)
    if not t0 < t1:
        return []
    v, step, tmax = [], [], []
    for a in range(3):
        vi = int(np.floor(o[a] + t0 * d[a]))
        vi = min(max(vi, 0), E[a] - 1)
        v.append(vi)
        s = 1 if d[a] > 0 else (-1 if d[a] < 0 else 0)
        step.append(s)
        tmax.append((_f(vi + 1) - o[a]) * inv[a] if s > 0 else
                    ((_f(vi) - o[a]) * inv[a] if s < 0 else _f(np.inf)))
    out, tprev = [], t0
    while True:
        a = 0 if (tmax[0] <= tmax[1] and tmax[0] <= tmax[2]) else (1 if tmax[1] <= tmax[2] else 2)
        te = tmax[a]
        ln = max(te - tprev, _f(0.0))
        out.append((tuple(v), ln, te))
        tprev = max(tprev, te)
        v[a] += step[a]
        if v[a] < 0 or v[a] >= E[a]:
            break
        nb = _f(v[a] + 1) if step[a] > 0 else _f(v[a])
        tmax[a] = (nb - o[a]) * inv[a]
    return out


def _py_ray(p, P, x, y):
    W, H = _f(p.cols), _f(p.rows)
    ndcx = _f(2.0) * ((_f(x) + _f(0.5)) / W) - _f(1.0)
    ndcy = _f(2.0) * ((_f(y) + _f(0.5)) / H) - _f(1.0)
    rx = ndcx * (_f(p.cx) / _f(p.fx))
    ry = ndcy * (_f(p.cy) / _f(p.fy))
    P = P.astype(np.float32)
    dw = [(P[a, 0] * rx + P[a, 1] * ry) + P[a, 2] for a in range(3)]
    n = np.sqrt((dw[0] * dw[0] + dw[1] * dw[1]) + dw[2] * dw[2], dtype=np.float32)
    d = [dw[a] / n for a in range(3)]
    res = _f(p.res)
    off = [(_f(p.dims[0]) * _f(0.5)) / res, (_f(p.dims[1]) * _f(0.5)) / res, _f(0.0)]
    o = [P[a, 3] / res + off[a] for a in range(3)]
    mult = res * abs((P[0, 2] * d[0] + P[1, 2] * d[1]) + P[2, 2] * d[2])
    return o, d, mult


def test_dda_bit_exact_against_independent_restatement(oracle_lib, small_room):
    w = small_room
    p = w.params
    m = O.OracleMap(p)
    for P, D in zip(w.poses[:2], w.depths[:2]):
        m.add_view(P, D, O.ACT_FULL_RAY)
    nb = np.zeros(3, np.int32)
    for a in range(3):
        g = _f(p.dims[a]) / _f(p.res)
        nb[a] = (int(np.ceil(g)) + 1 + 7) // 8
    E = [8 * int(n) for n in nb]
    active = {tuple(c) for c in m.brick_coords()}
    coords = [tuple(c) for c in m.brick_coords()]
    rng = np.random.default_rng(1)
    for _ in range(40):
        P = w.poses[rng.integers(len(w.poses))]
        x, y = int(rng.integers(p.cols)), int(rng.integers(p.rows))
        o, d, mult = _py_ray(p, P, x, y)
        steps = [(v, ln, te) for v, ln, te in _py_dda(o, d, E)
                 if (v[0] // 8, v[1] // 8, v[2] // 8) in active]
        vox, ln, s = m.trace_pixel(P, x, y)
        want_vox = [coords.index((v[0] // 8, v[1] // 8, v[2] // 8)) * 512 +
                    ((v[0] % 8) * 8 + v[1] % 8) * 8 + v[2] % 8 for v, _, _ in steps]
        assert list(vox) == want_vox
        np.testing.assert_array_equal(ln.view(np.uint32),
                                      np.array([l for _, l, _ in steps], np.float32).view(np.uint32))
        np.testing.assert_array_equal(
            s.view(np.uint32), np.array([te * mult for _, _, te in steps], np.float32).view(np.uint32))


def test_gauss_seidel_and_jacobi_reach_same_fixed_point(oracle_lib):
    from mrfmap_gb300 import synthetic
    w = synthetic.small_room(2, n_frames=3, rows=45, cols=60)
    res = {}
    for name, flags in (("gs", 0), ("jacobi", O.JACOBI)):
        m = O.OracleMap(w.params, threads=4)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D, O.ACT_ENDPOINT)
        m.infer(iters=60, flags=flags)
        res[name] = m.beliefs()
    a, b = res["gs"], res["jacobi"]
    touched = (a > 0) | (b > 0)
    assert ((a > 0.5) == (b > 0.5))[touched].mean() >= 0.99
    assert np.median(np.abs(a - b)[touched]) <= 1e-3


def test_second_infer_double_counts_unless_incremental(oracle_lib):
    """Reference quirk: perform_inference zeroes the camera messages but not
    the total log-odds, so a second call adds the messages again."""
    from mrfmap_gb300 import synthetic
    w = synthetic.small_room(4, n_frames=2, rows=30, cols=40)
    out = {}
    for flags in (0, O.INCREMENTAL):
        m = O.OracleMap(w.params)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.infer(iters=5)
        L1 = m.logodds().copy()
        m.infer(iters=5, flags=flags)
        out[flags] = (L1, m.logodds())
    L1, L2 = out[O.INCREMENTAL]
    assert np.max(np.abs(L2 - L1)) < 0.05 * max(1.0, np.max(np.abs(L1)))
    L1, L2 = out[0]
    lp = math.log(float(np.float32(0.1))) - math.log(1 - float(np.float32(0.1)))
    moved = np.abs(L1 - lp) > 1.0
    assert np.mean(np.abs(L2[moved] - lp) > 1.5 * np.abs(L1[moved] - lp)) > 0.5


def test_render_single_ray_known_answers(oracle_lib):
    """Evaluation renders on one ray through one active brick with a single
    occupied voxel (x = 10, belief 0.9): the ray starts at x = 0.5 so that
    voxel is left at s = 10.5."""
    p = _params(sigma=0.5)
    m = O.OracleMap(p)
    P = _pose_x((0.5, 16.5, 16.5), p)
    m.add_view(P, np.array([[10.0]], np.float32))
    b = np.zeros((m.num_bricks, 512), np.float32)
    slot = [tuple(c) for c in m.brick_coords()].index((1, 2, 2))
    b[slot, (2 * 8 + 0) * 8 + 0] = 0.9
    m.set_beliefs(b)

    def r(mode, d, thresh=0.5):
        img, cnt = m.render(mode, P, np.array([[d]], np.float32), thresh)
        return float(img[0, 0]), cnt

    # expected depth: (1 - 0.1) * z(corner 10 - 0.5) / (1 - 0.1 + F_EPS)
    v, _ = r(0, 10.0)
    assert v == pytest.approx(0.9 * 9.5 / (0.9 + F_EPS), rel=1e-5)
    # accuracy: density peak at s = 10.5, within one sigma (0.5) of d
    assert r(1, 10.2)[0] == 1.0
    assert r(1, 11.5)[0] == 0.0
    v, cnt = r(1, float("nan"))
    assert v == -1.0 and list(cnt) == [1, 0, 0, 0]
    # simple accuracy: first voxel >= thresh, true positive within one voxel
    assert r(2, 10.0)[0] == 1.0
    assert r(2, 12.0)[0] == 2.0
    assert r(2, 10.0, thresh=0.95)[0] == 0.0   # brick ends (s = 15.5) past d
    assert r(2, 20.0, thresh=0.95)[0] == -1.0  # never reaches d inside the map
    # occupancy at the first voxel past the measurement
    assert r(3, 10.0)[0] == 1.0
    assert r(3, 11.0)[0] == 0.0
    assert r(3, 20.0)[0] == -1.0
    v, cnt = r(3, 10.0)
    assert list(cnt) == [0, 0, 1, 0]


def test_logodds_insertion_known_answer(oracle_lib):
    """The classic log-odds insertion (the CPU insertion baseline) along one
    ray: every active voxel the ray crosses before its endpoint gets the
    miss log-odds, the voxel holding the endpoint the hit log-odds, and the
    ray stops there; a second insertion adds again, clamped."""
    from mrfmap_gb300 import synthetic
    w = synthetic.small_room(3, n_frames=2, rows=45, cols=60)
    m = O.OracleMap(w.params, threads=2)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D, O.ACT_FULL_RAY)
    P, D = w.poses[0], w.depths[0]
    ys, xs = np.nonzero(D > 0)
    y, x = int(ys[len(ys) // 2]), int(xs[len(xs) // 2])
    one = np.zeros_like(D)
    one[y, x] = D[y, x]
    vox, _, s = m.trace_pixel(P, x, y)
    hit = int(np.argmax(s >= one[y, x]))
    assert s[hit] >= one[y, x] and (hit == 0 or s[hit - 1] < one[y, x])
    n, L = m.insert_logodds(P, one, l_hit=0.85, l_miss=-0.4, l_min=-2.0, l_max=3.5)
    assert n == hit + 1
    expect = np.zeros_like(L)
    for v in vox[:hit]:
        expect[v] += float(np.float32(-0.4))  # the parameters pass as float
    expect[vox[hit]] += float(np.float32(0.85))
    np.testing.assert_allclose(L, expect, rtol=0, atol=1e-12)
    for _ in range(9):
        m.insert_logodds(P, one, logodds=L, l_hit=0.85, l_miss=-0.4, l_min=-2.0, l_max=3.5)
    assert L.min() >= -2.0 and L.max() <= 3.5
    np.testing.assert_allclose(L[vox[hit]], 3.5)
    np.testing.assert_allclose(L[vox[:hit]], -2.0)
    assert len(set(vox[:hit + 1].tolist())) == hit + 1  # a ray crosses a voxel once
    # a whole image: every valid pixel's ray makes at least its endpoint update
    n_all, L_all = m.insert_logodds(P, D)
    assert n_all >= 1 and np.isfinite(L_all).all()
    assert (L_all > 0).any() and (L_all < 0).any()


def test_camera_updates_are_one_gauss_seidel_iteration(oracle_lib, small_room):
    """orc_update_camera over every camera in order (the CPU baseline's unit)
    is one Gauss-Seidel iteration of orc_infer, bit for bit."""
    from oracle import oracle as O
    w = small_room
    a = O.OracleMap(w.params, threads=2)
    b = O.OracleMap(w.params, threads=2)
    for P, D in zip(w.poses, w.depths):
        a.add_view(P, D, O.ACT_FULL_RAY)
        b.add_view(P, D, O.ACT_FULL_RAY)
    b.build_all()
    for it in range(2):
        a.infer(iters=1, flags=O.INCREMENTAL)
        n = sum(b.update_camera(c) for c in range(len(w.poses)))
        assert n == a.last_updates
    np.testing.assert_array_equal(a.beliefs(), b.beliefs())
    with pytest.raises(ValueError):
        b.update_camera(len(w.poses))
    a.close()
    b.close()
