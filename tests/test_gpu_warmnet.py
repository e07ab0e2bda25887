"""The learned warm start on the GPU: the network's forward pass and
gradients against the CPU reference (oracle/warmnet.py), training on the
project's own kernels, the features, and the warm-started BP against plain
BP (whose converged map is the reference result)."""
import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic
from oracle import warmnet as R

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W(native_lib):
    from mrfmap_gb300 import warmstart
    return warmstart


def _case(seed=0, nb=5):
    rng = np.random.default_rng(seed)
    feat = rng.normal(0, 1, (nb, 512, 4)).astype(np.float32)
    feat[:, :, 0] = rng.random((nb, 512))
    target = rng.normal(0, 2, (nb, 512)).astype(np.float32)
    w = (rng.random((nb, 512)) < 0.6).astype(np.float32)
    return feat, target, w


def test_param_count(W):
    assert W.n_params() == R.N_PARAMS


def test_forward_matches_reference(W):
    feat, _, _ = _case()
    net = W.WarmNet(seed=3)
    p = net.params.cpu().numpy().astype(np.float64)
    y = net.predict(torch.from_numpy(feat).cuda()).cpu().numpy()
    yr, _ = R.forward(p, feat.astype(np.float64), bf16=True)
    scale = np.abs(yr).max()
    assert np.abs(y - yr).max() <= 1e-2 * scale, np.abs(y - yr).max() / scale


def test_gradients_match_reference(W):
    feat, target, w = _case(1)
    net = W.WarmNet(seed=4)
    p = net.params.cpu().numpy().astype(np.float64)
    norm = float(w.sum())
    loss = net.gradients(torch.from_numpy(feat).cuda(), torch.from_numpy(target).cuda(),
                         torch.from_numpy(w).cuda(), norm)
    g = net.grads.cpu().numpy()
    lr, gr = R.gradients(p, feat.astype(np.float64), target.astype(np.float64), w.astype(np.float64), norm,
                         bf16=True)
    assert float(loss.item()) == pytest.approx(lr, rel=1e-3)
    o = 0
    for name, shp in R.SHAPES:
        n = int(np.prod(shp))
        a, b = g[o:o + n], gr[o:o + n]
        assert np.abs(a - b).max() <= 2e-2 * np.abs(b).max() + 1e-7, (name, np.abs(a - b).max(), np.abs(b).max())
        o += n


def test_training_step_is_deterministic_and_learns(W):
    feat, _, w = _case(2, nb=8)
    # a smooth target the network can represent: a function of the features
    target = (2.0 * feat[:, :, 1] - 1.5 * np.maximum(feat[:, :, 2], 0) + feat[:, :, 0]).astype(np.float32)
    ft, tt, wt = (torch.from_numpy(a).cuda() for a in (feat, target, w))
    runs = []
    for _ in range(2):
        net = W.WarmNet(seed=5)
        hist = net.train(ft, tt, wt, epochs=60, batch=4, lr=3e-3, seed=1)
        runs.append((net.params.cpu().numpy(), hist))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    hist = runs[0][1]
    assert hist[-1] < 0.3 * hist[0], hist[::10]


def test_features(W):
    w = synthetic.small_room(0, n_frames=3, rows=60, cols=80)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=3)
    f = W.map_features(m).cpu().numpy()
    assert f.shape == (m.num_bricks, 512, 4)
    np.testing.assert_array_equal(f[:, :, 0], m.beliefs())
    assert (f[:, :, 1:] >= 0).all()
    touched = f[:, :, 1:].sum(-1) > 0
    assert touched.mean() > 0.1
    # voxels that some camera updates are all seen
    assert touched[m.beliefs() > 0].all()


def _mk(w):
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    return m


def test_warm_start_converges_to_plain_fixed_point(W):
    """Warm-started BP (perfect prediction, a prior-only prediction, and an
    untrained network) converges to the plain run's map."""
    w = synthetic.small_room(0)
    m = _mk(w)
    n_plain, _ = m.infer_converge(1e-5, max_iters=200)
    Bp, Lp = m.beliefs(), m.logodds()
    lp = np.log(w.params.prior / (1 - w.params.prior))
    preds = {"perfect": Lp, "prior": np.full_like(Lp, lp)}
    for name, pred in preds.items():
        m2 = _mk(w)
        m2.infer(iters=1)
        m2.warm_start(pred, sweeps=2)
        n, d = m2.infer_converge(1e-5, max_iters=200, flags=L.INCREMENTAL)
        Bw = m2.beliefs()
        touched = (Bp > 0) | (Bw > 0)
        assert np.abs(Bw - Bp).max() <= 1e-3, name
        assert ((Bw > 0.5) == (Bp > 0.5))[touched].mean() >= 0.999, name
    m3 = _mk(w)
    m3.infer(iters=1)
    net = W.WarmNet(seed=0)
    W.warm_start(m3, net, sweeps=1)
    m3.infer_converge(1e-5, max_iters=200, flags=L.INCREMENTAL)
    assert np.abs(m3.beliefs() - Bp).max() <= 1e-3


def test_trained_network_gain_over_prior_prediction(W):
    """What training buys: on held-out scenes the trained network's
    predicted log-odds are closer to plain BP's converged log-odds than the
    prediction without a network (the prior everywhere), and BP warm-started
    from it still converges to plain BP's map."""
    train = [synthetic.small_room(s, n_frames=4, rows=96, cols=128) for s in range(10, 16)]
    held = [synthetic.small_room(s, n_frames=4, rows=96, cols=128) for s in (40, 41)]
    feats, targets, weights = W.build_dataset(train, bricks_per_scene=512)
    net = W.WarmNet(seed=0)
    hist = net.train(feats, targets, weights, epochs=40, batch=64, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0]
    for w in held:
        m = _mk(w)
        feat, lo, wt = W.training_pairs(m)
        pred = net.predict(feat).clamp(-W.LOGIT_CLIP, W.LOGIT_CLIP)
        lp = float(np.log(w.params.prior / (1 - w.params.prior)))
        err_net = float(((pred - lo) ** 2 * wt).sum() / wt.sum())
        err_prior = float(((lp - lo) ** 2 * wt).sum() / wt.sum())
        assert err_net < 0.5 * err_prior, (err_net, err_prior)
        Bp = m.beliefs()
        m.reset_state()
        W.warm_start(m, net)
        m.infer_converge(1e-5, max_iters=200, flags=L.INCREMENTAL)
        assert np.abs(m.beliefs() - Bp).max() <= 1e-3
