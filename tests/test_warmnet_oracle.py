"""Pins of the warm-start network's CPU reference (no GPU): its analytic
gradients against central finite differences of the exact FP64 network,
and the bfloat16 rounding helper against known values."""
import numpy as np

from oracle import warmnet as R


def _case(seed=0, nb=2):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, R.N_PARAMS)
    feat = rng.normal(0, 1, (nb, 512, 4))
    target = rng.normal(0, 2, (nb, 512))
    w = (rng.random((nb, 512)) < 0.7).astype(np.float64)
    return p, feat, target, w


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.001953125, 1.005859375, -3.14159265, 65504.0, 1e-30])
    got = R.to_bf16(x)
    # bf16 keeps 8 significant bits: 1 + 2^-8 and 1 + 2^-9 round to 1 (the
    # first is a tie, even mantissa wins); 1 + 1.5 * 2^-8 rounds up to 1 + 2^-7
    np.testing.assert_array_equal(got[:4], [1.0, 1.0, 1.0, 1.0078125])
    assert got[4] == -3.140625
    assert got[5] == 65536.0
    assert abs(got[6] - 1e-30) < 1e-32


def test_gradients_match_finite_differences():
    p, feat, target, w = _case()
    norm = float(w.sum())
    loss, g = R.gradients(p, feat, target, w, norm, bf16=False)
    rng = np.random.default_rng(1)
    idx = rng.choice(R.N_PARAMS, 40, replace=False)
    idx = np.concatenate([idx, [R.N_PARAMS - 1, 1728, 1728 + 16 + 5]])  # b3, b1[0], W2 entry
    h = 1e-5
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = R.gradients(pp, feat, target, w, norm, bf16=False)
        lm, _ = R.gradients(pm, feat, target, w, norm, bf16=False)
        num = (lp - lm) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(num), (i, num, g[i])


def test_forward_zero_padding_and_taps():
    """A single tap weight moves a one-hot input by that tap's offset."""
    p = np.zeros(R.N_PARAMS)
    P = R.unpack(p)
    P["W1"][(2 * 3 + 1) * 3 + 1, 0, 0] = 1.0   # tap (dx,dy,dz) = (+1,0,0)
    P["W2"][13, 0, 0] = 1.0                    # centre tap
    P["W3"][13, 0, 0] = 1.0
    feat = np.zeros((1, 512, 4))
    feat[0, (3 * 8 + 4) * 8 + 5, 0] = 2.0       # voxel (3,4,5)
    y, _ = R.forward(R.pack(P), feat, bf16=False)
    # out[v] = in[v + (1,0,0)]: the value appears at (2,4,5)
    assert y[0, (2 * 8 + 4) * 8 + 5] == 2.0
    assert np.count_nonzero(y) == 1
    feat[:] = 0
    feat[0, (0 * 8 + 4) * 8 + 5, 0] = 2.0       # x = 0 would land at x = -1: outside the brick
    y, _ = R.forward(R.pack(P), feat, bf16=False)
    assert np.count_nonzero(y) == 0
