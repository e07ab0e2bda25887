"""Host logic of the learned warm start (no GPU): the network's parameter
layout and initialisation, and the summary rule of the warm-start
measurement -- a scene counts only when plain BP from the prior converged
to a reference map and every method reached that map (within the accept
tolerance, at the class-agreement floor); speed-ups are ratios of the
compared scenes' mean times."""
import numpy as np
import pytest

from mrfmap_gb300 import warmstart as W


def test_init_params_layout(native_lib):
    p = W.init_params(seed=3)
    assert p.dtype == np.float32 and p.size == W.n_params()
    # three 3x3x3 convolutions 4 -> 16 -> 16 -> 1 with their biases
    sizes = [27 * 4 * 16, 16, 27 * 16 * 16, 16, 27 * 16 * 1, 1]
    assert sum(sizes) == p.size
    parts = np.split(p, np.cumsum(sizes)[:-1])
    for k, (part, fan_in) in enumerate(zip(parts, (108, None, 432, None, 432, None))):
        if fan_in is None:
            assert np.all(part == 0.0), f"bias {k} not zero"
        else:
            assert abs(part.std() - np.sqrt(2.0 / fan_in)) < 0.1 * np.sqrt(2.0 / fan_in)
    np.testing.assert_array_equal(p, W.init_params(seed=3))
    assert not np.array_equal(p, W.init_params(seed=4))


def _row(seed, plain=(50, 100.0), learned=(40, 80.0), prior=(45, 90.0), ref=True, reached=True, err=5e-4,
         agree=1.0):
    r = {"seed": seed, "ref_converged": ref, "net_forward_ms": 2.0, "n_bricks": 1000}
    for k, (it, ms) in (("plain", plain), ("learned", learned), ("prior", prior)):
        r.update({k + "_iters": it, k + "_ms": ms, k + "_start_ms": 1.0, k + "_reached": reached,
                  k + "_max_err": err, k + "_agree": agree})
    return r


def test_summary_compares_only_scenes_every_method_reached():
    rows = [_row(0), _row(1, plain=(70, 140.0), learned=(60, 120.0), prior=(65, 130.0)),
            _row(2, ref=False),                     # no converged reference map
            _row(3, err=2e-3),                      # outside the accept tolerance
            _row(4, agree=0.99),                    # under the class-agreement floor
            _row(5, reached=False)]                 # a method never got there
    out = W.summarize(rows, accept_tol=1e-3, agree_min=0.999)
    assert out["scenes"] == 6 and out["scenes_ref_converged"] == 5 and out["scenes_compared"] == 2
    assert out["plain_ms"] == pytest.approx(120.0) and out["learned_ms"] == pytest.approx(100.0)
    assert out["prior_ms"] == pytest.approx(110.0)
    assert out["plain_iters"] == pytest.approx(60) and out["learned_iters"] == pytest.approx(50)
    assert out["prior_iters"] == pytest.approx(55)
    assert out["speedup_learned_vs_plain"] == pytest.approx(1.2)
    assert out["speedup_prior_vs_plain"] == pytest.approx(120.0 / 110.0)
    assert out["speedup_learned_vs_prior"] == pytest.approx(1.1)
    assert out["max_belief_err_vs_converged"]["learned"] == pytest.approx(5e-4)
    # 2 * 9072 multiply-adds per voxel, 512 voxels per brick, 1000 bricks in 2 ms
    assert out["net_forward_tflops"] == pytest.approx(2 * 9072 * 512 * 1000 / 2e9)


def test_summary_without_comparable_scenes():
    out = W.summarize([_row(0, ref=False)])
    assert out["scenes_compared"] == 0 and out["plain_ms"] is None
    assert "speedup_learned_vs_plain" not in out
