"""Learned warm start for the BP: a brick-local 3-D convolutional network
predicts each voxel's converged log-odds from per-voxel features of the
incidence lists; BP then starts from messages computed at that prediction
(``mrf_warm_start``) instead of from zero.

Everything numeric runs in the library's own kernels through the C ABI
(features ``mrf_warm_features``; network forward, gradients and Adam
``mrf_net_*``, BF16 tensor-core convolutions with FP32 accumulation).  torch
only provides device buffers and the stream.  Plain BP from the prior stays
the judge: a warm-started map is accepted only when its converged beliefs
match the plain run's.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import lib as L

LOGIT_CLIP = 9.21  # |logit| of the belief clamp 1e-4


def _torch():
    import torch
    return torch


def n_params() -> int:
    return int(L.load().mrf_net_num_params())


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases (layout of mrf_net_num_params)."""
    rng = np.random.default_rng(seed)
    out = []
    for fan_in, shape in ((27 * 4, (27, 4, 16)), (None, (16,)), (27 * 16, (27, 16, 16)), (None, (16,)),
                          (27 * 16, (27, 16, 1)), (None, (1,))):
        if fan_in is None:
            out.append(np.zeros(shape))
        else:
            out.append(rng.normal(0.0, np.sqrt(2.0 / fan_in), shape))
    p = np.concatenate([a.ravel() for a in out]).astype(np.float32)
    assert p.size == n_params()
    return p


def map_features(m: L.MRFMap):
    """[n_bricks, 512, 4] features of a map (device tensor)."""
    torch = _torch()
    f = torch.empty((m.num_bricks, 512, 4), dtype=torch.float32, device="cuda")
    if m.num_bricks:
        m.warm_features(f.data_ptr())
    return f


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@dataclass
class WarmNet:
    """Network parameters and Adam state on the device."""
    params: "object" = None
    seed: int = 0
    step: int = 0
    history: list = field(default_factory=list)

    def __post_init__(self):
        torch = _torch()
        p = init_params(self.seed) if self.params is None else np.asarray(self.params, np.float32)
        self.params = torch.from_numpy(p.copy()).cuda()
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)
        self.grads = torch.zeros_like(self.params)
        self._ws = None
        self._ws_nb = 0

    def _workspace(self, nb):
        torch = _torch()
        if self._ws is None or self._ws_nb < nb:
            self._ws = torch.empty(int(L.load().mrf_net_workspace_bytes(nb)), dtype=torch.uint8, device="cuda")
            self._ws_nb = nb
        return self._ws

    def predict(self, feat, stream: int = 0):
        """feat [nb, 512, 4] (device) -> predicted log-odds [nb, 512]."""
        torch = _torch()
        nb = feat.shape[0]
        out = torch.empty((nb, 512), dtype=torch.float32, device="cuda")
        if nb:
            L._check(L.load().mrf_net_forward(_ptr(self.params), _ptr(feat), nb, _ptr(out),
                                              _ptr(self._workspace(nb)), C.c_void_p(stream)))
        return out

    def gradients(self, feat, target, weight, norm: float):
        torch = _torch()
        nb = feat.shape[0]
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        L._check(L.load().mrf_net_gradients(_ptr(self.params), _ptr(feat), _ptr(target), _ptr(weight), nb,
                                            float(norm), _ptr(self.grads), _ptr(loss),
                                            _ptr(self._workspace(nb)), None))
        return loss

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        L._check(L.load().mrf_net_adam(_ptr(self.params), _ptr(self.grads), _ptr(self.m1), _ptr(self.m2),
                                       self.params.numel(), lr, b1, b2, eps, self.step, None))

    def train(self, feats, targets, weights, epochs: int = 10, batch: int = 512, lr: float = 1e-3,
              seed: int = 0):
        """Adam over shuffled batches of bricks; returns the mean loss per epoch."""
        torch = _torch()
        g = torch.Generator(device="cpu")
        g.manual_seed(seed)
        n = feats.shape[0]
        for _ in range(epochs):
            order = torch.randperm(n, generator=g).cuda()
            tot, cnt = 0.0, 0
            losses = []
            for s in range(0, n, batch):
                idx = order[s:s + batch]
                f, t, w = feats[idx].contiguous(), targets[idx].contiguous(), weights[idx].contiguous()
                norm = max(float(w.sum().item()), 1.0)
                losses.append(self.gradients(f, t, w, norm))
                self.adam(lr)
                cnt += 1
            tot = float(torch.stack(losses).mean().item()) if losses else 0.0
            self.history.append(tot)
        return self.history

    def save(self, path: str):
        np.asarray(self.params.cpu().numpy(), np.float32).tofile(path)

    @classmethod
    def load_file(cls, path: str):
        return cls(params=np.fromfile(path, dtype=np.float32))


def training_pairs(m: L.MRFMap, tol: float = 1e-4, max_iters: int = 200):
    """(features, converged log-odds, voxel weights) of one map after plain
    BP to convergence; weights select the voxels some camera updates."""
    torch = _torch()
    feat = map_features(m)  # before BP: belief feature of the fresh map
    m.reset_state()
    m.infer_converge(tol, max_iters=max_iters)
    lo = torch.from_numpy(np.clip(m.logodds(), -LOGIT_CLIP, LOGIT_CLIP).astype(np.float32)).cuda()
    touched = torch.from_numpy((m.beliefs() > 0).astype(np.float32)).cuda()
    return feat, lo, touched


def warm_start(m: L.MRFMap, net: WarmNet, sweeps: int = 1):
    """Predict the map's log-odds and start BP from messages at that field."""
    feat = map_features(m)
    pred = net.predict(feat)
    pred.clamp_(-LOGIT_CLIP, LOGIT_CLIP)
    _torch().cuda.synchronize()
    m.warm_start_device(pred.data_ptr(), sweeps)
    return pred


DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "warmnet_params.bin")
