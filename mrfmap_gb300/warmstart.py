"""Learned warm start for the BP: a brick-local 3-D convolutional network
predicts each voxel's converged log-odds from per-voxel features of the
incidence lists; BP then starts from messages computed at that prediction
(``mrf_warm_start``) instead of from zero.

Everything numeric runs in the library's own kernels through the C ABI
(features ``mrf_warm_features``; network forward, gradients and Adam
``mrf_net_*``, BF16 tensor-core convolutions with FP32 accumulation).  torch
only provides device buffers and the stream.  Plain BP from the prior stays
the reference result: a warm-started map is accepted only when its
converged beliefs match the plain run's.
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


def warm_start(m: L.MRFMap, net: WarmNet, sweeps: int = 0):
    """Predict the map's log-odds and start BP from messages at that field."""
    feat = map_features(m)
    pred = net.predict(feat)
    pred.clamp_(-LOGIT_CLIP, LOGIT_CLIP)
    _torch().cuda.synchronize()
    m.warm_start_device(pred.data_ptr(), sweeps)
    return pred


DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "warmnet_params.bin")


def _scene(seed: int, frames: int, rows: int, cols: int, res: float):
    from . import synthetic
    return synthetic.full_room(seed, n_frames=frames, rows=rows, cols=cols, res=res)


def scenes(seeds, frames=10, rows=240, cols=320, res=0.02, workers: int = 0):
    """Seeded training / held-out scenes (the C4 shape: 10 frames 320x240,
    2 cm); generated on host cores in spawned processes."""
    import multiprocessing as mp
    args = [(s, frames, rows, cols, res) for s in seeds]
    workers = workers or min(len(args), os.cpu_count() or 1)
    if workers <= 1:
        return [_scene(*a) for a in args]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.starmap(_scene, args)


def build_dataset(workloads, activation=L.ACT_FULL_RAY, bricks_per_scene: int = 2048, seed: int = 0,
                  tol: float = 1e-4, max_iters: int = 200):
    """Training tensors from plain BP run to convergence on each workload:
    every brick holding a dynamic (near-surface) voxel plus a random share
    of the others, up to bricks_per_scene per scene."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    F, T, Wt = [], [], []
    for w in workloads:
        m = L.MRFMap(w.params, activation=activation)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        feat, lo, wt = training_pairs(m, tol=tol, max_iters=max_iters)
        near = (feat[:, :, 2] > 0).any(dim=1).cpu().numpy()
        seen = (wt > 0).any(dim=1).cpu().numpy()
        idx = np.flatnonzero(near & seen)
        rest = np.flatnonzero(~near & seen)
        if len(idx) > bricks_per_scene:
            idx = rng.choice(idx, bricks_per_scene, replace=False)
        extra = min(len(rest), max(bricks_per_scene - len(idx), 0), bricks_per_scene // 4)
        if extra:
            idx = np.concatenate([idx, rng.choice(rest, extra, replace=False)])
        sel = torch.from_numpy(np.sort(idx)).cuda()
        F.append(feat[sel])
        T.append(lo[sel])
        Wt.append(wt[sel])
        m.close()
    return torch.cat(F), torch.cat(T), torch.cat(Wt)


def evaluate(net, workloads, accept_tol: float = 1e-3, ref_tol: float = 1e-4, ref_max_iters: int = 3000,
             max_iters: int = 3000, sweeps: int = 0, activation=L.ACT_FULL_RAY):
    """Time to the converged map, per scene.  The converged map is plain BP
    from the prior run until its largest belief change is below ref_tol
    (untimed).  Each method -- plain BP from the prior, BP warm-started by
    the network, and BP warm-started by a prediction of the prior everywhere
    (the method without the network) -- is then timed from its start until
    its map is within accept_tol of the converged map (mrf_infer_until,
    checked every iteration): the whole procedure (features, network,
    initial messages, iterations) with the incidence lists built
    beforehand.  One-time costs (the voxel CSR the warm start uses, the
    network's workspace) are paid before the timed runs."""
    torch = _torch()
    rows = []
    for w in workloads:
        m = L.MRFMap(w.params, activation=activation)
        for P, D in zip(w.poses, w.depths):
            m.add_view(P, D)
        m.infer(iters=1)  # incidence lists
        warm_start(m, net, sweeps)  # one-time costs, untimed
        m.reset_state()
        n_ref, d_ref = m.infer_converge(ref_tol, max_iters=ref_max_iters)
        Bref = m.beliefs()
        ref_dev = torch.from_numpy(Bref.reshape(-1)).cuda()
        rec = {"workload": w.name, "seed": w.seed, "ref_iters": n_ref, "ref_converged": d_ref < ref_tol}
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        lp = float(np.log(w.params.prior / (1 - w.params.prior)))
        for label in ("plain", "learned", "prior"):
            m.reset_state()
            torch.cuda.synchronize()
            ev[0].record()
            if label == "learned":
                warm_start(m, net, sweeps)
            elif label == "prior":
                m.warm_start(np.full((m.num_bricks, 512), lp, np.float32), sweeps)
            ev[1].record()
            n, dist = m.infer_until(ref_dev.data_ptr(), accept_tol, max_iters=max_iters,
                                    flags=0 if label == "plain" else L.INCREMENTAL)
            ev[2].record()
            torch.cuda.synchronize()
            B = m.beliefs()
            touched = (Bref > 0) | (B > 0)
            rec[label + "_iters"] = n
            rec[label + "_ms"] = ev[0].elapsed_time(ev[2])
            # the warm start alone (features, network, initial messages)
            rec[label + "_start_ms"] = ev[0].elapsed_time(ev[1])
            rec[label + "_reached"] = bool(dist <= accept_tol)
            rec[label + "_max_err"] = float(np.abs(B - Bref).max())
            rec[label + "_agree"] = float(((B > 0.5) == (Bref > 0.5))[touched].mean()) if touched.any() else 1.0
        # the network's three convolutions alone (mean of 5 calls on this
        # scene's features), and the bricks they cover
        feat = map_features(m)
        net.predict(feat)
        torch.cuda.synchronize()
        ev[0].record()
        for _ in range(5):
            net.predict(feat)
        ev[1].record()
        torch.cuda.synchronize()
        rec["net_forward_ms"] = ev[0].elapsed_time(ev[1]) / 5
        rec["n_bricks"] = int(m.num_bricks)
        rows.append(rec)
        m.close()
    return rows


def summarize(rows, accept_tol: float = 1e-3, agree_min: float = 0.999):
    """Speed-ups over the scenes whose converged map exists (the reference
    run converged) and that every method reached (within accept_tol, class
    agreement >= agree_min)."""
    ok = [r for r in rows if r["ref_converged"] and all(
        r[k + "_reached"] and r[k + "_max_err"] <= accept_tol and r[k + "_agree"] >= agree_min
        for k in ("plain", "learned", "prior"))]
    mean = lambda k: float(np.mean([r[k] for r in ok])) if ok else None
    out = {"scenes": len(rows), "scenes_ref_converged": sum(r["ref_converged"] for r in rows),
           "scenes_compared": len(ok)}
    for k in ("plain", "learned", "prior"):
        out[k + "_ms"] = mean(k + "_ms")
        out[k + "_start_ms"] = mean(k + "_start_ms")
        out[k + "_iters"] = mean(k + "_iters")
    if rows and "net_forward_ms" in rows[0]:
        # the convolutions' rate: 9072 multiply-adds per voxel (27 taps x
        # (4x16 + 16x16 + 16x1)), 512 voxels per brick
        out["net_forward_ms"] = float(np.mean([r["net_forward_ms"] for r in rows]))
        out["net_forward_tflops"] = float(np.mean([2 * 9072 * 512 * r["n_bricks"] / (r["net_forward_ms"] * 1e9)
                                                   for r in rows]))
    if ok:
        out["speedup_learned_vs_plain"] = out["plain_ms"] / out["learned_ms"]
        out["speedup_prior_vs_plain"] = out["plain_ms"] / out["prior_ms"]
        out["speedup_learned_vs_prior"] = out["prior_ms"] / out["learned_ms"]
        out["max_belief_err_vs_converged"] = {k: max(r[k + "_max_err"] for r in ok)
                                             for k in ("plain", "learned", "prior")}
        out["min_class_agreement"] = {k: min(r[k + "_agree"] for r in ok) for k in ("plain", "learned", "prior")}
    return out


def main(argv=None):
    """Train the warm-start network on plain-BP solutions of seeded scenes
    and write its parameters (fp32, mrf_net_num_params values)."""
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--scenes", type=int, default=200)
    ap.add_argument("--first-seed", type=int, default=1000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    a = ap.parse_args(argv)
    t0 = time.time()
    ws = scenes(range(a.first_seed, a.first_seed + a.scenes))
    t1 = time.time()
    print(f"{len(ws)} scenes in {t1 - t0:.1f} s", flush=True)
    feats, targets, weights = build_dataset(ws)
    t2 = time.time()
    print(f"{feats.shape[0]} training bricks in {t2 - t1:.1f} s", flush=True)
    net = WarmNet(seed=0)
    hist = net.train(feats, targets, weights, epochs=a.epochs, batch=a.batch, lr=a.lr)
    _torch().cuda.synchronize()
    t3 = time.time()
    net.save(a.out)
    print(json.dumps({"scenes": a.scenes, "bricks": int(feats.shape[0]), "epochs": a.epochs,
                      "loss_per_epoch": [round(h, 5) for h in hist], "scene_s": round(t1 - t0, 1),
                      "dataset_s": round(t2 - t1, 1), "train_s": round(t3 - t2, 1), "out": a.out}))


if __name__ == "__main__":
    main()
