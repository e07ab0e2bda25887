"""Repack the reference's own input fixture into tests/golden/coffin_world.npz.

The reference ships one realistic input set for this path: 13 depth frames
and body poses (``data/depth_{k}.bin``, ``data/pose_{k}.bin``, Eigen binary:
int64 rows, int64 cols, column-major float32) and the map/sensor config
``config/coffin_world_640.yaml``.  Its viewer test
(``src/testMRFMapViewer.cpp:18-67``) loads frames 0..11, turns each body
pose into a camera pose with ``cam_in_body`` (``pose * cam_in_body``), keeps
the frames a ``KeyframeSelector(0.1, 0.1)`` accepts, and for each keyframe
adds the camera and runs ``perform_inference`` (``src/Viewer.cpp:44-61``).

This script stores, for the parity tests (which must run where the
reference tree is absent):
  depth      (13, 480, 640) float32, row-major, NaN kept
  pose       (13, 4, 4) float32, row-major camera-to-world (cam_in_body applied)
  keyframe   (13,) bool: the viewer's keyframe decisions over frames 0..11
             (frame 12 is not loaded by the viewer test: False)
  yaml       the config file's text

Usage (in a tree where the reference is present):
    python tests/golden/make_coffin_world.py [REFERENCE_DIR]
REFERENCE_DIR defaults to $MRFMAP_REFERENCE_DIR, else /root/reference.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "coffin_world.npz")
N_FRAMES = 13
VIEWER_FRAMES = 12  # src/testMRFMapViewer.cpp: num_cams_ = 12


def read_eigen_binary(path):
    raw = open(path, "rb").read()
    r, c = np.frombuffer(raw[:16], dtype=np.int64)
    return np.frombuffer(raw[16:16 + 4 * r * c], np.float32).reshape(int(c), int(r)).T.copy()


def _log_se3_norms(T):
    """(|rotation vector|, |translation part of log(T)|) of a rigid motion."""
    R, p = T[:3, :3].astype(np.float64), T[:3, 3].astype(np.float64)
    v = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    sn = 0.5 * np.linalg.norm(v)
    t = np.arctan2(sn, 0.5 * (np.trace(R) - 1.0))
    if t < 1e-9:
        return 0.0, float(np.linalg.norm(p))
    w = t * v / (2.0 * sn)
    W = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    Vinv = np.eye(3) - 0.5 * W + (1.0 - t / (2.0 * np.tan(t / 2.0))) * (W @ W) / (t * t)
    return float(t), float(np.linalg.norm(Vinv @ p))


def keyframes(poses, rot_thresh=0.1, trans_thresh=0.1):
    """KeyframeSelector::is_keyframe (src/KeyframeSelector.cpp:74-99) in order."""
    kf, out = [], []
    for P in poses:
        ok = True
        for Q in reversed(kf):
            rot, trans = _log_se3_norms(np.linalg.inv(P.astype(np.float64)) @ Q)
            if trans < trans_thresh and rot < rot_thresh:
                ok = False
                break
        if ok:
            kf.append(P)
        out.append(ok)
    return out


def cam_in_body(yaml_text):
    lines = yaml_text.splitlines()
    i = next(k for k, l in enumerate(lines) if l.strip().startswith("cam_in_body:"))
    txt = ""
    for l in lines[i:]:
        txt += l.split("#", 1)[0]
        if "]" in l:
            break
    vals = [float(t) for t in txt.split("[", 1)[1].split("]", 1)[0].split(",") if t.strip()]
    return np.array(vals, np.float64).reshape(4, 4)  # listed row by row


def main(ref):
    yaml_text = open(os.path.join(ref, "config", "coffin_world_640.yaml")).read()
    C = cam_in_body(yaml_text)
    depth, pose = [], []
    for k in range(N_FRAMES):
        depth.append(read_eigen_binary(os.path.join(ref, "data", f"depth_{k}.bin")))
        body = read_eigen_binary(os.path.join(ref, "data", f"pose_{k}.bin")).astype(np.float64)
        pose.append((body @ C).astype(np.float32))
    kf = keyframes(pose[:VIEWER_FRAMES]) + [False] * (N_FRAMES - VIEWER_FRAMES)
    np.savez_compressed(OUT, depth=np.stack(depth), pose=np.stack(pose), keyframe=np.array(kf),
                        yaml=np.array(yaml_text))
    print(f"wrote {OUT}: {N_FRAMES} frames, keyframes {np.flatnonzero(kf).tolist()}")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MRFMAP_REFERENCE_DIR", "/root/reference")
    main(ref)
