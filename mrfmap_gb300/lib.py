"""ctypes binding of the C ABI (``include/mrfmap_gb300.h``).

This is the product path from Python: every call goes to
``libmrfmap_gb300.so``; there is no CPU fallback.  If the library is not
built, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .params import MapParams

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libmrfmap_gb300.so")

MRF_OK = 0
ACT_ENDPOINT = 0
ACT_FULL_RAY = 1
JACOBI = 1
INCREMENTAL = 2
FIX_PRE_RESET = 4
ASYNC = 8
PROFILE = 16
NO_GRAPH = 32
FULL_RAYS = 64
QUIET_PREFIX = 128
PRECISION_FP32 = 0
PRECISION_HALF_STREAMS = 1

_STATUS = {0: "MRF_OK", 1: "MRF_ERR_INVALID", 2: "MRF_ERR_CUDA", 3: "MRF_ERR_OOM",
           4: "MRF_ERR_CAPACITY", 5: "MRF_ERR_DEVICE", 6: "MRF_ERR_STATE"}

# every symbol declared in include/mrfmap_gb300.h
EXPORTS = ["mrf_create", "mrf_destroy", "mrf_release_cached_memory", "mrf_last_error", "mrf_add_view", "mrf_add_view_device",
           "mrf_set_pose", "mrf_infer", "mrf_infer_converge", "mrf_warm_start", "mrf_warm_start_device",
           "mrf_warm_features", "mrf_read_messages", "mrf_write_messages", "mrf_rebuild_logodds", "mrf_net_num_params", "mrf_net_workspace_bytes", "mrf_net_forward",
           "mrf_net_gradients", "mrf_net_adam",
           "mrf_ray_variants", "mrf_set_ray_variant",
           "mrf_autotune", "mrf_reset_state", "mrf_likelihood_view", "mrf_likelihood",
           "mrf_likelihood_device", "mrf_likelihood_device_noalloc", "mrf_num_bricks", "mrf_read_bricks", "mrf_read_logodds",
           "mrf_num_nodes", "mrf_read_nodes", "mrf_load_map", "mrf_view_incidences",
           "mrf_device_beliefs",
           "mrf_stats_get", "mrf_get_stream", "mrf_synchronize", "mrf_render", "mrf_render_view", "mrf_pixel_diagnostics", "mrf_add_view_camera",
           "mrf_view_camera", "mrf_set_memory_limit", "mrf_memory_in_use", "mrf_test_raise_device_error",
           "mrf_infer_until", "mrf_retire_view", "mrf_add_view_box", "mrf_autotune_flags",
           "mrf_set_precision", "mrf_set_home_share", "mrf_autotune_home_share", "mrf_get_tuning",
           "mrf_set_pair_variant", "mrf_test_brick_footprint", "mrf_test_fail_next_append",
           "mrf_test_region_lists"]

RENDER_EXPECTED_DEPTH = 0
RENDER_ACCURACY = 1
RENDER_SIMPLE_ACCURACY = 2
RENDER_OCC_THRESH = 3


class MrfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")
        self.status = status


class mrf_params(C.Structure):
    _fields_ = [("res", C.c_float), ("dims", C.c_float * 3), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("rows", C.c_int), ("cols", C.c_int),
                ("prior", C.c_float), ("max_iters", C.c_int), ("lookup_n", C.c_int),
                ("sigma_lut", C.POINTER(C.c_float)), ("bias_lut", C.POINTER(C.c_float)),
                ("occ_thresh", C.c_float), ("acc_thresh", C.c_float), ("activation", C.c_int),
                ("reserved", C.c_int * 7)]


class mrf_stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("n_views", "n_bricks", "n_rays", "n_inc_pre", "n_inc_post",
                                         "n_pairs", "n_pairs_active", "n_vox_touched", "iters_done",
                                         "kernel_launches")] + [("build_ms", C.c_double),
                                                                ("infer_ms", C.c_double),
                                                                ("kernel_ms", C.c_double * 4),
                                                                ("kernel_count", C.c_int64 * 4),
                                                                ("n_inc_dyn", C.c_int64),
                                                                ("n_pairs_dyn", C.c_int64),
                                                                ("n_rays_bp", C.c_int64),
                                                                ("n_inc_pre_bp", C.c_int64),
                                                                ("builds_full", C.c_int64),
                                                                ("builds_appended", C.c_int64),
                                                                ("n_inc_from_k4", C.c_int64),
                                                                ("n_loud_prefix", C.c_int64),
                                                                ("quiet_prefix_used", C.c_int64),
                                                                ("builds_oom_fallback", C.c_int64)]


_lib = None


def load(path: str | None = None):
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"{path} not built; run __graft_entry__.build() or python -m mrfmap_gb300._build")
    L = C.CDLL(path)
    vp, fp, ip, i64p = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_int64)
    sig = {
        "mrf_create": ([C.POINTER(mrf_params), C.POINTER(vp)], C.c_int),
        "mrf_destroy": ([vp], None),
        "mrf_release_cached_memory": ([], C.c_int),
        "mrf_last_error": ([], C.c_char_p),
        "mrf_add_view": ([vp, fp, fp, ip], C.c_int),
        "mrf_add_view_device": ([vp, fp, vp, ip], C.c_int),
        "mrf_set_pose": ([vp, C.c_int, fp], C.c_int),
        "mrf_infer": ([vp, ip, C.c_int, C.c_int, C.c_int], C.c_int),
        "mrf_infer_converge": ([vp, ip, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, ip, fp], C.c_int),
        "mrf_warm_start": ([vp, fp, C.c_int], C.c_int),
        "mrf_warm_start_device": ([vp, C.c_void_p, C.c_int], C.c_int),
        "mrf_warm_features": ([vp, C.c_void_p], C.c_int),
        "mrf_read_messages": ([vp, C.c_int, fp], C.c_int),
        "mrf_write_messages": ([vp, C.c_int, fp], C.c_int),
        "mrf_rebuild_logodds": ([vp], C.c_int),
        "mrf_net_num_params": ([], C.c_int64),
        "mrf_net_workspace_bytes": ([C.c_int64], C.c_int64),
        "mrf_net_forward": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "mrf_net_gradients": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "mrf_net_adam": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.c_float,
                          C.c_float, C.c_float, C.c_int, C.c_void_p], C.c_int),
        "mrf_ray_variants": ([], C.c_int),
        "mrf_set_ray_variant": ([vp, C.c_int], C.c_int),
        "mrf_autotune": ([vp, C.c_int, C.POINTER(C.c_double), C.c_int, ip], C.c_int),
        "mrf_reset_state": ([vp], C.c_int),
        "mrf_likelihood_view": ([vp, C.c_int, fp, fp], C.c_int),
        "mrf_likelihood": ([vp, fp, fp, fp, fp], C.c_int),
        "mrf_likelihood_device": ([vp, fp, vp, vp, vp], C.c_int),
        "mrf_likelihood_device_noalloc": ([vp, fp, vp, vp, vp], C.c_int),
        "mrf_num_bricks": ([vp, i64p], C.c_int),
        "mrf_read_bricks": ([vp, fp, fp, C.c_int64], C.c_int),
        "mrf_read_logodds": ([vp, fp, C.c_int64], C.c_int),
        "mrf_num_nodes": ([vp, C.c_int, i64p], C.c_int),
        "mrf_read_nodes": ([vp, C.c_int, fp, C.c_int64], C.c_int),
        "mrf_load_map": ([vp, fp, fp, C.c_int64], C.c_int),
        "mrf_view_incidences": ([vp, C.c_int, ip, C.POINTER(C.c_uint32), fp, fp, C.c_int64, i64p],
                                C.c_int),
        "mrf_device_beliefs": ([vp, C.POINTER(vp), i64p], C.c_int),
        "mrf_stats_get": ([vp, C.POINTER(mrf_stats)], C.c_int),
        "mrf_get_stream": ([vp, C.POINTER(vp)], C.c_int),
        "mrf_synchronize": ([vp], C.c_int),
        "mrf_render": ([vp, C.c_int, fp, fp, C.c_float, fp, fp, i64p], C.c_int),
        "mrf_render_view": ([vp, C.c_int, C.c_int, C.c_float, fp, fp, i64p], C.c_int),
        "mrf_pixel_diagnostics": ([vp, fp, C.c_int, C.c_int, fp, C.c_int64], C.c_int),
        "mrf_add_view_camera": ([vp, fp, fp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                 ip], C.c_int),
        "mrf_view_camera": ([vp, C.c_int, ip, ip, fp], C.c_int),
        "mrf_set_memory_limit": ([C.c_int64], C.c_int),
        "mrf_retire_view": ([vp, C.c_int], C.c_int),
        "mrf_set_precision": ([vp, C.c_int], C.c_int),
        "mrf_autotune_flags": ([vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int, ip], C.c_int),
        "mrf_set_home_share": ([vp, C.c_int], C.c_int),
        "mrf_autotune_home_share": ([vp, C.c_int, C.c_int, ip, C.c_int, C.POINTER(C.c_double), ip], C.c_int),
        "mrf_get_tuning": ([vp, ip, ip, ip], C.c_int),
        "mrf_set_pair_variant": ([vp, C.c_int], C.c_int),
        "mrf_add_view_box": ([vp, fp, fp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, ip, ip,
                              ip], C.c_int),
        "mrf_infer_until": ([vp, ip, C.c_int, C.c_int, C.c_void_p, C.c_float, C.c_int, C.c_int, ip, fp],
                            C.c_int),
        "mrf_memory_in_use": ([], C.c_int64),
        "mrf_test_raise_device_error": ([vp], C.c_int),
        "mrf_test_fail_next_append": ([vp, C.c_int], C.c_int),
        "mrf_test_region_lists": ([C.POINTER(C.c_int32), C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_uint32),
                                   i64p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), i64p], C.c_int),
        "mrf_test_brick_footprint": ([vp, C.c_int, C.c_int64, C.c_int64, C.POINTER(C.c_uint8), ip], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _check(st):
    if st != MRF_OK:
        raise MrfError(st, load().mrf_last_error().decode(errors="replace"))


def make_params(p: MapParams, activation: int = ACT_ENDPOINT):
    p.check()
    sig = _f32(p.sigma_lut)
    bias = _f32(p.bias_lut)
    s = mrf_params()
    s.res = p.res
    s.dims = (C.c_float * 3)(*[float(v) for v in p.dims])
    s.fx, s.fy, s.cx, s.cy = p.fx, p.fy, p.cx, p.cy
    s.rows, s.cols = p.rows, p.cols
    s.prior = p.prior
    s.max_iters = p.max_iters
    s.lookup_n = p.lookup_n
    s.sigma_lut = _fp(sig)
    s.bias_lut = _fp(bias)
    s.occ_thresh = p.occ_thresh
    s.acc_thresh = p.acc_thresh
    s.activation = activation
    return s, (sig, bias)


class MRFMap:
    """One occupancy map on the current CUDA device (C ABI handle)."""

    def __init__(self, params: MapParams, activation: int = ACT_ENDPOINT):
        self._L = load()
        self.params = params
        s, keep = make_params(params, activation)
        h = C.c_void_p()
        _check(self._L.mrf_create(C.byref(s), C.byref(h)))
        self._h = h
        self._keep = keep

    def close(self):
        if getattr(self, "_h", None):
            self._L.mrf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def add_view(self, pose, depth) -> int:
        vid = C.c_int()
        d = _f32(depth)
        if d.shape != (self.params.rows, self.params.cols):
            raise ValueError("depth image shape does not match params rows x cols")
        _check(self._L.mrf_add_view(self._h, _fp(_f32(pose)), _fp(d), C.byref(vid)))
        return vid.value

    def add_view_camera(self, pose, depth, fx: float, fy: float, cx: float, cy: float) -> int:
        """A view with its own camera; the depth image's shape is its size."""
        vid = C.c_int()
        d = _f32(depth)
        if d.ndim != 2:
            raise ValueError("depth image must be 2-D")
        _check(self._L.mrf_add_view_camera(self._h, _fp(_f32(pose)), _fp(d), d.shape[0], d.shape[1], fx, fy,
                                           cx, cy, C.byref(vid)))
        return vid.value

    def add_view_box(self, pose, depth, fx: float, fy: float, cx: float, cy: float, brick_lo, brick_hi) -> int:
        """A view with its own camera whose rays and bricks stay inside the
        scene box of bricks [brick_lo, brick_hi)."""
        vid = C.c_int()
        d = _f32(depth)
        lo = np.ascontiguousarray(brick_lo, dtype=np.int32)
        hi = np.ascontiguousarray(brick_hi, dtype=np.int32)
        _check(self._L.mrf_add_view_box(self._h, _fp(_f32(pose)), _fp(d), d.shape[0], d.shape[1], fx, fy, cx, cy,
                                        lo.ctypes.data_as(C.POINTER(C.c_int)), hi.ctypes.data_as(C.POINTER(C.c_int)),
                                        C.byref(vid)))
        return vid.value

    def view_camera(self, view: int):
        """(rows, cols, (fx, fy, cx, cy)) of a view."""
        r, c = C.c_int(), C.c_int()
        k = np.zeros(4, np.float32)
        _check(self._L.mrf_view_camera(self._h, view, C.byref(r), C.byref(c), _fp(k)))
        return r.value, c.value, tuple(float(x) for x in k)

    def add_view_device(self, pose, depth_dev_ptr: int) -> int:
        """A view whose depth image is already on the device: depth_dev_ptr
        must point at params.rows x params.cols floats (the map camera's
        image); views of other sizes go through add_view_camera."""
        vid = C.c_int()
        _check(self._L.mrf_add_view_device(self._h, _fp(_f32(pose)), C.c_void_p(depth_dev_ptr),
                                           C.byref(vid)))
        return vid.value

    def set_pose(self, view: int, pose):
        _check(self._L.mrf_set_pose(self._h, view, _fp(_f32(pose))))

    def retire_view(self, view: int):
        """Out of the iterated window; its messages stay in the log-odds."""
        _check(self._L.mrf_retire_view(self._h, view))

    def infer(self, ids=None, iters: int = 0, flags: int = 0):
        if ids is None:
            _check(self._L.mrf_infer(self._h, None, 0, iters, flags))
        else:
            a = np.ascontiguousarray(ids, dtype=np.int32)
            _check(self._L.mrf_infer(self._h, a.ctypes.data_as(C.POINTER(C.c_int)), len(a), iters, flags))

    def infer_converge(self, tol: float, max_iters: int = 0, ids=None, flags: int = 0,
                       check_every: int = 1):
        """Iterate until the largest belief change is below tol; returns
        (iterations run, last measured change)."""
        n = C.c_int()
        d = C.c_float()
        if ids is None:
            _check(self._L.mrf_infer_converge(self._h, None, 0, max_iters, tol, check_every, flags,
                                              C.byref(n), C.byref(d)))
        else:
            a = np.ascontiguousarray(ids, dtype=np.int32)
            _check(self._L.mrf_infer_converge(self._h, a.ctypes.data_as(C.POINTER(C.c_int)), len(a),
                                              max_iters, tol, check_every, flags, C.byref(n), C.byref(d)))
        return n.value, d.value

    def infer_until(self, target_dev_ptr: int, tol: float, max_iters: int = 0, ids=None, flags: int = 0,
                    check_every: int = 1):
        """Iterate until the largest |belief - target| is at most tol
        (target: a device array of n_bricks x 512 floats); returns
        (iterations run, last measured distance)."""
        n = C.c_int()
        d = C.c_float()
        a = None if ids is None else np.ascontiguousarray(ids, dtype=np.int32)
        _check(self._L.mrf_infer_until(self._h, None if a is None else a.ctypes.data_as(C.POINTER(C.c_int)),
                                       0 if a is None else len(a), max_iters, C.c_void_p(target_dev_ptr),
                                       tol, check_every, flags, C.byref(n), C.byref(d)))
        return n.value, d.value

    def warm_start(self, logodds, sweeps: int = 3):
        """Messages iterated at a predicted log-odds field [n_bricks, 512]
        held fixed; continue with flags=INCREMENTAL."""
        lo = np.ascontiguousarray(logodds, dtype=np.float32)
        if lo.size != self.num_bricks * 512:
            raise ValueError("logodds must hold n_bricks x 512 values")
        _check(self._L.mrf_warm_start(self._h, _fp(lo), sweeps))

    def warm_start_device(self, logodds_dev_ptr: int, sweeps: int = 3):
        _check(self._L.mrf_warm_start_device(self._h, C.c_void_p(logodds_dev_ptr), sweeps))

    def read_messages(self, view: int) -> np.ndarray:
        out = np.zeros((self.num_bricks, 512), np.float32)
        _check(self._L.mrf_read_messages(self._h, view, _fp(out)))
        return out

    def write_messages(self, view: int, dense):
        d = np.ascontiguousarray(dense, dtype=np.float32)
        if d.size != self.num_bricks * 512:
            raise ValueError("messages must hold n_bricks x 512 values")
        _check(self._L.mrf_write_messages(self._h, view, _fp(d)))

    def rebuild_logodds(self):
        _check(self._L.mrf_rebuild_logodds(self._h))

    def warm_features(self, feat_dev_ptr: int):
        """Writes [n_bricks, 512, 4] float features to a device buffer."""
        _check(self._L.mrf_warm_features(self._h, C.c_void_p(feat_dev_ptr)))

    def set_precision(self, mode: int):
        """PRECISION_FP32 (default) or PRECISION_HALF_STREAMS (fp16 lengths
        and ln q gathers in the ray kernel)."""
        _check(self._L.mrf_set_precision(self._h, mode))

    def set_ray_variant(self, variant: int):
        _check(self._L.mrf_set_ray_variant(self._h, variant))

    def autotune(self, reps: int = 3, flags: int = 0):
        """Times every ray-kernel variant on this map (iterations of the
        schedule in flags: JACOBI or Gauss-Seidel); keeps the fastest.
        Returns (chosen variant, ms per pass of each variant)."""
        nv = self._L.mrf_ray_variants()
        ms = np.zeros(nv, np.float64)
        ch = C.c_int()
        _check(self._L.mrf_autotune_flags(self._h, reps, flags, ms.ctypes.data_as(C.POINTER(C.c_double)), nv,
                                          C.byref(ch)))
        return ch.value, ms

    def set_home_share(self, percent: int):
        """Per cent of an SM region's incidences taken by its home blocks in
        the SM-region schedule (default 75); results do not change."""
        _check(self._L.mrf_set_home_share(self._h, percent))

    def autotune_home_share(self, shares=(60, 75, 90), reps: int = 3, flags: int = 0):
        """Times each home share on this map; keeps the fastest.  Returns
        (chosen share, ms per iteration of each share)."""
        sh = np.ascontiguousarray(shares, np.int32)
        ms = np.zeros(len(sh), np.float64)
        ch = C.c_int()
        _check(self._L.mrf_autotune_home_share(self._h, reps, flags, sh.ctypes.data_as(C.POINTER(C.c_int)),
                                               len(sh), ms.ctypes.data_as(C.POINTER(C.c_double)),
                                               C.byref(ch)))
        return ch.value, ms

    def set_pair_variant(self, variant: int):
        """Pair-reduction variant (0 or 1; the same results)."""
        _check(self._L.mrf_set_pair_variant(self._h, variant))

    def tuning(self):
        """(ray-kernel variant, home share, pair-reduction variant) in use."""
        v, h, p = C.c_int(), C.c_int(), C.c_int()
        _check(self._L.mrf_get_tuning(self._h, C.byref(v), C.byref(h), C.byref(p)))
        return v.value, h.value, p.value

    def reset_state(self):
        _check(self._L.mrf_reset_state(self._h))

    def synchronize(self):
        _check(self._L.mrf_synchronize(self._h))

    @property
    def num_bricks(self) -> int:
        n = C.c_int64()
        _check(self._L.mrf_num_bricks(self._h, C.byref(n)))
        return n.value

    def read_bricks(self, centres=None, beliefs=None):
        """Brick centres (n, 3) and beliefs (n, 512); pass preallocated
        float32 arrays (pinned host memory, e.g. numpy views of pinned
        torch tensors, makes the device-to-host copy run at full speed)."""
        n = self.num_bricks
        cen = np.zeros((n, 3), np.float32) if centres is None else centres
        bel = np.zeros((n, 512), np.float32) if beliefs is None else beliefs
        if cen.shape != (n, 3) or bel.shape != (n, 512) or cen.dtype != np.float32 or bel.dtype != np.float32 \
                or not cen.flags.c_contiguous or not bel.flags.c_contiguous:
            raise ValueError("read_bricks: outputs must be C-contiguous float32 of shapes (n, 3) and (n, 512)")
        _check(self._L.mrf_read_bricks(self._h, _fp(cen), _fp(bel), n))
        return cen, bel

    def beliefs(self):
        return self.read_bricks()[1]

    def logodds(self):
        n = self.num_bricks
        out = np.zeros((n, 512), np.float32)
        _check(self._L.mrf_read_logodds(self._h, _fp(out), n))
        return out

    def brick_coords(self) -> np.ndarray:
        cen, _ = self.read_bricks()
        return ((cen - 4) / 8).astype(np.int32)

    def nodes(self, level: int):
        n = C.c_int64()
        _check(self._L.mrf_num_nodes(self._h, level, C.byref(n)))
        out = np.zeros((n.value, 3), np.float32)
        _check(self._L.mrf_read_nodes(self._h, level, _fp(out), n.value))
        return out

    def likelihood(self, pose, depth, image: bool = True):
        img = np.zeros((self.params.rows, self.params.cols), np.float32) if image else None
        s = C.c_float()
        _check(self._L.mrf_likelihood(self._h, _fp(_f32(pose)), _fp(_f32(depth)),
                                      _fp(img) if image else None, C.byref(s)))
        return s.value, img

    def likelihood_view(self, view: int, image: bool = True):
        rows, cols, _ = self.view_camera(view)
        img = np.zeros((rows, cols), np.float32) if image else None
        s = C.c_float()
        _check(self._L.mrf_likelihood_view(self._h, view, _fp(img) if image else None, C.byref(s)))
        return s.value, img

    def likelihood_device(self, pose, depth_ptr: int, img_ptr: int | None, sum_ptr: int):
        _check(self._L.mrf_likelihood_device(self._h, _fp(_f32(pose)), C.c_void_p(depth_ptr),
                                             C.c_void_p(img_ptr) if img_ptr else None,
                                             C.c_void_p(sum_ptr)))

    def render(self, mode: int, pose, depth, threshold: float = -1.0):
        """Evaluation render at a pose: (image, score, label counts -1/0/1/2)."""
        img = np.zeros((self.params.rows, self.params.cols), np.float32)
        s = C.c_float()
        cnt = np.zeros(4, np.int64)
        _check(self._L.mrf_render(self._h, mode, _fp(_f32(pose)), _fp(_f32(depth)), threshold, _fp(img),
                                  C.byref(s), cnt.ctypes.data_as(C.POINTER(C.c_int64))))
        return img, s.value, cnt

    def render_view(self, mode: int, view: int, threshold: float = -1.0):
        rows, cols, _ = self.view_camera(view)
        img = np.zeros((rows, cols), np.float32)
        s = C.c_float()
        cnt = np.zeros(4, np.int64)
        _check(self._L.mrf_render_view(self._h, mode, view, threshold, _fp(img), C.byref(s),
                                       cnt.ctypes.data_as(C.POINTER(C.c_int64))))
        return img, s.value, cnt

    def pixel_diagnostics(self, pose, x: int, y: int, n_floats: int | None = None):
        """Per-voxel records of pixel (x, y)'s ray at a pose (the layout of
        mrf_pixel_diagnostics), parsed: dict of arrays s, belief, vox, w, vis,
        slot, local (n x 3)."""
        n_floats = n_floats or self.params.rows * self.params.cols
        buf = np.zeros(n_floats + (n_floats & 1), np.float32)  # 8-byte records need an even count
        _check(self._L.mrf_pixel_diagnostics(self._h, _fp(_f32(pose)), x, y, _fp(buf), n_floats))
        cnt = int(buf[n_floats - 1])
        rec = buf[:cnt * 10].reshape(cnt, 10)
        u64 = buf[:cnt * 10].view(np.uint64).reshape(cnt, 5)
        loc = rec[:, 8].copy().view(np.uint8).reshape(cnt, 4)[:, :3]
        return dict(s=rec[:, 0].copy(), belief=rec[:, 1].copy(), vox=u64[:, 1].copy(), w=rec[:, 4].copy(),
                    vis=rec[:, 5].copy(), slot=u64[:, 3].copy(), local=loc.astype(np.int32))

    def load_map(self, points, occupancies):
        pts = _f32(points).reshape(-1, 3)
        occ = _f32(occupancies).reshape(-1)
        if len(pts) != len(occ):
            raise ValueError("points and occupancies differ in length")
        _check(self._L.mrf_load_map(self._h, _fp(pts), _fp(occ), len(pts)))

    def view_incidences(self, view: int):
        """Per-pixel meta (rows*cols, 5) and the view's incidences in ray order."""
        n = C.c_int64()
        rows, cols, _ = self.view_camera(view)
        meta = np.zeros((rows * cols, 5), np.int32)
        _check(self._L.mrf_view_incidences(self._h, view, meta.ctypes.data_as(C.POINTER(C.c_int)),
                                           None, None, None, 0, C.byref(n)))
        k = n.value
        vox = np.zeros(max(k, 1), np.uint32)
        ln = np.zeros(max(k, 1), np.float32)
        mu = np.zeros(max(k, 1), np.float32)
        _check(self._L.mrf_view_incidences(self._h, view, None,
                                           vox.ctypes.data_as(C.POINTER(C.c_uint32)), _fp(ln), _fp(mu),
                                           k, C.byref(n)))
        return meta, vox[:k], ln[:k], mu[:k]

    def stream(self) -> int:
        s = C.c_void_p()
        _check(self._L.mrf_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def stats(self) -> dict:
        st = mrf_stats()
        _check(self._L.mrf_stats_get(self._h, C.byref(st)))
        out = {k: getattr(st, k) for k, _ in st._fields_}
        out["kernel_ms"] = list(st.kernel_ms)
        out["kernel_count"] = list(st.kernel_count)
        return out
