"""ctypes wrapper of the CPU oracle (``mrf_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the checker; the product path
never touches it.  Parity against the reference itself is unpinned (see the
header of ``mrf_oracle.c``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libmrf_oracle.so")

ACT_ENDPOINT = 0
ACT_FULL_RAY = 1
JACOBI = 1
INCREMENTAL = 2
FIX_PRE_RESET = 4


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "mrf_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "mrf_oracle.h"))):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB


class _Params(C.Structure):
    _fields_ = [("res", C.c_float), ("dims", C.c_float * 3), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("rows", C.c_int), ("cols", C.c_int),
                ("prior", C.c_float), ("lookup_n", C.c_int), ("n_tiles_u", C.c_int),
                ("n_tiles_v", C.c_int), ("sigma_lut", C.POINTER(C.c_float)),
                ("bias_lut", C.POINTER(C.c_float))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        vp, fp, ip = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(_Params)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_add_view.argtypes = [vp, fp, fp, C.c_int]
        L.orc_add_view.restype = C.c_int
        L.orc_add_view_camera.argtypes = [vp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                          C.c_float, C.c_float]
        L.orc_add_view_camera.restype = C.c_int
        L.orc_add_view_box.argtypes = [vp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                       C.c_float, C.c_float, ip, ip]
        L.orc_add_view_box.restype = C.c_int
        L.orc_view_pixels.argtypes = [vp, C.c_int]
        L.orc_view_pixels.restype = C.c_int
        L.orc_set_pose.argtypes = [vp, C.c_int, fp, C.c_int]
        L.orc_num_views.argtypes = [vp]
        L.orc_num_bricks.argtypes = [vp]
        L.orc_brick_coords.argtypes = [vp, ip]
        L.orc_brick_dims.argtypes = [vp, ip]
        L.orc_infer.argtypes = [vp, ip, C.c_int, C.c_int, C.c_int]
        L.orc_get_beliefs.argtypes = [vp, fp]
        L.orc_get_beliefs_f64.argtypes = [vp, C.POINTER(C.c_double)]
        L.orc_get_logodds_f64.argtypes = [vp, C.POINTER(C.c_double)]
        L.orc_set_beliefs.argtypes = [vp, fp]
        L.orc_view_num_incidences.argtypes = [vp, C.c_int]
        L.orc_view_num_incidences.restype = C.c_int64
        L.orc_view_trace.argtypes = [vp, C.c_int, ip, C.POINTER(C.c_int64), ip, ip, fp, fp,
                                     C.POINTER(C.c_ubyte), C.POINTER(C.c_double)]
        L.orc_trace_pixel.argtypes = [vp, fp, C.c_int, C.c_int, ip, fp, fp, C.c_int]
        L.orc_likelihood.argtypes = [vp, fp, fp, fp]
        L.orc_likelihood.restype = C.c_double
        L.orc_render.argtypes = [vp, C.c_int, fp, fp, C.c_float, fp, C.POINTER(C.c_int64)]
        L.orc_build_all.argtypes = [vp]
        L.orc_retire_view.argtypes = [vp, C.c_int]
        L.orc_update_camera.argtypes = [vp, C.c_int, C.c_int]
        L.orc_update_camera.restype = C.c_int64
        L.orc_last_updates.argtypes = [vp]
        L.orc_last_updates.restype = C.c_int64
        L.orc_insert_logodds.argtypes = [vp, fp, fp, C.c_float, C.c_float, C.c_float, C.c_float,
                                         C.POINTER(C.c_double)]
        L.orc_insert_logodds.restype = C.c_int64
        _lib = L
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t=C.c_float):
    return a.ctypes.data_as(C.POINTER(t))


class OracleMap:
    """FP64 host BP map over the same params as the product."""

    def __init__(self, params, threads: int = 1):
        self._L = lib()
        self.params = params
        self._sig = _f(params.sigma_lut)
        self._bias = _f(params.bias_lut)
        p = _Params()
        p.res = params.res
        p.dims = (C.c_float * 3)(*params.dims)
        p.fx, p.fy, p.cx, p.cy = params.fx, params.fy, params.cx, params.cy
        p.rows, p.cols = params.rows, params.cols
        p.prior = params.prior
        p.lookup_n = params.lookup_n
        p.n_tiles_u, p.n_tiles_v = params.n_tiles_u, params.n_tiles_v
        p.sigma_lut = _ptr(self._sig)
        p.bias_lut = _ptr(self._bias)
        self._p = p
        self._h = self._L.orc_create(C.byref(p))
        self._L.orc_set_threads(threads)

    def close(self):
        if self._h:
            self._L.orc_destroy(self._h)
            self._h = None

    __del__ = close

    def add_view(self, pose, depth, policy=ACT_ENDPOINT) -> int:
        return self._L.orc_add_view(self._h, _ptr(_f(pose)), _ptr(_f(depth)), policy)

    def add_view_camera(self, pose, depth, rows, cols, fx, fy, cx, cy, policy=ACT_ENDPOINT) -> int:
        d = _f(depth)
        assert d.size == rows * cols
        return self._L.orc_add_view_camera(self._h, _ptr(_f(pose)), _ptr(d), policy, rows, cols, fx, fy, cx, cy)

    def add_view_box(self, pose, depth, rows, cols, fx, fy, cx, cy, brick_lo, brick_hi, policy=ACT_ENDPOINT) -> int:
        d = _f(depth)
        assert d.size == rows * cols
        lo = np.ascontiguousarray(brick_lo, np.int32)
        hi = np.ascontiguousarray(brick_hi, np.int32)
        v = self._L.orc_add_view_box(self._h, _ptr(_f(pose)), _ptr(d), policy, rows, cols, fx, fy, cx, cy,
                                     _ptr(lo, C.c_int), _ptr(hi, C.c_int))
        if v < 0:
            raise ValueError("bad scene box")
        return v

    def set_pose(self, view, pose, policy=ACT_ENDPOINT):
        return self._L.orc_set_pose(self._h, view, _ptr(_f(pose)), policy)

    @property
    def num_bricks(self) -> int:
        return self._L.orc_num_bricks(self._h)

    def brick_coords(self) -> np.ndarray:
        out = np.zeros((self.num_bricks, 3), np.int32)
        self._L.orc_brick_coords(self._h, _ptr(out, C.c_int))
        return out

    def infer(self, ids=None, iters=None, flags=0):
        n = self._L.orc_num_views(self._h)
        ids = np.arange(n, dtype=np.int32) if ids is None else np.asarray(ids, np.int32)
        iters = self.params.max_iters if iters is None else iters
        self._L.orc_infer(self._h, _ptr(ids, C.c_int), len(ids), iters, flags)

    def retire_view(self, view: int):
        """Out of the iterated window; its messages stay in the log-odds."""
        self._L.orc_retire_view(self._h, view)

    def build_all(self):
        """Incidence lists of every view (views built in parallel)."""
        self._L.orc_build_all(self._h)

    def update_camera(self, view: int, flags: int = 0) -> int:
        """One Gauss-Seidel camera update of ``view`` (messages kept);
        returns the Post incidences it processed."""
        n = self._L.orc_update_camera(self._h, view, flags)
        if n < 0:
            raise ValueError("bad view")
        return n

    @property
    def last_updates(self) -> int:
        return self._L.orc_last_updates(self._h)

    def beliefs(self) -> np.ndarray:
        out = np.zeros((self.num_bricks, 512), np.float64)
        self._L.orc_get_beliefs_f64(self._h, _ptr(out, C.c_double))
        return out

    def logodds(self) -> np.ndarray:
        out = np.zeros((self.num_bricks, 512), np.float64)
        self._L.orc_get_logodds_f64(self._h, _ptr(out, C.c_double))
        return out

    def set_beliefs(self, b):
        self._L.orc_set_beliefs(self._h, _ptr(_f(b)))

    def view_trace(self, view):
        ninc = self._L.orc_view_num_incidences(self._h, view)
        npx = self._L.orc_view_pixels(self._h, view)
        pix = np.zeros(npx, np.int32)
        off = np.zeros(npx, np.int64)
        meta = np.zeros((npx, 5), np.int32)
        vox = np.zeros(max(ninc, 1), np.int32)
        ln = np.zeros(max(ninc, 1), np.float32)
        s = np.zeros(max(ninc, 1), np.float32)
        run = np.zeros(max(ninc, 1), np.uint8)
        mu = np.zeros(max(ninc, 1), np.float64)
        nr = self._L.orc_view_trace(self._h, view, _ptr(pix, C.c_int), _ptr(off, C.c_int64),
                                    _ptr(meta, C.c_int), _ptr(vox, C.c_int), _ptr(ln), _ptr(s),
                                    _ptr(run, C.c_ubyte), _ptr(mu, C.c_double))
        return dict(pix=pix[:nr], off=off[:nr], meta=meta[:nr], vox=vox[:ninc], len=ln[:ninc],
                    s=s[:ninc], run=run[:ninc], mu=mu[:ninc])

    def trace_pixel(self, pose, x, y, max_n=1 << 16):
        vox = np.zeros(max_n, np.int32)
        ln = np.zeros(max_n, np.float32)
        s = np.zeros(max_n, np.float32)
        n = self._L.orc_trace_pixel(self._h, _ptr(_f(pose)), x, y, _ptr(vox, C.c_int), _ptr(ln),
                                    _ptr(s), max_n)
        n = min(n, max_n)
        return vox[:n], ln[:n], s[:n]

    def render(self, mode, pose, depth, thresh):
        img = np.zeros((self.params.rows, self.params.cols), np.float32)
        cnt = np.zeros(4, np.int64)
        self._L.orc_render(self._h, mode, _ptr(_f(pose)), _ptr(_f(depth)), thresh, _ptr(img),
                           cnt.ctypes.data_as(C.POINTER(C.c_int64)))
        return img, cnt

    def likelihood(self, pose, depth):
        img = np.zeros((self.params.rows, self.params.cols), np.float32)
        tot = self._L.orc_likelihood(self._h, _ptr(_f(pose)), _ptr(_f(depth)), _ptr(img))
        return tot, img

    def insert_logodds(self, pose, depth, logodds=None, l_hit=0.85, l_miss=-0.4, l_min=-2.0, l_max=3.5):
        """Classic log-odds ray insertion (miss along the ray, hit at the
        endpoint voxel, clamped; OctoMap's default parameters) of one depth
        image into ``logodds`` (one float64 per active voxel, updated in
        place; zeros when None).  A CPU baseline, not part of MRFMap.
        Returns (voxel updates, logodds)."""
        if logodds is None:
            logodds = np.zeros(self.num_bricks * 512, np.float64)
        n = self._L.orc_insert_logodds(self._h, _ptr(_f(pose)), _ptr(_f(depth)), l_hit, l_miss, l_min,
                                       l_max, _ptr(logodds, C.c_double))
        return int(n), logodds
