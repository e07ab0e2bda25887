"""The SM-affine ray schedule an incidence build makes (host code of the
library, run without a GPU through mrf_test_region_lists).  A view's pixels
are cut into R runs of consecutive pixels holding equal shares of the BP
rays' Pre incidences, one run per SM; each run's longest rays up to the home
share of its incidences are served first by that SM's warps, the other rays
go to the view's leftover queue, longest first.  Checked on seeded random
ray records: every BP ray is scheduled exactly once, the runs follow the
pixel order and the work split, a run's home rays are its longest ones and
just reach the share, and both lists are longest first with pixel order
within a length."""
import ctypes as C

import numpy as np
import pytest

from mrfmap_gb300 import lib as L


def _lists(records, regions, share):
    lib = L.load()
    n = len(records)
    rec = np.ascontiguousarray(records, dtype=np.int32)
    home = np.zeros(max(n, 1), np.uint32)
    left = np.zeros(max(n, 1), np.uint32)
    starts = np.zeros(regions + 1, np.uint32)
    nh, nl = C.c_int64(), C.c_int64()
    u32 = C.POINTER(C.c_uint32)
    st = lib.mrf_test_region_lists(rec.ctypes.data_as(C.POINTER(C.c_int32)), n, regions, share,
                                   home.ctypes.data_as(u32), C.byref(nh), starts.ctypes.data_as(u32),
                                   left.ctypes.data_as(u32), C.byref(nl))
    assert st == 0, lib.mrf_last_error()
    return home[:nh.value].astype(np.int64), starts.astype(np.int64), left[:nl.value].astype(np.int64)


def _longest_first(ids, n_pre):
    """ids ordered by n_pre descending, then by pixel"""
    if len(ids) < 2:
        return True
    a, b = n_pre[ids[:-1]], n_pre[ids[1:]]
    return bool(np.all((a > b) | ((a == b) & (ids[:-1] < ids[1:]))))


@pytest.mark.parametrize("regions,share", [(16, 75), (152, 60), (7, 100), (5, 0), (1, 90)])
def test_region_lists_schedule_every_bp_ray_once(native_lib, regions, share):
    rng = np.random.default_rng(11 + regions)
    n = 6000
    n_pre = rng.integers(0, 2000, n)
    n_pre[rng.random(n) < 0.1] = 0
    n_pre[rng.random(n) < 0.05] = 40  # ties
    n_post = np.minimum(n_pre, rng.integers(0, 2000, n))
    kdyn = rng.integers(0, 2100, n)
    records = np.stack([n_pre, n_post, kdyn], 1)
    bp = (n_pre > 0) & (kdyn < n_post)
    home, starts, left = _lists(records, regions, share)

    scheduled = np.concatenate([home, left])
    assert len(scheduled) == int(bp.sum())
    assert np.array_equal(np.sort(scheduled), np.flatnonzero(bp))

    # the runs: each BP pixel's run from the BP work before it
    w = np.where(bp, n_pre, 0)
    work = int(w.sum())
    region = np.minimum(regions - 1, (np.cumsum(w) - w) * regions // max(work, 1))
    assert starts[0] == 0 and starts[regions] == len(home)
    assert np.all(np.diff(starts) >= 0)
    for r in range(regions):
        h = home[starts[r]:starts[r + 1]]
        members = np.flatnonzero(bp & (region == r))
        assert np.all(np.isin(h, members)), f"run {r}: a home ray from another run"
        assert _longest_first(h, n_pre)
        rest = np.setdiff1d(members, h)
        if len(h) and len(rest):
            assert n_pre[rest].max() <= n_pre[h[-1]], f"run {r}: a longer ray left out of its home rays"
        rw, hw = int(n_pre[members].sum()), int(n_pre[h].sum())
        assert hw * 100 >= rw * share, f"run {r}: home rays short of the share"
        if len(h):
            assert (hw - int(n_pre[h[-1]])) * 100 < rw * share, f"run {r}: more home rays than the share needs"
    assert _longest_first(left, n_pre)
    if share == 100:
        assert len(left) == 0
    if share == 0:
        assert len(home) == 0


def test_region_lists_reject_bad_records(native_lib):
    lib = L.load()
    rec = np.array([[10, 5, 2], [70000, 5, 2]], np.int32)
    home = np.zeros(2, np.uint32)
    left = np.zeros(2, np.uint32)
    starts = np.zeros(3, np.uint32)
    nh, nl = C.c_int64(), C.c_int64()
    u32 = C.POINTER(C.c_uint32)
    st = lib.mrf_test_region_lists(rec.ctypes.data_as(C.POINTER(C.c_int32)), 2, 2, 75, home.ctypes.data_as(u32),
                                   C.byref(nh), starts.ctypes.data_as(u32), left.ctypes.data_as(u32), C.byref(nl))
    assert st == 1 and b"65535" in lib.mrf_last_error()
    assert lib.mrf_test_region_lists(rec.ctypes.data_as(C.POINTER(C.c_int32)), 2, 0, 75, home.ctypes.data_as(u32),
                                     C.byref(nh), starts.ctypes.data_as(u32), left.ctypes.data_as(u32),
                                     C.byref(nl)) == 1
