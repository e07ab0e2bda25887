"""Error paths of the C ABI, each raised on the host (no GPU fault):

* MRF_ERR_OOM: a bound on the device memory the maps may hold
  (mrf_set_memory_limit) refuses to grow a buffer; the map stays usable and,
  once the bound is lifted, gives the same beliefs as a map never bounded.
* MRF_ERR_DEVICE: the map's device error flag (set by a traversal kernel on a
  ray longer than 65532 incidences) raised from the host by a test hook; the
  next incidence-list build fails, clears it, and the build after succeeds.
* MRF_ERR_CAPACITY: a brick pool whose voxel ids would pass 32 bits
  (8.6 M bricks of a 205^3 brick grid activated by load_map), refused before
  the pool is allocated.

The reference prints and carries on in all three cases
(src/GVDBInference.cpp:31-37 checks CUDA calls with cudaCheck(..., false)).
"""
import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic
from mrfmap_gb300.params import MapParams

pytestmark = pytest.mark.gpu

OOM, CAPACITY, DEVICE = 3, 4, 5


def _map(w, views):
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for k in views:
        m.add_view(w.poses[k], w.depths[k])
    return m


def test_memory_limit_gives_oom_and_recovers(native_lib):
    lib = L.load()
    w = synthetic.small_room(0)
    a = _map(w, range(5))
    a.infer()
    ref = a.beliefs()
    a.close()
    b = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    try:
        assert lib.mrf_set_memory_limit(lib.mrf_memory_in_use() + (1 << 20)) == 0
        with pytest.raises(L.MrfError) as e:
            for k in range(5):
                b.add_view(w.poses[k], w.depths[k])
        assert e.value.status == OOM and "memory limit" in str(e.value)
    finally:
        assert lib.mrf_set_memory_limit(0) == 0
    n_added = b.stats()["n_views"]
    for k in range(n_added, 5):
        b.add_view(w.poses[k], w.depths[k])
    b.infer()
    np.testing.assert_array_equal(b.beliefs(), ref)
    b.close()
    assert lib.mrf_set_memory_limit(-1) == 1  # MRF_ERR_INVALID


def test_memory_limit_during_the_build(native_lib):
    """The bound hit inside the incidence-list build of mrf_infer."""
    lib = L.load()
    w = synthetic.small_room(1)
    m = _map(w, range(5))
    try:
        assert lib.mrf_set_memory_limit(lib.mrf_memory_in_use() + (256 << 10)) == 0
        with pytest.raises(L.MrfError) as e:
            m.infer()
        assert e.value.status == OOM
    finally:
        lib.mrf_set_memory_limit(0)
    m.infer()
    ref = _map(w, range(5))
    ref.infer()
    np.testing.assert_array_equal(m.beliefs(), ref.beliefs())
    m.close()
    ref.close()


def test_device_error_flag_fails_the_next_build(native_lib):
    lib = L.load()
    w = synthetic.small_room(2)
    m = _map(w, range(4))
    m.infer(iters=2)
    assert lib.mrf_test_raise_device_error(m.handle) == 0
    m.add_view(w.poses[4], w.depths[4])   # the view set changed: the next call builds
    with pytest.raises(L.MrfError) as e:
        m.infer()
    assert e.value.status == DEVICE
    # flag cleared: the build runs (from the prior, as the fresh map below;
    # mrf_infer alone would keep the log-odds of the two iterations above)
    m.reset_state()
    m.infer()
    ref = _map(w, range(5))
    ref.infer()
    np.testing.assert_array_equal(m.beliefs(), ref.beliefs())
    m.close()
    ref.close()


def test_capacity_of_32_bit_voxel_ids(native_lib):
    # 1632 voxels per axis -> 205^3 = 8.6 M bricks > 2^32 / 512 voxel ids
    p = MapParams(res=0.1, dims=(163.2, 163.2, 163.2), rows=20, cols=20, fx=20.0, fy=20.0,
                  cx=10.0, cy=10.0, prior=0.1)
    m = L.MRFMap(p)
    nb = 205
    # a point on a brick corner activates the 2x2x2 bricks around it
    c = np.arange(1, nb, 2, dtype=np.float32) * 8
    c = np.append(c, np.float32(8 * nb - 8)) if (nb - 1) % 2 else c
    pts = np.stack(np.meshgrid(c, c, c, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    with pytest.raises(L.MrfError) as e:
        m.load_map(pts, np.full(len(pts), 0.5, np.float32))
    assert e.value.status == CAPACITY
    assert m.num_bricks == 0
    # the map is still usable for a map that fits
    m.load_map(np.array([[100.5, 100.5, 100.5]], np.float32), np.array([0.9], np.float32))
    assert m.num_bricks == 1
    m.close()


def test_capacity_of_32_bit_incidence_indices(native_lib):
    """Copies of one 640x480 1 cm view, enough for ~4.4 G incidences: the
    build counts them in 64 bits and refuses before forming any 32-bit
    offset (only the per-pixel counts are allocated by then).  With the
    copies retired the map builds and iterates normally."""
    w = synthetic.full_room(1, n_frames=1)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    m.add_view(w.poses[0], w.depths[0])
    m.infer(iters=1)
    per_view = m.stats()["n_inc_pre"]
    copies = int(4.4e9 // per_view) + 2
    for _ in range(copies - 1):
        m.add_view(w.poses[0], w.depths[0])
    with pytest.raises(L.MrfError) as e:
        m.infer(iters=1)
    assert e.value.status == CAPACITY and "32-bit incidence" in str(e.value)
    for k in range(1, copies):
        m.retire_view(k)
    m.infer(iters=2)
    st = m.stats()
    assert st["n_inc_pre"] == per_view
    assert np.isfinite(m.beliefs()).all()
    m.close()
