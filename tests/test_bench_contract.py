"""bench.py's JSON-line contract, checked on the CPU through the reference arm
(the FP64 oracle port timed on the host cores; no GPU needed)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run("--impl", "reference", "--workload", "small", "--steps", "2", "--warmup", "1")
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["higher_is_better"] is True and d["unit"] == "updates/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["unit"] == d["unit"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("small_room")
    # the same config object as the GPU arm's line (same function, same args)
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.workload_config(bench.workload("small"), "fullray", 1)
    assert d["views_held"] == 5 and "camera update" in d["step"]


def test_cpu_baselines_of_our_line():
    """The cpu_baseline and cpu_insertion objects of our arm's line (the same
    function runs inside bench.py's GPU arm)."""
    sys.path.insert(0, ROOT)
    import bench
    w = bench.workload("small")
    cpu, ins = bench.cpu_baselines(w, "fullray", 2)
    assert "error" not in ins, ins
    assert cpu["kind"] == "port" and cpu["unit"] == bench.UNIT and cpu["value"] > 0 and cpu["cores"] >= 1
    assert "holding 5 of 5 keyframes" in cpu["sample"] and "sweep of 5 camera updates" in cpu["sample"]
    assert ins["unit"] == "voxel updates/s" and ins["value"] > 0 and ins["rays_per_s"] > 0
    assert "error" not in ins and ins["cores"] == 1
    json.dumps({"cpu_baseline": cpu, "cpu_insertion": ins})


def test_ray_kernel_bytes_of_both_paths():
    """The ray kernel's algorithmic bytes per call: every iteration over the
    whole Pre ranges on the full path; two such iterations, the quiet sums
    and the fast iterations (from k4 plus the loud prefix entries) when the
    call took the fast path."""
    import bench
    st = {"n_inc_pre_bp": 1000, "n_inc_from_k4": 200, "n_loud_prefix": 50, "n_inc_dyn": 150,
          "n_rays_bp": 10, "quiet_prefix_used": 0}
    full = 12 * 1000 + 8 * 150 + 16 * 10
    assert bench.ray_kernel_bytes(st, 20) == 20 * full
    assert bench.ray_kernel_bytes(st, 20, half=True) == 20 * (8 * 1000 + 8 * 150 + 16 * 10)
    st["quiet_prefix_used"] = 1
    quiet = 12 * 800 + 16 * 10
    fast = 12 * 200 + 14 * 50 + 8 * 150 + 36 * 10
    assert bench.ray_kernel_bytes(st, 20) == 2 * full + quiet + 18 * fast
    assert bench.ray_kernel_bytes(st, 2) == 2 * full
