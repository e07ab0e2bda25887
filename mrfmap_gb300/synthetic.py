"""Seeded synthetic depth scenes (rooms with boxes and spheres).

The reference publishes no dataset for its benchmarks; these scenes stand in
with the shapes, sizes and noise model of the benchmark workloads:

* ``small``  -- room 4x4x3 m, 6 boxes, 4 cm voxels, 5 frames 160x120
  (fx=fy=120, cx=80, cy=60) on a 1.5 m circle at 1.2 m height aimed at the
  room centre with +-5 deg yaw jitter, 10 BP iterations.
* ``full``   -- room 6x6x3 m, 20 boxes + 3 spheres, 1 cm voxels, 13 frames
  640x480 (fx=fy=525, cx=320, cy=240) on a seeded arc, max range 5 m,
  20 BP iterations.

Depth is an analytic z-depth ray cast through pixel centres plus Gaussian
noise sigma(z) = 0.002 + 0.0012 z^2, with 2 % of pixels dropped to 0.  The
sensor model handed to BP is the same polynomial (``const_sigmasq_poly``
``[0.002, 0, 0.0012]``, bias 0), the prior is 0.1.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .params import MapParams


@dataclass
class Scene:
    room: np.ndarray                     # (6,) xmin ymin zmin xmax ymax zmax, seen from inside
    boxes: np.ndarray                    # (n, 6) axis-aligned solids
    spheres: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))


def look_at(eye, target, yaw_jitter_rad: float = 0.0) -> np.ndarray:
    """Camera-to-world pose (x right, y down, z forward), row-major 4x4."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    if yaw_jitter_rad:
        c, s = np.cos(yaw_jitter_rad), np.sin(yaw_jitter_rad)
        f = np.array([c * f[0] - s * f[1], s * f[0] + c * f[1], f[2]])
    f /= np.linalg.norm(f)
    up = np.array([0.0, 0.0, 1.0])
    x = np.cross(f, up)
    x /= np.linalg.norm(x)
    y = np.cross(f, x)
    P = np.eye(4)
    P[:3, 0], P[:3, 1], P[:3, 2], P[:3, 3] = x, y, f, eye
    return P.astype(np.float32)


def _ray_dirs(params: MapParams, pose: np.ndarray):
    H, W = params.rows, params.cols
    fx, fy, cx, cy = params.fx, params.fy, params.cx, params.cy
    xs = (np.arange(W) + 0.5 - cx) / fx
    ys = (np.arange(H) + 0.5 - cy) / fy
    rc = np.stack(np.broadcast_arrays(xs[None, :], ys[:, None], np.ones((H, W))), -1)
    R = pose[:3, :3].astype(np.float64)
    return rc @ R.T  # unnormalised: z component in the camera frame is 1


def render_depth(scene: Scene, params: MapParams, pose: np.ndarray) -> np.ndarray:
    """Noise-free z-depth image (H, W) of the scene from ``pose``."""
    d = _ray_dirs(params, pose).reshape(-1, 3)
    o = pose[:3, 3].astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
        # room seen from inside: exit parameter of the slab intersection
        lo = (scene.room[:3] - o) * inv
        hi = (scene.room[3:] - o) * inv
        t = np.min(np.maximum(lo, hi), axis=1)
        for b in scene.boxes:
            l = (b[:3] - o) * inv
            h = (b[3:] - o) * inv
            tn = np.max(np.minimum(l, h), axis=1)
            tf = np.min(np.maximum(l, h), axis=1)
            hit = (tn <= tf) & (tn > 0)
            t = np.where(hit & (tn < t), tn, t)
        for s in scene.spheres:
            oc = o - s[:3]
            a = np.einsum("ij,ij->i", d, d)
            bq = 2.0 * d @ oc
            c = oc @ oc - s[3] ** 2
            disc = bq * bq - 4 * a * c
            ok = disc >= 0
            tt = (-bq - np.sqrt(np.where(ok, disc, 0))) / (2 * a)
            hit = ok & (tt > 0)
            t = np.where(hit & (tt < t), tt, t)
    return t.reshape(params.rows, params.cols).astype(np.float32)


def add_noise(depth: np.ndarray, rng: np.random.Generator, dropout: float = 0.02,
              max_range: float | None = None) -> np.ndarray:
    sig = 0.002 + 0.0012 * depth.astype(np.float64) ** 2
    out = depth + rng.standard_normal(depth.shape) * sig
    out = out.astype(np.float32)
    out[rng.random(depth.shape) < dropout] = 0.0
    if max_range is not None:
        out[out > max_range] = 0.0
    return out


def _boxes(rng, n, half_xy, zmax, keep_out):
    out = []
    while len(out) < n:
        side = rng.uniform(0.2, 1.0, 3)
        c = np.array([rng.uniform(-half_xy + 0.6, half_xy - 0.6),
                      rng.uniform(-half_xy + 0.6, half_xy - 0.6), side[2] / 2])
        b = np.concatenate([c - side / 2, c + side / 2])
        if b[5] > zmax:
            continue
        if any(np.all(k >= b[:3] - 0.1) and np.all(k <= b[3:] + 0.1) for k in keep_out):
            continue
        out.append(b)
    return np.array(out)


def sensor_params(params: MapParams) -> MapParams:
    params.set_const_polys([0.002, 0.0, 0.0012], [0.0, 0.0, 0.0])
    return params


@dataclass
class Workload:
    name: str
    params: MapParams
    poses: list
    depths: list
    seed: int
    cams: list | None = None  # per view (fx, fy, cx, cy) when views differ in camera
    scene: Scene | None = None


def small_room(seed: int = 0, n_frames: int = 5, rows: int = 120, cols: int = 160) -> Workload:
    """Room 4x4x3 m, 6 boxes, 4 cm voxels, 5 frames 160x120."""
    rng = np.random.default_rng(seed)
    p = MapParams(res=0.04, dims=(4.0, 4.0, 3.0), rows=rows, cols=cols,
                  fx=120.0 * cols / 160, fy=120.0 * cols / 160, cx=cols / 2, cy=rows / 2,
                  prior=0.1, max_iters=10)
    sensor_params(p)
    eps = p.res / 2
    room = np.array([-2 + eps, -2 + eps, eps, 2 - eps, 2 - eps, 3 - eps])
    target = np.array([0.0, 0.0, 1.5])
    phase = rng.uniform(0, 2 * np.pi)
    eyes = [np.array([1.5 * np.cos(phase + 2 * np.pi * k / n_frames),
                      1.5 * np.sin(phase + 2 * np.pi * k / n_frames), 1.2]) for k in range(n_frames)]
    scene = Scene(room=room, boxes=_boxes(rng, 6, 2.0, 1.1, eyes))
    poses, depths = [], []
    for e in eyes:
        P = look_at(e, target, np.deg2rad(rng.uniform(-5, 5)))
        poses.append(P)
        depths.append(add_noise(render_depth(scene, p, P), rng))
    return Workload("small_room_5x160x120_4cm", p, poses, depths, seed)


def full_room(seed: int = 1, n_frames: int = 13, rows: int = 480, cols: int = 640,
              res: float = 0.01) -> Workload:
    """Room 6x6x3 m, 20 boxes + 3 spheres, 1 cm voxels, 13 frames 640x480."""
    rng = np.random.default_rng(seed)
    f = 525.0 * cols / 640
    p = MapParams(res=res, dims=(6.0, 6.0, 3.0), rows=rows, cols=cols,
                  fx=f, fy=f, cx=cols / 2, cy=rows / 2, prior=0.1, max_iters=20)
    sensor_params(p)
    eps = res / 2
    room = np.array([-3 + eps, -3 + eps, eps, 3 - eps, 3 - eps, 3 - eps])
    a0 = rng.uniform(0, 2 * np.pi)
    eyes = []
    for k in range(n_frames):
        a = a0 + np.pi * k / max(n_frames - 1, 1)
        rad = 2.2 + rng.uniform(-0.2, 0.2)
        eyes.append(np.array([rad * np.cos(a), rad * np.sin(a), 1.4 + rng.uniform(-0.2, 0.2)]))
    boxes = _boxes(rng, 20, 3.0, 1.2, eyes)
    sph = []
    while len(sph) < 3:
        r = rng.uniform(0.2, 0.5)
        c = np.array([rng.uniform(-2.2, 2.2), rng.uniform(-2.2, 2.2), rng.uniform(0.6, 2.4)])
        if all(np.linalg.norm(c - e) > r + 0.3 for e in eyes):
            sph.append(np.concatenate([c, [r]]))
    scene = Scene(room=room, boxes=boxes, spheres=np.array(sph))
    poses, depths = [], []
    target = np.array([0.0, 0.0, 1.2])
    for e in eyes:
        P = look_at(e, target, np.deg2rad(rng.uniform(-5, 5)))
        poses.append(P)
        depths.append(add_noise(render_depth(scene, p, P), rng, max_range=5.0))
    return Workload(f"full_room_{n_frames}x{cols}x{rows}_{int(round(res * 100))}cm", p, poses, depths, seed,
                    scene=scene)


def mixed_room(seed: int = 2, n_frames: int = 12,
               sizes=((120, 160), (240, 320), (480, 640)), res: float = 0.02) -> Workload:
    """The full room's scene seen by views of mixed resolution (the sizes
    cycle over the frames; f = 525 cols / 640, principal point at the
    centre), 2 cm voxels: uneven image sizes and ray lengths in one map.
    ``params`` is the largest camera (the sensor tables' image)."""
    base = full_room(seed, n_frames=n_frames, rows=24, cols=32, res=res)  # scene and poses
    rows0, cols0 = sizes[-1]
    f0 = 525.0 * cols0 / 640
    base.params = sensor_params(MapParams(res=res, dims=base.params.dims, rows=rows0, cols=cols0, fx=f0, fy=f0,
                                          cx=cols0 / 2, cy=rows0 / 2, prior=0.1, max_iters=20))
    rng = np.random.default_rng(seed + 1000)
    scene = base.scene
    poses, depths, cams = [], [], []
    for k, P in enumerate(base.poses):
        rows, cols = sizes[k % len(sizes)]
        f = 525.0 * cols / 640
        cp = MapParams(res=res, dims=base.params.dims, rows=rows, cols=cols, fx=f, fy=f, cx=cols / 2,
                       cy=rows / 2, prior=0.1, max_iters=20)
        poses.append(P)
        depths.append(add_noise(render_depth(scene, cp, P), rng, max_range=5.0))
        cams.append((f, f, cols / 2, rows / 2))
    return Workload(f"mixed_room_{n_frames}x{len(sizes)}res_{int(round(res * 100))}cm", base.params, poses,
                    depths, seed, cams)


# ---- the streamed large-map workload ---------------------------------------

@dataclass
class Walk:
    """A camera walking through a room of boxes: the scene, the params and the
    per-frame poses; depth frames are rendered on demand (render_frame /
    render_frames_torch), since thousands of full-resolution frames do not
    fit in host memory at once."""
    name: str
    params: MapParams
    scene: Scene
    poses: list
    seed: int
    max_range: float = 5.0


def walk_room(seed: int = 5, n_frames: int = 2000, rows: int = 480, cols: int = 640, res: float = 0.02,
              dims=(20.0, 20.0, 4.0), n_boxes: int = 150, step: float = 0.05) -> Walk:
    """Seeded random walk through a dims-sized room holding n_boxes boxes on
    the floor (footprints 0.2-1.5 m, heights 0.2-1.2 m): the camera moves
    `step` metres per frame at 1.4-1.6 m height (above every box), its
    heading turning by N(0, 0.15 rad) per frame and reflecting off a band
    0.8 m inside the walls, looking 15 degrees down.  640x480 frames,
    fx = fy = 525, principal point at the centre, max range 5 m, 2 cm voxels,
    5 iterations per frame."""
    rng = np.random.default_rng(seed)
    f = 525.0 * cols / 640
    p = MapParams(res=res, dims=tuple(dims), rows=rows, cols=cols, fx=f, fy=f, cx=cols / 2, cy=rows / 2,
                  prior=0.1, max_iters=5)
    sensor_params(p)
    hx, hy, hz = dims[0] / 2, dims[1] / 2, dims[2]
    eps = res / 2
    room = np.array([-hx + eps, -hy + eps, eps, hx - eps, hy - eps, hz - eps])
    boxes = []
    while len(boxes) < n_boxes:
        fx_, fy_ = rng.uniform(0.2, 1.5, 2)
        h = rng.uniform(0.2, 1.2)
        cx_, cy_ = rng.uniform(-hx + 1.0, hx - 1.0), rng.uniform(-hy + 1.0, hy - 1.0)
        boxes.append([cx_ - fx_ / 2, cy_ - fy_ / 2, 0.0, cx_ + fx_ / 2, cy_ + fy_ / 2, h])
    scene = Scene(room=room, boxes=np.array(boxes))
    pos = np.array([rng.uniform(-hx / 2, hx / 2), rng.uniform(-hy / 2, hy / 2)])
    head = rng.uniform(0, 2 * np.pi)
    band = 0.8
    poses = []
    for k in range(n_frames):
        head += rng.normal(0.0, 0.15)
        nxt = pos + step * np.array([np.cos(head), np.sin(head)])
        if abs(nxt[0]) > hx - band:
            head = np.pi - head
        if abs(nxt[1]) > hy - band:
            head = -head
        pos = pos + step * np.array([np.cos(head), np.sin(head)])
        z = 1.5 + 0.1 * np.sin(0.01 * k)
        eye = np.array([pos[0], pos[1], z])
        target = eye + np.array([np.cos(head), np.sin(head), -np.tan(np.deg2rad(15.0))])
        poses.append(look_at(eye, target))
    return Walk(f"walk_room_{n_frames}x{cols}x{rows}_{int(round(res * 100))}cm", p, scene, poses, seed)


def render_frame(walk: Walk, k: int) -> np.ndarray:
    """Frame k of the walk on the host (numpy; seeded per frame)."""
    rng = np.random.default_rng((walk.seed, k))
    return add_noise(render_depth(walk.scene, walk.params, walk.poses[k]), rng, max_range=walk.max_range)


def render_frames_torch(walk: Walk, frames, device="cuda"):
    """Frames of the walk rendered with torch on `device` (the same scene,
    camera and noise model as render_frame, a torch generator seeded per
    frame): a list of (rows, cols) float32 tensors."""
    import torch
    p = walk.params
    H, W = p.rows, p.cols
    xs = (torch.arange(W, device=device, dtype=torch.float64) + 0.5 - p.cx) / p.fx
    ys = (torch.arange(H, device=device, dtype=torch.float64) + 0.5 - p.cy) / p.fy
    rc = torch.stack(torch.broadcast_tensors(xs[None, :], ys[:, None], torch.ones(H, W, device=device,
                                                                                   dtype=torch.float64)), -1)
    room = torch.tensor(walk.scene.room, device=device, dtype=torch.float64)
    boxes = torch.tensor(walk.scene.boxes, device=device, dtype=torch.float64)
    out = []
    for k in frames:
        P = torch.tensor(walk.poses[k], device=device, dtype=torch.float64)
        d = (rc @ P[:3, :3].T).reshape(-1, 3)
        o = P[:3, 3]
        inv = 1.0 / d
        lo = (room[:3] - o) * inv
        hi = (room[3:] - o) * inv
        t = torch.maximum(lo, hi).min(dim=1).values  # room seen from inside: its exit
        bl = (boxes[None, :, :3] - o) * inv[:, None, :]
        bh = (boxes[None, :, 3:] - o) * inv[:, None, :]
        tn = torch.minimum(bl, bh).max(dim=2).values
        tf = torch.maximum(bl, bh).min(dim=2).values
        hit = (tn <= tf) & (tn > 0)
        tb = torch.where(hit, tn, torch.full_like(tn, float("inf"))).min(dim=1).values
        t = torch.minimum(t, tb).reshape(H, W)
        g = torch.Generator(device=device)
        g.manual_seed(int(walk.seed) * 100003 + int(k))
        sig = 0.002 + 0.0012 * t * t
        z = t + torch.randn(t.shape, generator=g, device=device, dtype=torch.float64) * sig
        z = z.float()
        z[torch.rand(t.shape, generator=g, device=device) < 0.02] = 0.0
        z[z > walk.max_range] = 0.0
        out.append(z.contiguous())
    return out


# ---- the batched workload: several scenes in one map -------------------------

@dataclass
class Batch:
    """Scenes placed side by side in one map, each in its own brick-aligned
    box; every view belongs to one scene (box) and has its own camera."""
    name: str
    params: MapParams
    scenes: list          # Scene per box (world coordinates of the map)
    boxes: list           # (brick_lo[3], brick_hi[3]) per scene
    poses: list
    cams: list            # (rows, cols, fx, fy, cx, cy) per view
    scene_of: list        # scene index per view
    seed: int
    max_range: float


def batch_scenes(seed: int = 3, n_scenes: int = 8, views_per_scene: int = 32,
                 sizes=((120, 160), (240, 320), (480, 640)),
                 size_cycle=(0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 2),
                 res: float = 0.02, max_range: float = 9.5, n_boxes: int = 20,
                 room_range=(3.0, 7.0)) -> Batch:
    """n_scenes seeded box rooms of different sizes (room_range metres wide
    and deep, 2.5-4 m high), laid out along x with a one-brick gap,
    views_per_scene views each on a seeded loop inside the room aimed at its
    centre, image sizes taken from `sizes` in the order `size_cycle`
    (f = 525 cols / 640, principal point at the centre).  The default mix
    (10 in 16 views 160x120, 5 in 16 320x240, 1 in 16 640x480: 160 / 80 / 16
    of 256) keeps a map of such views at 2 cm near 3.2 G incidences, inside
    the 32-bit incidence index range (4.29 G).  Ray lengths run
    from a few voxels to several hundred crossings: the range is capped
    below the reference's 10 m Z_MAX."""
    rng = np.random.default_rng(seed)
    bsz = 8 * res
    rooms = []
    for s in range(n_scenes):
        w = rng.uniform(*room_range)
        dpt = rng.uniform(*room_range)
        h = rng.uniform(2.5, 4.0)
        rooms.append((w, dpt, h))
    nbx = [int(np.ceil(w / bsz)) + 1 for (w, _, _) in rooms]
    nby = max(int(np.ceil(d / bsz)) for (_, d, _) in rooms) + 1
    nbz = max(int(np.ceil(h / bsz)) for (_, _, h) in rooms) + 1
    NBx = sum(nbx) + (n_scenes - 1)
    dims = (NBx * bsz - res, nby * bsz - res, nbz * bsz - res)  # brick grids of exactly NBx, nby, nbz
    rows0, cols0 = sizes[-1]
    f0 = 525.0 * cols0 / 640
    p = MapParams(res=res, dims=dims, rows=rows0, cols=cols0, fx=f0, fy=f0, cx=cols0 / 2, cy=rows0 / 2,
                  prior=0.1, max_iters=20)
    sensor_params(p)
    off = np.array([dims[0] / 2 / res, dims[1] / 2 / res, 0.0])
    scenes, boxes, poses, cams, scene_of = [], [], [], [], []
    bx0 = 0
    for s, (w, dpt, h) in enumerate(rooms):
        lo = np.array([bx0, 0, 0])
        hi = np.array([bx0 + nbx[s], nby, nbz])
        boxes.append((lo.tolist(), hi.tolist()))
        # the room inside the box, in map world coordinates (metres)
        wlo = (lo * 8 - off) * res
        centre = np.array([wlo[0] + w / 2 + res, wlo[1] + dpt / 2 + res, 0.0])
        eps = res / 2
        room = np.array([centre[0] - w / 2 + eps, centre[1] - dpt / 2 + eps, eps,
                         centre[0] + w / 2 - eps, centre[1] + dpt / 2 - eps, h - eps])
        bxs = []
        while len(bxs) < n_boxes:
            side = rng.uniform(0.2, min(1.2, w / 4), 3)
            side[2] = rng.uniform(0.2, h / 2)
            c = np.array([rng.uniform(room[0] + 0.5, room[3] - 0.5), rng.uniform(room[1] + 0.5, room[4] - 0.5),
                          side[2] / 2])
            bxs.append(np.concatenate([c - side / 2, c + side / 2]))
        scenes.append(Scene(room=room, boxes=np.array(bxs)))
        target = np.array([centre[0], centre[1], h / 2])
        a0 = rng.uniform(0, 2 * np.pi)
        rad = 0.3 * min(w, dpt)
        for k in range(views_per_scene):
            a = a0 + 2 * np.pi * k / views_per_scene
            eye = np.array([centre[0] + rad * np.cos(a), centre[1] + rad * np.sin(a),
                            min(h - 0.3, 1.2 + rng.uniform(-0.2, 0.2))])
            poses.append(look_at(eye, target, np.deg2rad(rng.uniform(-5, 5))))
            rows, cols = sizes[size_cycle[k % len(size_cycle)]]
            f = 525.0 * cols / 640
            cams.append((rows, cols, f, f, cols / 2, rows / 2))
            scene_of.append(s)
        bx0 += nbx[s] + 1
    n = n_scenes * views_per_scene
    return Batch(f"batch_{n_scenes}scenes_{n}views_{int(round(res * 100))}cm", p, scenes, boxes, poses, cams,
                 scene_of, seed, max_range)


def render_batch_view(batch: Batch, k: int) -> np.ndarray:
    """View k of the batch on the host (numpy; seeded per view)."""
    rows, cols, fx, fy, cx, cy = batch.cams[k]
    cp = MapParams(res=batch.params.res, dims=batch.params.dims, rows=rows, cols=cols, fx=fx, fy=fy, cx=cx,
                   cy=cy, prior=0.1)
    rng = np.random.default_rng((batch.seed, k))
    return add_noise(render_depth(batch.scenes[batch.scene_of[k]], cp, batch.poses[k]), rng,
                     max_range=batch.max_range)


def render_batch_torch(batch: Batch, views, device="cuda"):
    """Views of the batch rendered with torch on `device` (box scenes, the
    noise model of add_noise, a generator seeded per view)."""
    out = []
    for k in views:
        rows, cols, fx, fy, cx, cy = batch.cams[k]
        out.append(_render_boxes_torch(batch.scenes[batch.scene_of[k]], rows, cols, fx, fy, cx, cy,
                                       batch.poses[k], batch.seed * 100003 + k, batch.max_range, device))
    return out


def _render_boxes_torch(scene, rows, cols, fx, fy, cx, cy, pose, seed, max_range, device):
    import torch
    xs = (torch.arange(cols, device=device, dtype=torch.float64) + 0.5 - cx) / fx
    ys = (torch.arange(rows, device=device, dtype=torch.float64) + 0.5 - cy) / fy
    rc = torch.stack(torch.broadcast_tensors(xs[None, :], ys[:, None],
                                             torch.ones(rows, cols, device=device, dtype=torch.float64)), -1)
    room = torch.tensor(scene.room, device=device, dtype=torch.float64)
    boxes = torch.tensor(scene.boxes, device=device, dtype=torch.float64)
    P = torch.tensor(pose, device=device, dtype=torch.float64)
    d = (rc @ P[:3, :3].T).reshape(-1, 3)
    o = P[:3, 3]
    inv = 1.0 / d
    t = torch.maximum((room[:3] - o) * inv, (room[3:] - o) * inv).min(dim=1).values
    bl = (boxes[None, :, :3] - o) * inv[:, None, :]
    bh = (boxes[None, :, 3:] - o) * inv[:, None, :]
    tn = torch.minimum(bl, bh).max(dim=2).values
    tf = torch.maximum(bl, bh).min(dim=2).values
    hit = (tn <= tf) & (tn > 0)
    tb = torch.where(hit, tn, torch.full_like(tn, float("inf"))).min(dim=1).values
    t = torch.minimum(t, tb).reshape(rows, cols)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    z = (t + torch.randn(t.shape, generator=g, device=device, dtype=torch.float64) * (0.002 + 0.0012 * t * t)).float()
    z[torch.rand(t.shape, generator=g, device=device) < 0.02] = 0.0
    z[z > max_range] = 0.0
    return z.contiguous()
