"""Map / sensor parameters -- the host-side mirror of ``gvdb_params_t``.

Field names, defaults and the sensor-polynomial tables follow the reference's
``include/mrfmap/GVDBParams.h:11-104`` (``res``, ``dims``, ``K``, ``rows``,
``cols``, ``prior``, ``max_iters``, ``lookup_n``, ``const_sigmasq_poly``,
``const_bias_poly``, per-20-pixel-tile lookup tables).  ``load_from_file``
reads the same ``gvdb_params:`` YAML block (a flat subset of YAML: scalars
and ``[a, b, c]`` lists), see ``GVDBParams.h:106-214``.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

LOOKUP_PX = 20          # include/mrfmap/GVDBCommon.cuh:11
LOOKUP_NUM = 3096       # include/mrfmap/GVDBCommon.cuh:10


def _parse_scalar(tok: str):
    tok = tok.strip()
    if tok.startswith(("'", '"')) and tok.endswith(("'", '"')):
        return tok[1:-1]
    low = tok.lower()
    if low in ("true", "false"):
        return low == "true"
    try:
        return int(tok)
    except ValueError:
        pass
    try:
        return float(tok)
    except ValueError:
        return tok


def parse_flat_yaml(text: str) -> dict:
    """Two-level YAML subset: ``section:`` then ``  key: value`` lines,
    values being scalars or one-line/multi-line ``[..]`` lists."""
    out: dict = {}
    section = None
    pending_key, pending = None, ""
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip():
            continue
        if pending_key is not None:
            pending += " " + line.strip()
            if "]" in pending:
                out[section][pending_key] = [_parse_scalar(t) for t in
                                             pending.strip()[1:pending.index("]")].split(",") if t.strip()]
                pending_key, pending = None, ""
            continue
        if not raw.startswith((" ", "\t")):
            section = line.strip().rstrip(":")
            out[section] = {}
            continue
        key, _, val = line.strip().partition(":")
        val = val.strip()
        if val.startswith("["):
            if "]" in val:
                out[section][key] = [_parse_scalar(t) for t in val[1:val.index("]")].split(",") if t.strip()]
            else:
                pending_key, pending = key, val
        else:
            out[section][key] = _parse_scalar(val) if val else ""
    return out


@dataclass
class MapParams:
    res: float = 0.01
    dims: tuple = (1.0, 1.0, 1.0)
    rows: int = 1
    cols: int = 1
    fx: float = 0.0
    fy: float = 0.0
    cx: float = 0.5
    cy: float = 0.5
    prior: float = 0.01
    max_iters: int = 1
    occ_thresh: float = 0.1
    acc_thresh: float = 0.5
    use_polys: bool = False
    lookup_n: int = 3
    const_sigmasq_poly: list = field(default_factory=lambda: [0.015, 0.0, 0.0])
    const_bias_poly: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    sigma_lut: np.ndarray | None = None
    bias_lut: np.ndarray | None = None
    gvdb_map_config: tuple = (1, 3, 3, 3, 3)

    def __post_init__(self):
        if self.fx == 0.0:
            # GVDBParams.h:30-47 default: hfov 0.01 rad
            self.fx = self.fy = (self.cols / 2.0) / math.tan(0.01 / 2.0)
        self.populate_lookup_tables()

    @property
    def n_tiles_u(self) -> int:
        return int(math.ceil(self.cols / LOOKUP_PX))

    @property
    def n_tiles_v(self) -> int:
        return int(math.ceil(self.rows / LOOKUP_PX))

    @property
    def K(self) -> np.ndarray:
        return np.array([[self.fx, 0, self.cx], [0, self.fy, self.cy], [0, 0, 1]], np.float32)

    def populate_lookup_tables(self):
        """Replicate the constant polynomials into every 20x20 tile
        (GVDBParams.h:93-104)."""
        n = self.n_tiles_u * self.n_tiles_v
        sg = np.asarray(self.const_sigmasq_poly[: self.lookup_n], np.float32)
        bs = np.asarray((list(self.const_bias_poly) + [0.0] * 3)[: self.lookup_n], np.float32)
        self.sigma_lut = np.tile(sg, n).astype(np.float32)
        self.bias_lut = np.tile(bs, n).astype(np.float32)

    def set_const_polys(self, sigma, bias=None, lookup_n=None):
        if lookup_n is not None:
            self.lookup_n = lookup_n
        self.const_sigmasq_poly = list(sigma)
        self.const_bias_poly = list(bias) if bias is not None else [0.0] * len(sigma)
        self.populate_lookup_tables()

    def check(self):
        if self.lookup_n not in (2, 3):
            raise ValueError("lookup_n must be 2 or 3")
        if self.sigma_lut.size != self.n_tiles_u * self.n_tiles_v * self.lookup_n:
            raise ValueError("sensor lookup table size does not match rows/cols")
        if self.sigma_lut.size > LOOKUP_NUM:
            raise ValueError("sensor lookup table larger than LOOKUP_NUM (3096) floats")

    def load_from_file(self, path: str):
        """Read the ``gvdb_params`` block of a MRFMap YAML config."""
        with open(path) as f:
            y = parse_flat_yaml(f.read())
        if "gvdb_params" not in y:
            raise ValueError("[gvdb_params] Could not read [gvdb_params]!")
        g = y["gvdb_params"]
        if "rows" in g:
            self.rows = int(g["rows"])
        if "cols" in g:
            self.cols = int(g["cols"])
        if "dims" in g:
            self.dims = tuple(float(v) for v in g["dims"])
        if "res" in g:
            self.res = float(g["res"])
        if "use_polys" not in g:
            raise ValueError("[gvdb_params] Please configure use_polys in config file.")
        self.use_polys = bool(g["use_polys"])
        if self.use_polys:
            self.lookup_n = int(g["poly_degree"])
            base = os.path.dirname(path)
            n = self.n_tiles_u * self.n_tiles_v * self.lookup_n
            tabs = []
            for key in ("depth_sigma_lookup", "depth_bias_lookup"):
                with open(os.path.join(base, g[key])) as f:
                    vals = [float(t) for t in f.read().replace("[", " ").replace("]", " ")
                            .replace(",", " ").replace("-", " -").split() if t not in ("-",)]
                tabs.append(np.asarray(vals[:n], np.float32))
            self.sigma_lut, self.bias_lut = tabs
        elif "const_sigmasq_poly" in g:
            self.lookup_n = int(g["poly_degree"])
            self.const_sigmasq_poly = [float(v) for v in g["const_sigmasq_poly"]][: self.lookup_n]
            if "const_bias_poly" in g:
                self.const_bias_poly = [float(v) for v in g["const_bias_poly"]][: self.lookup_n]
            self.populate_lookup_tables()
        for key in ("prior", "occ_thresh", "acc_thresh"):
            if key in g:
                setattr(self, key, float(g[key]))
        if "max_iters" in g:
            self.max_iters = int(g["max_iters"])
        if "K" in g:
            K = [float(v) for v in g["K"]]
            self.fx, self.cx, self.fy, self.cy = K[0], K[2], K[4], K[5]
        if "gvdb_map_config" in g:
            self.gvdb_map_config = tuple(int(v) for v in g["gvdb_map_config"])
        if not self.use_polys and "const_sigmasq_poly" not in g:
            self.populate_lookup_tables()
        return self


def read_eigen_binary(path: str) -> np.ndarray:
    """Reader for the reference's fixture format (src/testMRFMapViewer.cpp:18-27):
    int64 rows, int64 cols, then column-major float32 data."""
    with open(path, "rb") as f:
        raw = f.read()
    r, c = np.frombuffer(raw[:16], dtype=np.int64)
    return np.frombuffer(raw[16:16 + 4 * r * c], dtype=np.float32).reshape(int(c), int(r)).T.copy()
