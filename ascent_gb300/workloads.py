"""Seeded synthetic inputs for the volume-plot workloads.

Each workload is the data one Ascent volume plot would receive: domains of
a uniform (or rectilinear) mesh with a float32 nodal field, a camera built
the way the reference's renders build it (reset to the scene bounds, then
azimuth / elevation), control points of a transfer function, and the plot's
`samples` count. Fields are sums of separable Gaussian blobs (plus noise or
sinusoidal turbulence), so even 513^3 grids generate in seconds.
"""
from __future__ import annotations

from dataclasses import dataclass, field as dc_field

import numpy as np


@dataclass
class UniformDomain:
    field: np.ndarray            # (nz, ny, nx) float32 node values
    origin: tuple
    spacing: tuple

    @property
    def dims(self):
        nz, ny, nx = self.field.shape
        return (nx, ny, nz)

    @property
    def bounds(self):
        b = []
        for a, n in enumerate(self.dims):
            b += [self.origin[a], self.origin[a] + (n - 1) * self.spacing[a]]
        return np.array(b, dtype=np.float64)


@dataclass
class Workload:
    name: str
    domains: list
    width: int
    height: int
    samples: int
    azimuth: float = 0.0
    elevation: float = 0.0
    rgb_pos: np.ndarray = dc_field(default_factory=lambda: np.zeros(0))
    rgb: np.ndarray = dc_field(default_factory=lambda: np.zeros((0, 3)))
    alpha_pos: np.ndarray = dc_field(default_factory=lambda: np.zeros(0))
    alpha: np.ndarray = dc_field(default_factory=lambda: np.zeros(0))

    @property
    def bounds(self) -> np.ndarray:
        bs = np.stack([d.bounds for d in self.domains])
        return np.array([bs[:, 0].min(), bs[:, 1].max(), bs[:, 2].min(), bs[:, 3].max(),
                         bs[:, 4].min(), bs[:, 5].max()])

    @property
    def scalar_range(self):
        lo = min(float(d.field.min()) for d in self.domains)
        hi = max(float(d.field.max()) for d in self.domains)
        return lo, hi

    @property
    def single_domain(self) -> bool:
        """One structured domain: the reference's RenderOneDomainPerRank path."""
        return len(self.domains) == 1 and isinstance(self.domains[0], UniformDomain)


def linear_ramp_tf(n: int = 256, alpha_max: float = 0.3):
    """n rgb + n alpha control points: colour (x, 0.5, 1-x), opacity alpha_max * x."""
    x = np.linspace(0.0, 1.0, n)
    rgb = np.stack([x, np.full_like(x, 0.5), 1.0 - x], axis=1)
    return x, rgb, x.copy(), alpha_max * x


def blob_params(rng: np.random.Generator, n: int = 8):
    centres = rng.uniform(0.2, 0.8, size=(n, 3))
    sigmas = rng.uniform(0.05, 0.15, size=n)
    amps = rng.uniform(0.5, 1.0, size=n)
    return centres, sigmas, amps


def blob_field(coords, centres, sigmas, amps) -> np.ndarray:
    """Sum of separable Gaussians on the grid coords = (x[nx], y[ny], z[nz])."""
    x, y, z = (np.asarray(c, dtype=np.float64) for c in coords)
    out = np.zeros((len(z), len(y), len(x)), dtype=np.float32)
    for c, s, a in zip(centres, sigmas, amps):
        gx = np.exp(-((x - c[0]) ** 2) / (2 * s * s)).astype(np.float32)
        gy = np.exp(-((y - c[1]) ** 2) / (2 * s * s)).astype(np.float32)
        gz = (a * np.exp(-((z - c[2]) ** 2) / (2 * s * s))).astype(np.float32)
        out += gz[:, None, None] * (gy[:, None] * gx[None, :])[None, :, :]
    return out


def turbulence(coords, rng: np.random.Generator, octaves: int = 3, amplitude: float = 0.2):
    """Sum over octaves o of amplitude 2^-o sin(2^o 2 pi (x+px)) sin(..y..) sin(..z..)."""
    x, y, z = (np.asarray(c, dtype=np.float64) for c in coords)
    out = np.zeros((len(z), len(y), len(x)), dtype=np.float32)
    for o in range(octaves):
        ph = rng.uniform(0.0, 1.0, size=3)
        f = 2.0 * np.pi * (2 ** o) * 2.0
        sx = np.sin(f * (x + ph[0])).astype(np.float32)
        sy = np.sin(f * (y + ph[1])).astype(np.float32)
        sz = (amplitude * 0.5 ** o * np.sin(f * (z + ph[2]))).astype(np.float32)
        out += sz[:, None, None] * (sy[:, None] * sx[None, :])[None, :, :]
    return out


def split_uniform(field: np.ndarray, origin, spacing, parts=(2, 2, 2)) -> list:
    """Split a node grid into parts[0] x parts[1] x parts[2] domains sharing face nodes."""
    nz, ny, nx = field.shape
    cuts = []
    for n, p in zip((nx, ny, nz), parts):
        cells = n - 1
        edges = [round(i * cells / p) for i in range(p + 1)]
        cuts.append(edges)
    out = []
    for k in range(parts[2]):
        for j in range(parts[1]):
            for i in range(parts[0]):
                x0, x1 = cuts[0][i], cuts[0][i + 1]
                y0, y1 = cuts[1][j], cuts[1][j + 1]
                z0, z1 = cuts[2][k], cuts[2][k + 1]
                sub = np.ascontiguousarray(field[z0:z1 + 1, y0:y1 + 1, x0:x1 + 1])
                o = (origin[0] + x0 * spacing[0], origin[1] + y0 * spacing[1],
                     origin[2] + z0 * spacing[2])
                out.append(UniformDomain(sub, o, tuple(spacing)))
    return out


def plain_small(n: int = 64, seed: int = 1, width: int = 512, height: int = 512,
                samples: int = 218, parts=None) -> Workload:
    """One uniform n^3 float32 nodal field: 8 Gaussian blobs + N(0, 0.01) noise on the
    unit cube, camera at azimuth 30 / elevation 20, 256-point linear TF (alpha 0 -> 0.3).
    The default (n=64, 512^2, samples=218 ~ 0.5 cell) is the CPU-runnable plain case."""
    rng = np.random.default_rng(seed)
    coords = [np.linspace(0.0, 1.0, n)] * 3
    c, s, a = blob_params(rng)
    f = blob_field(coords, c, s, a)
    f += rng.normal(0.0, 0.01, size=f.shape).astype(np.float32)
    sp = (1.0 / (n - 1),) * 3
    doms = [UniformDomain(f, (0.0, 0.0, 0.0), sp)] if parts is None else split_uniform(f, (0, 0, 0), sp, parts)
    rp, rgb, ap, al = linear_ramp_tf()
    return Workload(f"uniform{n}^3x{len(doms)}dom@{width}x{height}", doms, width, height, samples,
                    30.0, 20.0, rp, rgb, ap, al)


@dataclass
class HexDomain:
    x: np.ndarray            # node coordinates, float32
    y: np.ndarray
    z: np.ndarray
    conn: np.ndarray         # (n_cells, 8) int32, VTK hexahedron order
    field: np.ndarray        # node values, float32

    @property
    def bounds(self):
        return np.array([self.x.min(), self.x.max(), self.y.min(), self.y.max(), self.z.min(),
                         self.z.max()], dtype=np.float64)


def hex_grid_connectivity(n: int) -> np.ndarray:
    """(n^3, 8) int32 node ids of the hexahedra of an n^3-cell grid of (n+1)^3
    nodes (x fastest), in VTK hexahedron order."""
    m = n + 1
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = ((k * m + j) * m + i).astype(np.int64).ravel()
    off = np.array([0, 1, m + 1, m, m * m, m * m + 1, m * m + m + 1, m * m + m], dtype=np.int64)
    return (base[:, None] + off[None, :]).astype(np.int32)


def hex_mesh(n_cells: int = 200, seed: int = 3, width: int = 1024, height: int = 1024,
             jitter: float = 0.2) -> Workload:
    """n_cells^3 hexahedra from a uniform grid on the unit cube with every node
    moved by U[-jitter, jitter] cell per axis (seeded), and a float32 nodal field
    of Gaussian blobs evaluated at the moved nodes; samples ~ 0.5 cell."""
    rng = np.random.default_rng(seed)
    m = n_cells + 1
    h = 1.0 / n_cells
    g = np.arange(m, dtype=np.float64) * h
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    pts = [c.ravel() + rng.uniform(-jitter * h, jitter * h, size=m ** 3) for c in (x, y, z)]
    c, s, a = blob_params(rng)
    f = np.zeros(m ** 3, dtype=np.float64)
    for cc, ss, aa in zip(c, s, a):
        d2 = (pts[0] - cc[0]) ** 2 + (pts[1] - cc[1]) ** 2 + (pts[2] - cc[2]) ** 2
        f += aa * np.exp(-d2 / (2 * ss * ss))
    dom = HexDomain(*(p.astype(np.float32) for p in pts), hex_grid_connectivity(n_cells),
                    f.astype(np.float32))
    samples = int(np.ceil(np.sqrt(3.0) * n_cells / 0.5))
    rp, rgb, ap, al = linear_ramp_tf()
    return Workload(f"hex{n_cells}^3@{width}x{height}", [dom], width, height, samples, 30.0, 20.0,
                    rp, rgb, ap, al)


EDGES = (32, 48, 64, 96, 128, 192, 256)


def kd_boxes(root, n_boxes: int, rng: np.random.Generator) -> list:
    """Split the integer box `root` = (x0, y0, z0, x1, y1, z1) (cells) into
    n_boxes boxes: repeatedly split the largest box along a random axis at an
    offset that leaves both parts with edge lengths in EDGES."""
    boxes = [tuple(root)]
    while len(boxes) < n_boxes:
        order = sorted(range(len(boxes)), key=lambda i: -np.prod(
            [boxes[i][3 + a] - boxes[i][a] for a in range(3)]))
        for i in order:
            b = boxes[i]
            axes = rng.permutation(3)
            done = False
            for a in axes:
                L = b[3 + a] - b[a]
                cuts = [e for e in EDGES if (L - e) in EDGES]
                if cuts:
                    e = int(rng.choice(cuts))
                    lo = list(b)
                    hi = list(b)
                    lo[3 + a] = b[a] + e
                    hi[a] = b[a] + e
                    boxes[i:i + 1] = [tuple(lo), tuple(hi)]
                    done = True
                    break
            if done:
                break
        else:
            raise ValueError("cannot split further with the allowed edge lengths")
    return boxes


def cinema_batch(n_domains: int = 37, box_cells: int = 256, seed: int = 4, width: int = 512,
                 height: int = 512, n_phi: int = 8, n_theta: int = 8) -> Workload:
    """n_domains uniform float32 domains of uneven sizes (edges from
    {32,48,64,96,128,192,256} cells per axis, seeded k-d splits) tiling a
    box_cells^3 box of one Gaussian-blob field (nodes shared across faces),
    spacing 1/box_cells; rendered for n_phi x n_theta Cinema cameras."""
    rng = np.random.default_rng(seed)
    boxes = kd_boxes((0, 0, 0, box_cells, box_cells, box_cells), n_domains, rng)
    c, s, a = blob_params(rng)
    h = 1.0 / box_cells
    doms = []
    for b in boxes:
        coords = [np.arange(b[ax], b[3 + ax] + 1) * h for ax in range(3)]
        f = blob_field(coords, c, s, a)
        doms.append(UniformDomain(f, (b[0] * h, b[1] * h, b[2] * h), (h, h, h)))
    samples = int(np.ceil(np.sqrt(3.0) * box_cells / 0.5))
    rp, rgb, ap, al = linear_ramp_tf()
    wl = Workload(f"cinema{n_domains}dom{box_cells}^3x{n_phi * n_theta}views@{width}x{height}", doms,
                  width, height, samples, 0.0, 0.0, rp, rgb, ap, al)
    wl.phi_theta = cinema_angles(n_phi, n_theta)
    return wl


def cinema_angles(n_phi: int, n_theta: int) -> np.ndarray:
    """(phi, theta) pairs of a Cinema sweep given `phi`/`theta` counts:
    phi from -180 in steps of 360/n_phi, theta from 0 in steps of 180/n_theta
    (CinemaManager, ascent_runtime_rendering_filters.cpp:555-610)."""
    phis = [-180.0 + i * 360.0 / n_phi for i in range(n_phi)]
    thetas = [0.0 + j * 180.0 / n_theta for j in range(n_theta)]
    return np.array([(p, t) for p in phis for t in thetas], dtype=np.float32)


def plain_large(n_cells: int = 512, seed: int = 2, width: int = 1024, height: int = 1024,
                parts=(2, 2, 2)) -> Workload:
    """A (n_cells+1)^3-node float32 field (Gaussian blobs + 3-octave sinusoidal turbulence)
    split into 8 domains of (n_cells/2)^3 cells sharing face nodes, 1024^2 image,
    samples = ceil(|extent| / 0.5 cell)."""
    rng = np.random.default_rng(seed)
    n = n_cells + 1
    coords = [np.linspace(0.0, 1.0, n)] * 3
    c, s, a = blob_params(rng)
    f = blob_field(coords, c, s, a)
    f += turbulence(coords, rng)
    sp = (1.0 / n_cells,) * 3
    doms = split_uniform(f, (0.0, 0.0, 0.0), sp, parts)
    samples = int(np.ceil(np.sqrt(3.0) * n_cells / 0.5))
    rp, rgb, ap, al = linear_ramp_tf()
    return Workload(f"uniform{n_cells}^3x{len(doms)}dom@{width}x{height}", doms, width, height,
                    samples, 30.0, 20.0, rp, rgb, ap, al)


def to_blueprint(wl, field: str = "braid") -> list:
    """The workload's domains as Blueprint-shaped dicts (uniform or explicit hex)."""
    out = []
    for i, d in enumerate(wl.domains):
        if isinstance(d, HexDomain):
            out.append({
                "state": {"domain_id": i, "cycle": 100, "time": 1.5},
                "coordsets": {"coords": {"type": "explicit", "values": {"x": d.x, "y": d.y, "z": d.z}}},
                "topologies": {"mesh": {"type": "unstructured", "coordset": "coords",
                                        "elements": {"shape": "hex", "connectivity": d.conn.ravel()}}},
                "fields": {field: {"association": "vertex", "topology": "mesh", "values": d.field}},
            })
        else:
            nx, ny, nz = d.dims
            out.append({
                "state": {"domain_id": i, "cycle": 100, "time": 1.5},
                "coordsets": {"coords": {"type": "uniform", "dims": {"i": nx, "j": ny, "k": nz},
                                         "origin": {"x": d.origin[0], "y": d.origin[1], "z": d.origin[2]},
                                         "spacing": {"dx": d.spacing[0], "dy": d.spacing[1],
                                                     "dz": d.spacing[2]}}},
                "topologies": {"mesh": {"type": "uniform", "coordset": "coords"}},
                "fields": {field: {"association": "vertex", "topology": "mesh", "values": d.field.ravel()}},
            })
    return out
