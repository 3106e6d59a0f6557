"""Seeded procedural airbox geometry (the lower, raw-air part of a filter box).

The reference ships no STL at all, so every workload of this library is made
here.  The geometry is built as a union of *closed, pairwise disjoint* solids
that may touch on faces, which is what the reference's parity voxelizer
(`src/engine.js:45-93`) needs: a ray along local Z must cross each solid's
surface an even number of times.

Model coordinates follow the reference's default airbox orientation
(`airbox_cfd.py:47-50`, prepare params of `src/ui.html:477-479`):

* the filter seal plane is Y = 0 and the box extends in +Y (``sealAxis=1``,
  ``sealSign=-1``), so local depth D = y;
* the inlet sits on the Z-min face and air flows in +Z (``inletAxis=2``,
  ``inletSign=-1``);
* an inlet yaw rotates the stub axis about Y; the reference rotates its grid
  by the same angle (`src/engine.js:35-41`), so the stub's end face is
  perpendicular to local Z.

Parts of the tray (wall thickness ``t``):

* bottom plate  ``y in [Ly-t, Ly]`` over the full x/z extent;
* two side walls ``x in [0,t]`` and ``x in [Lx-t, Lx]``, ``y in [0, Ly-t]``;
* the far wall  ``z in [Lz-t, Lz]`` between the side walls;
* the inlet wall ``z in [0, t]`` between the side walls, with a round hole;
* a tube (inner radius r, wall ``t``) from the hole outwards, cut by the
  plane z = 0 and closed by an annular end face perpendicular to its axis;
* optionally one baffle plate standing on the bottom, perpendicular to Z.

The top (Y = 0) is open: that is where the filter seals.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field, asdict
from typing import Optional

import numpy as np


# ----------------------------------------------------------------------------- primitives
def _box(x0, x1, y0, y1, z0, z1):
    """Closed cuboid as 12 triangles, shape (12, 3, 3)."""
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], float)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
         (3, 6, 2), (3, 7, 6), (0, 4, 7), (0, 7, 3), (1, 2, 6), (1, 6, 5)]
    return np.array([[v[a], v[b], v[c]] for a, b, c in f])


def _quads(ring_a, ring_b):
    """Closed band between two rings of equal length (M, 3) → (2M, 3, 3)."""
    m = len(ring_a)
    out = []
    for i in range(m):
        j = (i + 1) % m
        out.append([ring_a[i], ring_a[j], ring_b[j]])
        out.append([ring_a[i], ring_b[j], ring_b[i]])
    return np.array(out)


def _rect_minus_hole(rect, hole_xy, centre, z):
    """Triangulate the planar region ``rect`` minus polygon ``hole_xy`` at height z.

    ``rect = (x0, x1, y0, y1)``; ``hole_xy`` (M, 2) is star-shaped around
    ``centre`` with strictly increasing angle.  For each hole edge the sector
    between the two rays through its end points is fanned from the edge's
    first vertex over the rectangle boundary chain (ray hits plus any corner
    inside the sector), which is valid because the rectangle is convex.
    """
    x0, x1, y0, y1 = rect
    cx, cy = centre
    m = len(hole_xy)
    ang = np.arctan2(hole_xy[:, 1] - cy, hole_xy[:, 0] - cx)

    def ray_hit(a):
        dx, dy = math.cos(a), math.sin(a)
        ts = []
        if dx > 1e-15: ts.append((x1 - cx) / dx)
        if dx < -1e-15: ts.append((x0 - cx) / dx)
        if dy > 1e-15: ts.append((y1 - cy) / dy)
        if dy < -1e-15: ts.append((y0 - cy) / dy)
        tt = min(ts)
        return np.array([cx + tt * dx, cy + tt * dy])

    corners = np.array([[x0, y0], [x1, y0], [x1, y1], [x0, y1]], float)
    cang = np.arctan2(corners[:, 1] - cy, corners[:, 0] - cx)
    tris = []
    for i in range(m):
        j = (i + 1) % m
        a0, a1 = ang[i], ang[j]
        span = (a1 - a0) % (2 * math.pi)
        inside = []
        for c, ca in zip(corners, cang):
            d = (ca - a0) % (2 * math.pi)
            if 0 < d < span:
                inside.append((d, c))
        inside.sort(key=lambda t: t[0])
        chain = [ray_hit(a0)] + [c for _, c in inside] + [ray_hit(a1)]
        p0, p1 = hole_xy[i], hole_xy[j]
        for k in range(len(chain) - 1):
            tris.append([p0, chain[k], chain[k + 1]])
        tris.append([p0, chain[-1], p1])
    out = np.array([[[p[0], p[1], z] for p in t] for t in tris], float)
    return out


# ----------------------------------------------------------------------------- airbox
@dataclass
class AirboxSpec:
    """Dimensions in mm (model coordinates, see module docstring)."""
    Lx: float = 240.0            # width (free axis)
    Ly: float = 120.0            # depth below the seal plane, into the box
    Lz: float = 180.0            # length along the inlet direction
    t: float = 3.0               # wall thickness
    d_in: float = 70.0           # inlet inner diameter
    stub: float = 30.0           # stub length along its axis (outside the wall)
    hole_x: Optional[float] = None   # hole centre x (default: middle)
    hole_y: Optional[float] = None   # hole centre depth (default: as deep as fits)
    yaw: float = 0.0             # inlet yaw about Y, degrees
    baffle: Optional[dict] = None    # {"z": .., "x0": .., "x1": .., "y0": ..} or None
    segments: int = 64           # polygon segments of the round inlet
    pleat: float = 40.0
    dx: float = 4.0

    def prepare_params(self) -> dict:
        """The reference's prepare() parameter object for this box."""
        return {"dx": float(self.dx), "sealAxis": 1, "sealSign": -1, "seal": 0.0,
                "inletAxis": 2, "inletSign": -1, "inletYaw": float(self.yaw),
                "pleat": float(self.pleat), "click": None, "outlet": None}


def build_airbox(spec: AirboxSpec) -> np.ndarray:
    """Triangles of the airbox, float32 array of shape (ntri, 9)."""
    Lx, Ly, Lz, t = spec.Lx, spec.Ly, spec.Lz, spec.t
    r = 0.5 * spec.d_in
    R = r + t
    yaw = math.radians(spec.yaw)
    cyw, syw = math.cos(yaw), math.sin(yaw)
    u = np.array([-syw, 0.0, cyw])          # stub axis, pointing into the box
    e1 = np.array([cyw, 0.0, syw])          # perpendicular to u in the x-z plane
    e2 = np.array([0.0, 1.0, 0.0])
    hx = spec.hole_x if spec.hole_x is not None else 0.5 * Lx
    hy = spec.hole_y if spec.hole_y is not None else Ly - t - R - 2.0
    H = np.array([hx, hy, 0.0])
    m = spec.segments
    th = 2 * math.pi * (np.arange(m) + 0.5) / m

    def ring(rad, zplane=None, s_fixed=None):
        pts = []
        for a in th:
            off = rad * (math.cos(a) * e1 + math.sin(a) * e2)
            if zplane is not None:
                s = (zplane - off[2]) / cyw
            else:
                s = s_fixed
            p = H + s * u + off
            if zplane is not None:
                p[2] = zplane           # exactly on the plane, like the faces it meets
            pts.append(p)
        return np.array(pts)

    parts = []
    parts.append(_box(0, Lx, Ly - t, Ly, 0, Lz))                 # bottom
    parts.append(_box(0, t, 0, Ly - t, 0, Lz))                   # side x-
    parts.append(_box(Lx - t, Lx, 0, Ly - t, 0, Lz))             # side x+
    parts.append(_box(t, Lx - t, 0, Ly - t, Lz - t, Lz))         # far wall
    # inlet wall with the hole: faces z=0 and z=t, hole band, rim faces
    q0, q1 = ring(r, zplane=0.0), ring(r, zplane=t)
    rect = (t, Lx - t, 0.0, Ly - t)
    parts.append(_rect_minus_hole(rect, q0[:, :2], (hx, hy), 0.0))
    parts.append(_rect_minus_hole(rect, q1[:, :2], (hx, hy), t))
    parts.append(_quads(q0, q1))
    x0, x1, y0, y1 = rect
    parts.append(np.array([[[x0, y0, 0], [x1, y0, 0], [x1, y0, t]], [[x0, y0, 0], [x1, y0, t], [x0, y0, t]],
                           [[x0, y1, 0], [x1, y1, t], [x1, y1, 0]], [[x0, y1, 0], [x0, y1, t], [x1, y1, t]],
                           [[x0, y0, 0], [x0, y1, t], [x0, y1, 0]], [[x0, y0, 0], [x0, y0, t], [x0, y1, t]],
                           [[x1, y0, 0], [x1, y1, 0], [x1, y1, t]], [[x1, y0, 0], [x1, y1, t], [x1, y0, t]]], float))
    # the stub: inner and outer cylinder from the end cap to the plane z=0
    s_end = -spec.stub
    qi_end, qo_end = ring(r, s_fixed=s_end), ring(R, s_fixed=s_end)
    qo0 = ring(R, zplane=0.0)
    parts.append(_quads(qi_end, q0))        # inner surface
    parts.append(_quads(qo_end, qo0))       # outer surface
    parts.append(_quads(qi_end, qo_end))    # end annulus (perpendicular to the axis)
    parts.append(_quads(q0, qo0))           # annulus in the plane z=0
    if spec.baffle:
        b = spec.baffle
        zb = b["z"]
        parts.append(_box(b["x0"], b["x1"], b["y0"], Ly - t, zb, zb + t))
    tris = np.concatenate(parts, 0).reshape(-1, 9)
    return tris.astype(np.float32)


def check_spec(spec: AirboxSpec) -> None:
    """Raise ValueError when the inlet does not fit the wall it sits in."""
    r = 0.5 * spec.d_in
    R = r + spec.t
    hx = spec.hole_x if spec.hole_x is not None else 0.5 * spec.Lx
    hy = spec.hole_y if spec.hole_y is not None else spec.Ly - spec.t - R - 2.0
    yaw = math.radians(spec.yaw)
    half_x = R / math.cos(yaw) + spec.t * abs(math.tan(yaw)) + 1.0
    if hy - R < 1.0 or hy + R > spec.Ly - spec.t - 1.0:
        raise ValueError("inlet does not fit the box depth")
    if hx - half_x < spec.t + 1.0 or hx + half_x > spec.Lx - spec.t - 1.0:
        raise ValueError("inlet does not fit the box width")
    if spec.stub * math.cos(yaw) <= R * abs(math.sin(yaw)) + 1.0:
        raise ValueError("stub too short for the yaw angle")


# ----------------------------------------------------------------------------- workloads
def config1_spec() -> AirboxSpec:
    """The reference-CPU-sized airbox: 240 x D x 180 mm, 3 mm walls, 70 mm inlet
    with a 30 mm stub on Z-min, pleat 40 mm, dx 4 mm.

    A 70 mm inlet cannot sit in a 60 mm deep wall below the seal, so the
    depth is 120 mm here (inlet centre 77 mm below the seal)."""
    return AirboxSpec(Lx=240.0, Ly=120.0, Lz=180.0, t=3.0, d_in=70.0, stub=30.0,
                      yaw=0.0, pleat=40.0, dx=4.0)


def random_spec(seed: int, dx: float = 1.5) -> AirboxSpec:
    """Seeded airbox of the variant generator.

    Width U(200,320) mm, length U(150,250) mm, depth = pleat 40 mm +
    U(50,90) mm, 3 mm walls, one 3 mm baffle on the bottom covering 30-60 %
    of the inner width at 30-70 % of the length, inlet diameter U(55,80) mm
    clamped to what the depth holds, yaw U(-30,30) degrees.
    """
    rng = np.random.default_rng(seed)
    t = 3.0
    Lx = float(rng.uniform(200, 320))
    Lz = float(rng.uniform(150, 250))
    Ly = 40.0 + float(rng.uniform(50, 90))
    d = float(rng.uniform(55, 80))
    d = min(d, Ly - 3 * t - 6.0)
    yaw = float(rng.uniform(-30, 30))
    R = 0.5 * d + t
    # The reference searches the opening 1.5 mm behind the front-most point of
    # the yawed frame (src/engine.js:142), so the stub's end must lie in front
    # of every rotated box corner: local Z of a point is -sin(yaw) x + cos(yaw) z.
    sy = math.sin(math.radians(yaw))
    front = sy * (Lx - 0.5 * Lx) if sy > 0 else -sy * 0.5 * Lx
    stub = max(30.0, R * abs(math.tan(math.radians(yaw))) + 12.0, front + 8.0)
    frac = float(rng.uniform(0.3, 0.6))
    inner = Lx - 2 * t
    w = frac * inner
    left = bool(rng.integers(0, 2))
    zb = float(rng.uniform(0.3, 0.7)) * Lz
    raw = Ly - t - 40.0                      # raw-air depth below the pleat
    hb = float(rng.uniform(0.3, 0.7)) * raw
    x0, x1 = (t, t + w) if left else (Lx - t - w, Lx - t)
    baffle = {"z": zb, "x0": x0, "x1": x1, "y0": Ly - t - hb}
    spec = AirboxSpec(Lx=Lx, Ly=Ly, Lz=Lz, t=t, d_in=d, stub=stub, yaw=yaw,
                      baffle=baffle, pleat=40.0, dx=dx)
    check_spec(spec)
    return spec


def grid_spec(nx: int, ny: int, nz: int, dx: float, seed: int = 7) -> AirboxSpec:
    """An airbox sized so that prepare() gives exactly an nx x ny x nz grid
    at cell size dx (no yaw; baffle and inlet drawn from the seed).

    The grid formula of `src/engine.js:121-122` is n = ceil((mx - origin + h)/h)
    with origin = mn - h (mn - 10 h along Z), so the extents are chosen a
    quarter cell below the integer boundary."""
    rng = np.random.default_rng(seed)
    t = 3.0
    h = dx
    Lx = (nx - 2) * h - 0.25 * h
    Ly = (ny - 2) * h - 0.25 * h
    d = min(float(rng.uniform(55, 80)), Ly - 3 * t - 6.0)
    stub = 30.0
    Lz = (nz - 11) * h - 0.25 * h - stub
    frac = float(rng.uniform(0.3, 0.6))
    w = frac * (Lx - 2 * t)
    raw = Ly - t - 40.0
    hb = float(rng.uniform(0.3, 0.7)) * raw
    baffle = {"z": float(rng.uniform(0.3, 0.7)) * Lz, "x0": t, "x1": t + w, "y0": Ly - t - hb}
    spec = AirboxSpec(Lx=Lx, Ly=Ly, Lz=Lz, t=t, d_in=d, stub=stub, yaw=0.0,
                      baffle=baffle, pleat=40.0, dx=dx)
    check_spec(spec)
    return spec


# ----------------------------------------------------------------------------- STL I/O
def to_binary_stl(tris: np.ndarray) -> bytes:
    """Binary STL (80-byte header, uint32 count, 50 bytes per facet)."""
    tris = np.asarray(tris, np.float32).reshape(-1, 9)
    n = len(tris)
    rec = np.zeros(n, dtype=np.dtype([("n", "<3f4"), ("v", "<9f4"), ("a", "<u2")]))
    rec["v"] = tris
    return b"airboxcalc_gb300 procedural airbox".ljust(80, b" ") + struct.pack("<I", n) + rec.tobytes()


def to_ascii_stl(tris: np.ndarray) -> bytes:
    """ASCII STL with ``vertex x y z`` lines (repr of the float32 values)."""
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    lines = ["solid airbox"]
    for t in tris:
        lines.append("facet normal 0 0 0\n outer loop")
        for v in t:
            lines.append("  vertex %r %r %r" % (float(v[0]), float(v[1]), float(v[2])))
        lines.append(" endloop\nendfacet")
    lines.append("endsolid airbox")
    return ("\n".join(lines) + "\n").encode()
