"""Seeded synthetic bake scenes (the workloads the benchmark and the parity tests bake).

No scene file ships with the reference; these stand in for its bench scene
(benches/bake.rs:16-129) at the sizes of the five workloads the project measures:

1. `small_room`      - closed 10x4x10 m room (inward faces) plus 5 cubes, 4 point lights,
                       8 texels/m, direct light only.
2. `room_grid`       - 6x6 rooms of 8x3.5x8 m with doorways, 20 boxes/ramps each (~50k tris),
                       64 point lights with one bounce (64 gather samples), 16 texels/m.
3. `soft_rooms`      - the same level re-meshed with log-normal triangle sizes, 128 lights:
                       64 point, 32 rectangle, 32 tube, 16 soft samples per texel.
4. `outdoor`         - 512x512 heightfield (522k tris) in 8x8 chunks plus 2000 boxes and thin
                       planks, a soft 0.53 deg sun with colored bounce (128 samples), a sky
                       (256 samples) and 32 point lights, 4 texels/m.

Every random choice comes from SplitMix64 (src/effects/rng.rs:10-15) keyed by the workload
number, so a scene is the same on every machine. Meshes get one UV1 atlas cell per face as the
reference bench does (benches/bake.rs:33-44). Each generator takes a `scale` that shrinks the
scene for tests while keeping its structure.
"""
from __future__ import annotations

import math

import numpy as np

from . import (ANGULAR, BakeBounce, BakeInput, BakeLight, BakeMesh, BakeOptions, LIGHTING_ONLY,
               LightShape, SINGLE_BOUNCE, DIRECT)

MASK = (1 << 64) - 1


def splitmix64(v: int) -> int:
    v = (v + 0x9E3779B97F4A7C15) & MASK
    v = ((v ^ (v >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    v = ((v ^ (v >> 27)) * 0x94D049BB133111EB) & MASK
    return v ^ (v >> 31)


class Rng:
    """Sequential SplitMix64 stream."""

    def __init__(self, seed: int):
        self.state = seed & MASK

    def u64(self):
        self.state = splitmix64(self.state)
        return self.state

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.u64() >> 40) / float(1 << 24))

    def integer(self, n):
        return self.u64() % n


def hashed_uniform(seed: int, n: int) -> np.ndarray:
    """n uniform floats in [0, 1): SplitMix64 of (seed, i), vectorised."""
    with np.errstate(over="ignore"):
        v = (np.uint64(seed & MASK) * np.uint64(0x9E3779B97F4A7C15)
             + np.arange(n, dtype=np.uint64))
        v = v + np.uint64(0x9E3779B97F4A7C15)
        v = (v ^ (v >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        v = (v ^ (v >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        v = v ^ (v >> np.uint64(31))
    return (v >> np.uint64(40)).astype(np.float64) / float(1 << 24)


# ---- mesh building --------------------------------------------------------------------------

class Part:
    """Positions, normals, UVs in [0,1]^2 and triangle indices of one atlas cell."""

    def __init__(self, positions, normals, uvs, indices):
        self.positions = np.asarray(positions, np.float64).reshape(-1, 3)
        self.normals = np.asarray(normals, np.float64).reshape(-1, 3)
        self.uvs = np.asarray(uvs, np.float64).reshape(-1, 2)
        self.indices = np.asarray(indices, np.int64).reshape(-1)


def grid_quad(origin, u_axis, v_axis, nu, nv, normal, keep=None) -> Part:
    """A planar rectangle origin + s*u_axis + t*v_axis (s,t in [0,1]) cut into nu x nv quads,
    wound so every triangle faces `normal`. `keep(cu, cv)` drops cells (doorways)."""
    origin, u_axis, v_axis, normal = (np.asarray(x, np.float64) for x in
                                      (origin, u_axis, v_axis, normal))
    s = np.linspace(0.0, 1.0, nu + 1)
    t = np.linspace(0.0, 1.0, nv + 1)
    S, T = np.meshgrid(s, t)  # (nv+1, nu+1)
    pos = origin + S[..., None] * u_axis + T[..., None] * v_axis
    uv = np.stack([S, T], -1)
    flip = np.dot(np.cross(u_axis, v_axis), normal) < 0
    idx = []
    for cv in range(nv):
        for cu in range(nu):
            if keep is not None and not keep(cu, cv):
                continue
            a = cv * (nu + 1) + cu
            b, c, d = a + 1, a + nu + 2, a + nu + 1
            if flip:
                idx += [a, c, b, a, d, c]
            else:
                idx += [a, b, c, a, c, d]
    return Part(pos.reshape(-1, 3), np.repeat(normal[None], pos.shape[0] * pos.shape[1], 0),
                uv.reshape(-1, 2), idx)


def box_parts(lo, hi, outward=True, faces=(0, 1, 2, 3, 4, 5), cells=1):
    """The faces of an axis-aligned box, facing out (or in), one part per face."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    ext = hi - lo
    parts = []
    axes = np.eye(3)
    for f in faces:
        axis, positive = f // 2, f % 2 == 0
        n = axes[axis] * (1.0 if positive else -1.0)
        u, v = axes[(axis + 1) % 3], axes[(axis + 2) % 3]
        o = lo.copy()
        if positive:
            o[axis] = hi[axis]
        nn = n if outward else -n
        parts.append(grid_quad(o, u * ext[(axis + 1) % 3], v * ext[(axis + 2) % 3], cells, cells, nn))
    return parts


def wedge_parts(lo, hi):
    """A ramp: a box's bottom, back and slope, plus its two triangular sides (8 triangles)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    parts = [grid_quad((x0, y0, z0), (x1 - x0, 0, 0), (0, 0, z1 - z0), 1, 1, (0, -1, 0)),
             grid_quad((x1, y0, z0), (0, y1 - y0, 0), (0, 0, z1 - z0), 1, 1, (1, 0, 0))]
    slope = np.array([-(y1 - y0), x1 - x0, 0.0])
    slope /= np.linalg.norm(slope)
    parts.append(grid_quad((x0, y0, z0), (x1 - x0, y1 - y0, 0), (0, 0, z1 - z0), 1, 1, slope))
    for z, nz in ((z0, -1.0), (z1, 1.0)):
        p = np.array([[x0, y0, z], [x1, y0, z], [x1, y1, z]])
        n = np.array([0, 0, nz])
        idx = [0, 1, 2] if np.dot(np.cross(p[1] - p[0], p[2] - p[0]), n) > 0 else [0, 2, 1]
        parts.append(Part(p, np.repeat(n[None], 3, 0), [[0, 0], [1, 0], [1, 1]], idx))
    return parts


def atlas_mesh(mesh_id, parts, albedo=(1.0, 1.0, 1.0), flat_normals=False) -> BakeMesh:
    """One mesh with each part in its own cell of a ceil(sqrt(n))^2 UV1 atlas, scaled by 0.9
    with a 0.05 margin (benches/bake.rs:33-44)."""
    cells = math.ceil(math.sqrt(len(parts)))
    pos, nrm, uv1, idx = [], [], [], []
    base = 0
    for k, p in enumerate(parts):
        cell = np.array([k % cells, k // cells], np.float64)
        pos.append(p.positions)
        nrm.append(p.normals)
        uv1.append((cell + p.uvs * 0.9 + 0.05) / cells)
        idx.append(p.indices + base)
        base += len(p.positions)
    positions = np.concatenate(pos).astype(np.float32)
    return BakeMesh(id=mesh_id, positions=positions,
                    indices=np.concatenate(idx).astype(np.uint32),
                    uv1=np.concatenate(uv1).astype(np.float32),
                    normals=None if flat_normals else np.concatenate(nrm).astype(np.float32),
                    albedo=tuple(float(a) for a in albedo),
                    content_hash=splitmix64(mesh_id ^ len(positions)))


def rotation_arc(frm, to):
    """Unit quaternion (x, y, z, w) turning `frm` onto `to` (glam Quat::from_rotation_arc)."""
    frm = np.asarray(frm, np.float64) / np.linalg.norm(frm)
    to = np.asarray(to, np.float64) / np.linalg.norm(to)
    d = float(np.dot(frm, to))
    if d > 1 - 1e-6:
        return (0.0, 0.0, 0.0, 1.0)
    if d < -1 + 1e-6:
        axis = np.cross(frm, [1, 0, 0])
        if np.linalg.norm(axis) < 1e-6:
            axis = np.cross(frm, [0, 1, 0])
        axis /= np.linalg.norm(axis)
        return (float(axis[0]), float(axis[1]), float(axis[2]), 0.0)
    c = np.cross(frm, to)
    q = np.array([c[0], c[1], c[2], 1.0 + d])
    q /= np.linalg.norm(q)
    return tuple(float(x) for x in q.astype(np.float32))


def rotation_x(angle):
    return (math.sin(angle / 2), 0.0, 0.0, math.cos(angle / 2))


def rotation_y(angle):
    return (0.0, math.sin(angle / 2), 0.0, math.cos(angle / 2))


def quat_mul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return (aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
            aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz)


def _options(**kw):
    o = BakeOptions(dynamic_geometry=LIGHTING_ONLY)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


# ---- workload 1: small room ---------------------------------------------------------------

def small_room(seed=1, lights=4):
    """10x4x10 m room with inward faces (12 tris) + 5 cubes (edges U[0.5, 2] m), 4 point lights
    of radius 8 m, 8 texels/m, direct light only."""
    rng = Rng(seed)
    meshes = [atlas_mesh(1, box_parts((-5, 0, -5), (5, 4, 5), outward=False))]
    for i in range(5):
        e = rng.uniform(0.5, 2.0)
        cx, cz = rng.uniform(-5 + e / 2, 5 - e / 2), rng.uniform(-5 + e / 2, 5 - e / 2)
        cy = rng.uniform(0.0, 4.0 - e)
        meshes.append(atlas_mesh(10 + i, box_parts((cx - e / 2, cy, cz - e / 2),
                                                   (cx + e / 2, cy + e, cz + e / 2))))
    ls = [BakeLight(id=100 + i, position=(rng.uniform(-4.5, 4.5), rng.uniform(0.5, 3.5),
                                          rng.uniform(-4.5, 4.5)), radius=8.0)
          for i in range(lights)]
    return BakeInput(meshes, ls), _options(pixel_density=8.0)


# ---- workloads 2 and 3: a grid of rooms ------------------------------------------------------

ROOM = 8.0
ROOM_H = 3.5
GAP = 0.3
DOOR_W, DOOR_H = 1.2, 2.2


def _room_shell(mesh_id, ox, oz, nx, nz, ix, iz, cell, albedo):
    """Floor, ceiling and four inward walls of room (ix, iz), doorways towards neighbours."""
    parts = []
    n = max(1, int(round(ROOM / cell)))
    nh = max(1, int(round(ROOM_H / cell)))
    parts.append(grid_quad((ox, 0, oz), (ROOM, 0, 0), (0, 0, ROOM), n, n, (0, 1, 0)))
    parts.append(grid_quad((ox, ROOM_H, oz), (ROOM, 0, 0), (0, 0, ROOM), n, n, (0, -1, 0)))

    def door(cu, cv):
        u0, u1 = cu / n * ROOM, (cu + 1) / n * ROOM
        v0, v1 = cv / nh * ROOM_H, (cv + 1) / nh * ROOM_H
        mid = ROOM / 2
        inside = (u0 + u1) / 2 > mid - DOOR_W / 2 and (u0 + u1) / 2 < mid + DOOR_W / 2
        return not (inside and (v0 + v1) / 2 < DOOR_H)

    walls = [((ox, 0, oz), (ROOM, 0, 0), (0, 0, 1), iz > 0),          # z = oz, faces +z
             ((ox, 0, oz + ROOM), (ROOM, 0, 0), (0, 0, -1), iz < nz - 1),
             ((ox, 0, oz), (0, 0, ROOM), (1, 0, 0), ix > 0),
             ((ox + ROOM, 0, oz), (0, 0, ROOM), (-1, 0, 0), ix < nx - 1)]
    for o, u, normal, has_door in walls:
        parts.append(grid_quad(o, u, (0, ROOM_H, 0), n, nh, normal, door if has_door else None))
    return atlas_mesh(mesh_id, parts, albedo)


def room_grid(seed=2, rooms=6, lights=64, boxes_per_room=20, bounce=True, cell=0.667,
              soft=False, samples=64):
    """6x6 rooms (8x3.5x8 m, 1.2x2.2 m doorways), 20 boxes/ramps each, 64 point lights of
    radius U[4, 12] with one bounce, albedo U[0.2, 0.8], 16 texels/m."""
    rng = Rng(seed)
    meshes = []
    mesh_id = 1
    for iz in range(rooms):
        for ix in range(rooms):
            ox, oz = ix * (ROOM + GAP), iz * (ROOM + GAP)
            c = cell
            if soft:  # log-normal surface subdivision: per room a cell size around 0.8 m
                c = float(np.clip(0.8 * math.exp(rng.uniform(-1.0, 1.6)), 0.28, 5.6))
            a = rng.uniform(0.2, 0.8)
            meshes.append(_room_shell(mesh_id, ox, oz, rooms, rooms, ix, iz, c, (a, a, a)))
            mesh_id += 1
            for b in range(boxes_per_room):
                ex, ey, ez = rng.uniform(0.3, 1.5), rng.uniform(0.3, 1.8), rng.uniform(0.3, 1.5)
                x = ox + rng.uniform(0.2, ROOM - 0.2 - ex)
                z = oz + rng.uniform(0.2, ROOM - 0.2 - ez)
                a = (rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))
                cells = 1
                if soft:
                    cells = int(np.clip(round(math.exp(rng.uniform(-0.5, 2.0))), 1, 8))
                if rng.integer(4) == 0:
                    parts = wedge_parts((x, 0, z), (x + ex, ey, z + ez))
                else:
                    parts = box_parts((x, 0, z), (x + ex, ey, z + ez), cells=cells)
                meshes.append(atlas_mesh(mesh_id, parts, a))
                mesh_id += 1
    ls = []
    for i in range(lights):
        ix, iz = rng.integer(rooms), rng.integer(rooms)
        pos = (ix * (ROOM + GAP) + rng.uniform(0.5, ROOM - 0.5), rng.uniform(1.0, 3.2),
               iz * (ROOM + GAP) + rng.uniform(0.5, ROOM - 0.5))
        radius = rng.uniform(4.0, 12.0)
        shape = LightShape.point()
        if soft and i % 4 == 2:
            rot = quat_mul(rotation_y(rng.uniform(0, 2 * math.pi)), rotation_x(-math.pi / 2))
            shape = LightShape.rectangle(rot, rng.uniform(0.5, 3.0), rng.uniform(0.5, 3.0))
        elif soft and i % 4 == 3:
            shape = LightShape.tube(rotation_y(rng.uniform(0, 2 * math.pi)), rng.uniform(1.0, 4.0))
        ls.append(BakeLight(id=10_000 + i, position=pos, radius=radius,
                            illumination=SINGLE_BOUNCE if bounce else DIRECT,
                            bounce=BakeBounce(samples=samples), shape=shape))
    opts = _options(pixel_density=16.0)
    if soft:
        opts.area_light_samples = 16
        opts.area_light_min_samples = 16
    return BakeInput(meshes, ls), opts


def soft_rooms(seed=3, rooms=6, lights=128, boxes_per_room=20):
    """Workload 3: the room grid re-meshed with log-normal triangle sizes, 128 lights (64 point,
    32 rectangle, 32 tube), 16 soft samples per texel, direct light only."""
    return room_grid(seed=seed, rooms=rooms, lights=lights, boxes_per_room=boxes_per_room,
                     bounce=False, soft=True)


# ---- workload 4: outdoor ------------------------------------------------------------------

def _fbm(seed, n, octaves=6):
    """fBm value noise on an n x n grid, scaled to [0, 1]."""
    h = np.zeros((n, n))
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = 4 * (2 ** o)
        lattice = hashed_uniform(seed * 131 + o, (cells + 2) ** 2).reshape(cells + 2, cells + 2)
        g = np.linspace(0, cells, n)
        i = np.minimum(g.astype(int), cells - 1)
        f = g - i
        f = f * f * (3 - 2 * f)
        a = lattice[np.ix_(i, i)]
        b = lattice[np.ix_(i, i + 1)]
        c = lattice[np.ix_(i + 1, i)]
        d = lattice[np.ix_(i + 1, i + 1)]
        fx, fy = f[None, :], f[:, None]
        h += amp * ((a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy)
        total += amp
        amp *= 0.5
    h /= total
    return (h - h.min()) / max(h.max() - h.min(), 1e-9)


def _terrain(seed, grid, chunks, rng, first_id=1):
    """fBm heightfield (0..40 m, 1 m spacing) as chunks x chunks meshes facing +y; returns
    (meshes, heights)."""
    heights = (_fbm(seed, grid) * 40.0)
    size = float(grid - 1)
    meshes = []
    per = (grid - 1) // chunks
    mesh_id = first_id
    gx_all, gz_all = np.gradient(heights, axis=1), np.gradient(heights, axis=0)
    for cz in range(chunks):
        for cx in range(chunks):
            x0, z0 = cx * per, cz * per
            x1 = grid - 1 if cx == chunks - 1 else x0 + per
            z1 = grid - 1 if cz == chunks - 1 else z0 + per
            xs, zs = np.arange(x0, x1 + 1), np.arange(z0, z1 + 1)
            X, Z = np.meshgrid(xs, zs)
            H = heights[z0:z1 + 1, x0:x1 + 1]
            pos = np.stack([X - size / 2, H, Z - size / 2], -1).reshape(-1, 3)
            # central-difference normals
            gx = gx_all[z0:z1 + 1, x0:x1 + 1]
            gz = gz_all[z0:z1 + 1, x0:x1 + 1]
            nrm = np.stack([-gx, np.ones_like(gx), -gz], -1)
            nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
            w, h = x1 - x0 + 1, z1 - z0 + 1
            uv = np.stack([(X - x0) / (w - 1), (Z - z0) / (h - 1)], -1).reshape(-1, 2)
            uv = uv * 0.98 + 0.01
            a = (np.arange(h - 1)[:, None] * w + np.arange(w - 1)[None, :]).reshape(-1)
            b, c, d = a + 1, a + w + 1, a + w
            idx = np.stack([a, d, c, a, c, b], -1).reshape(-1)  # faces +y
            col = (rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))
            meshes.append(BakeMesh(id=mesh_id, positions=pos.astype(np.float32),
                                   indices=idx.astype(np.uint32), uv1=uv.astype(np.float32),
                                   normals=nrm.reshape(-1, 3).astype(np.float32), albedo=col,
                                   content_hash=splitmix64(mesh_id)))
            mesh_id += 1
    return meshes, heights


def outdoor(seed=4, grid=512, chunks=8, boxes=2000, point_lights=32, density=4.0,
            sun_samples=32, sky_samples=256, bounce_samples=128):
    """512x512-vertex heightfield (heights 0..40 m, 1 m spacing) in 8x8 chunk meshes, 2000
    boxes and 0.02 m planks, a 0.53 deg sun (4-bit, 32 samples, colored bounce with 128
    samples), a sky (256 samples) and 32 point lights of radius U[4, 12], 4 texels/m."""
    rng = Rng(seed)
    meshes, heights = _terrain(seed, grid, chunks, rng)
    size = float(grid - 1)
    mesh_id = len(meshes) + 1

    def ground(x, z):
        i = int(np.clip(round(z + size / 2), 0, grid - 1))
        j = int(np.clip(round(x + size / 2), 0, grid - 1))
        return float(heights[i, j])

    for b in range(boxes):
        x, z = rng.uniform(-size / 2 + 4, size / 2 - 4), rng.uniform(-size / 2 + 4, size / 2 - 4)
        y = ground(x, z) - 0.2
        col = (rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))
        if b % 4 == 3:  # plank: 0.02 m thick, lifted on its box below
            lx, lz = rng.uniform(1.0, 3.0), rng.uniform(0.2, 0.6)
            y += rng.uniform(0.5, 2.0)
            parts = box_parts((x, y, z), (x + lx, y + 0.02, z + lz))
        else:
            e = (rng.uniform(0.5, 3.0), rng.uniform(0.5, 3.0), rng.uniform(0.5, 3.0))
            parts = box_parts((x, y, z), (x + e[0], y + e[1], z + e[2]))
        meshes.append(atlas_mesh(mesh_id, parts, col))
        mesh_id += 1
    ls = []
    for i in range(point_lights):
        x, z = rng.uniform(-size / 2 + 2, size / 2 - 2), rng.uniform(-size / 2 + 2, size / 2 - 2)
        ls.append(BakeLight(id=20_000 + i, position=(x, ground(x, z) + rng.uniform(1.0, 5.0), z),
                            radius=rng.uniform(4.0, 12.0)))
    sun = rotation_arc((0, 0, 1), (0.35, 1.0, 0.25))
    ls.append(BakeLight(id=30_000, position=(0.0, 0.0, 0.0), radius=1.0,
                        illumination=SINGLE_BOUNCE, bounce=BakeBounce(samples=bounce_samples),
                        shape=LightShape.sun(sun, 0.53)))
    ls.append(BakeLight(id=30_001, position=(0.0, 0.0, 0.0), radius=1.0, shape=LightShape.sky()))
    opts = _options(pixel_density=density, area_light_samples=sun_samples,
                    area_light_min_samples=16, sky_samples=sky_samples, colored_bounce=True)
    return BakeInput(meshes, ls), opts


# ---- workload 5: precision stress ---------------------------------------------------------

def _atlas_triangles(mesh_id, corners, quads, albedo, occludes=True):
    """A mesh of n independent quads (corners (n, 4, 3), as two triangles 0-1-2, 0-2-3) or
    triangles (n, 3, 3), each in its own cell of a square UV1 atlas (0.9 scale, 0.05 margin)."""
    n, k = corners.shape[0], corners.shape[1]
    cells = math.ceil(math.sqrt(n))
    cell = np.stack([np.arange(n) % cells, np.arange(n) // cells], -1).astype(np.float64)
    unit = np.array([[0, 0], [1, 0], [1, 1], [0, 1]] if quads else [[0, 0], [1, 0], [0, 1]], np.float64)
    uv = (cell[:, None, :] + unit[None, :, :] * 0.9 + 0.05) / cells
    base = (np.arange(n) * k)[:, None]
    local = np.array([0, 1, 2, 0, 2, 3] if quads else [0, 1, 2])
    idx = (base + local[None, :]).reshape(-1)
    return BakeMesh(id=mesh_id, positions=corners.reshape(-1, 3).astype(np.float32),
                    indices=idx.astype(np.uint32), uv1=uv.reshape(-1, 2).astype(np.float32),
                    albedo=albedo, occludes=occludes, content_hash=splitmix64(mesh_id ^ n))


def precision_stress(seed=5, grid=1024, chunks=16, boxes=2000, decals=200_000, slivers=20_000,
                     lights=256, density=4.0, area_samples=32, sky_samples=256, bounce_samples=128,
                     decal_lift=1.0e-4, per_mesh=800):
    """The outdoor scene at grid x grid vertices (1024: 2.09 M terrain triangles) plus `decals`
    quads lying on terrain triangles lifted `decal_lift` m along their normal, `slivers` standing
    triangles of aspect ratio log-uniform in [10, 1e4] (1..4 m long), boxes and planks, and
    `lights` mixed lights: a sun (0.53 deg, colored bounce), a sky, then half point lights and a
    quarter each rectangles and tubes, radius U[4, 12]."""
    rng = Rng(seed)
    meshes, heights = _terrain(seed, grid, chunks, rng)
    size = float(grid - 1)
    mesh_id = len(meshes) + 1
    half = size / 2

    def vertex(i, j):  # heightfield vertex at row i (z), column j (x), float64
        return np.stack([j - half, heights[i, j], i - half], -1).astype(np.float64)

    # decals: a kite inside a terrain triangle (barycentric corners), lifted along its normal
    cell_i = (hashed_uniform(seed * 7 + 1, decals) * (grid - 1)).astype(np.int64)
    cell_j = (hashed_uniform(seed * 7 + 2, decals) * (grid - 1)).astype(np.int64)
    upper = hashed_uniform(seed * 7 + 3, decals) < 0.5
    a = vertex(cell_i, cell_j)
    b = vertex(cell_i, cell_j + 1)
    c = vertex(cell_i + 1, cell_j + 1)
    d = vertex(cell_i + 1, cell_j)
    # the terrain's triangles are (a, d, c) and (a, c, b)
    p0, p1, p2 = a, np.where(upper[:, None], d, c), np.where(upper[:, None], c, b)
    n = np.cross(p1 - p0, p2 - p0)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    kite = np.array([[0.15, 0.15], [0.65, 0.15], [0.42, 0.42], [0.15, 0.65]])
    corners = (p0[:, None, :] + kite[None, :, 0:1] * (p1 - p0)[:, None, :]
               + kite[None, :, 1:2] * (p2 - p0)[:, None, :] + decal_lift * n[:, None, :])
    for start in range(0, decals, per_mesh):
        meshes.append(_atlas_triangles(mesh_id, corners[start:start + per_mesh], True,
                                       (rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))))
        mesh_id += 1

    # slivers: standing triangles, long edge L, base width L / aspect
    if slivers:
        x = (hashed_uniform(seed * 7 + 4, slivers) - 0.5) * (size - 8)
        z = (hashed_uniform(seed * 7 + 5, slivers) - 0.5) * (size - 8)
        i = np.clip(np.round(z + half).astype(np.int64), 0, grid - 1)
        j = np.clip(np.round(x + half).astype(np.int64), 0, grid - 1)
        base = np.stack([x, heights[i, j] - 0.05, z], -1)
        length = 1.0 + 3.0 * hashed_uniform(seed * 7 + 6, slivers)
        aspect = 10.0 ** (1.0 + 3.0 * hashed_uniform(seed * 7 + 7, slivers))
        turn = hashed_uniform(seed * 7 + 8, slivers) * 2 * math.pi
        lean = (hashed_uniform(seed * 7 + 9, slivers) - 0.5) * 0.6
        side = np.stack([np.cos(turn), np.zeros_like(turn), np.sin(turn)], -1)
        up = np.stack([-np.sin(turn) * lean, np.ones_like(turn), np.cos(turn) * lean], -1)
        up /= np.linalg.norm(up, axis=-1, keepdims=True)
        tri = np.stack([base, base + side * (length / aspect)[:, None], base + up * length[:, None]], 1)
        for start in range(0, slivers, per_mesh):
            meshes.append(_atlas_triangles(mesh_id, tri[start:start + per_mesh], False, (0.6, 0.6, 0.5)))
            mesh_id += 1

    def ground(x, z):
        i = int(np.clip(round(z + half), 0, grid - 1))
        j = int(np.clip(round(x + half), 0, grid - 1))
        return float(heights[i, j])

    for k in range(boxes):
        x, z = rng.uniform(-half + 4, half - 4), rng.uniform(-half + 4, half - 4)
        y = ground(x, z) - 0.2
        col = (rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8))
        if k % 4 == 3:
            lx, lz = rng.uniform(1.0, 3.0), rng.uniform(0.2, 0.6)
            y += rng.uniform(0.5, 2.0)
            parts = box_parts((x, y, z), (x + lx, y + 0.02, z + lz))
        else:
            e = (rng.uniform(0.5, 3.0), rng.uniform(0.5, 3.0), rng.uniform(0.5, 3.0))
            parts = box_parts((x, y, z), (x + e[0], y + e[1], z + e[2]))
        meshes.append(atlas_mesh(mesh_id, parts, col))
        mesh_id += 1

    sun = rotation_arc((0, 0, 1), (0.35, 1.0, 0.25))
    ls = [BakeLight(id=30_000, position=(0.0, 0.0, 0.0), radius=1.0, illumination=SINGLE_BOUNCE,
                    bounce=BakeBounce(samples=bounce_samples), shape=LightShape.sun(sun, 0.53)),
          BakeLight(id=30_001, position=(0.0, 0.0, 0.0), radius=1.0, shape=LightShape.sky())]
    local = max(lights - 2, 0)
    for k in range(local):
        x, z = rng.uniform(-half + 2, half - 2), rng.uniform(-half + 2, half - 2)
        pos = (x, ground(x, z) + rng.uniform(1.0, 5.0), z)
        shape = LightShape.point()
        if k % 4 == 2:
            rot = quat_mul(rotation_y(rng.uniform(0, 2 * math.pi)), rotation_x(-math.pi / 2))
            shape = LightShape.rectangle(rot, rng.uniform(0.5, 3.0), rng.uniform(0.5, 3.0))
        elif k % 4 == 3:
            shape = LightShape.tube(rotation_y(rng.uniform(0, 2 * math.pi)), rng.uniform(1.0, 4.0))
        ls.append(BakeLight(id=20_000 + k, position=pos, radius=rng.uniform(4.0, 12.0), shape=shape))
    opts = _options(pixel_density=density, area_light_samples=area_samples,
                    area_light_min_samples=16, sky_samples=sky_samples, colored_bounce=True)
    return BakeInput(meshes, ls), opts


WORKLOADS = {
    "small_room": small_room,
    "room_grid": room_grid,
    "soft_rooms": soft_rooms,
    "outdoor": outdoor,
    "precision_stress": precision_stress,
}
