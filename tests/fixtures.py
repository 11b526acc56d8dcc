"""Scene fixtures of the reference's bake tests (src/bake/tests/mod.rs:23-137), as BakeInput
parts: a floor, a cuboid with a 3x2 UV1 atlas, point/area/sun/sky lights."""
import math

import numpy as np

import dynlight_gb300 as dl
from dynlight_gb300 import scenes


def floor(mesh_id, center, half):
    """mod.rs:23-34: a square of side 2*half facing +Y, UV1 spanning it."""
    corners = [(-1.0, -1.0), (1.0, -1.0), (1.0, 1.0), (-1.0, 1.0)]
    c = np.asarray(center, np.float32)
    pos = np.array([c + np.float32([x * half, 0.0, z * half]) for x, z in corners], np.float32)
    uv1 = np.array([((x + 1) * 0.5, (z + 1) * 0.5) for x, z in corners], np.float32)
    return dl.BakeMesh(id=mesh_id, positions=pos, indices=np.array([0, 2, 1, 0, 3, 2], np.uint32),
                       uv1=uv1, normals=np.tile(np.float32([0, 1, 0]), (4, 1)))


def cuboid(mesh_id, lo, hi):
    """mod.rs:37-65: an axis-aligned box with outward faces, each in a 3x2 UV1 atlas cell."""
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    faces = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    pos, nrm, idx, uv1 = [], [], [], []
    for f, n in enumerate(faces):
        n = np.float32(n)
        u = np.float32([1, 0, 0]) if abs(n[1]) > 0.5 else np.float32([0, 1, 0])
        v = np.cross(n, u).astype(np.float32)
        base = len(pos)
        cell = np.float32([f % 3, f // 3])
        for a, b in [(-1.0, -1.0), (1.0, -1.0), (1.0, 1.0), (-1.0, 1.0)]:
            local = n + u * np.float32(a) + v * np.float32(b)
            pos.append((lo + hi) * np.float32(0.5) + local * (hi - lo) * np.float32(0.5))
            nrm.append(n)
            inner = np.float32([(a + 1) * 0.5 * 0.8 + 0.1, (b + 1) * 0.5 * 0.8 + 0.1])
            uv1.append((cell + inner) / np.float32([3.0, 2.0]))
        idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    return dl.BakeMesh(id=mesh_id, positions=np.array(pos, np.float32),
                       indices=np.array(idx, np.uint32), uv1=np.array(uv1, np.float32),
                       normals=np.array(nrm, np.float32))


def point_light(light_id, position, radius, **kw):
    return dl.BakeLight(id=light_id, position=tuple(position), radius=radius, **kw)


def area_light(light_id, position, radius, rotation, size, **kw):
    shape = (dl.LightShape.rectangle(rotation, size[0], size[1]) if size[1] > 0
             else dl.LightShape.tube(rotation, size[0]))
    return dl.BakeLight(id=light_id, position=tuple(position), radius=radius, shape=shape, **kw)


def sun_light(light_id, toward, degrees, **kw):
    rot = scenes.rotation_arc((0, 0, 1), toward)
    return dl.BakeLight(id=light_id, position=(500.0, -300.0, 70.0), radius=0.5,
                        shape=dl.LightShape.sun(rot, degrees), **kw)


def sky_light(light_id, **kw):
    return dl.BakeLight(id=light_id, position=(-40.0, 900.0, 3.0), radius=0.5,
                        shape=dl.LightShape.sky(), **kw)


def options(**kw):
    o = dl.BakeOptions(dynamic_geometry=dl.LIGHTING_ONLY)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def determinism_room():
    """The scene of the reference's determinism test (src/bake/tests/determinism.rs:11-44)."""
    meshes = [floor(5, (0, 0, 0), 3.0), cuboid(3, (-1.0, 0.0, -1.0), (0.0, 1.0, 0.5)),
              cuboid(9, (1.0, 0.2, 1.0), (1.5, 2.0, 1.4)), floor(4, (0.5, 2.5, 0.0), 1.0)]
    lights = [point_light(30, (0.0, 2.0, 0.0), 4.0), point_light(10, (-2.0, 1.5, 2.0), 3.0),
              point_light(20, (2.0, 1.0, -2.0), 5.0), point_light(40, (0.5, 3.0, 0.2), 2.0),
              point_light(50, (-2.5, 0.3, -2.5), 1.5),
              area_light(60, (0.2, 2.4, -0.3), 4.0, scenes.rotation_x(-math.pi / 2), (1.0, 0.6)),
              area_light(70, (-1.5, 1.8, 0.8), 3.0, scenes.rotation_y(0.7), (1.2, 0.0)),
              sun_light(25, (0.3, 1.0, 0.2), 0.53), sun_light(15, (-0.5, 1.0, 0.4), 0.0),
              sky_light(12)]
    return dl.BakeInput(meshes, lights), options(pixel_density=12.0, sky_samples=16)


def triangle_texels(mesh, triangle, size, face=None):
    """The texels whose centers triangle `triangle` of `mesh` covers in a `size`-texel map
    (src/bake/texels.rs triangle_texels, through the oracle), as [(x, y, position)]. `face`
    defaults to the normalized cross product of the triangle's edges."""
    import ctypes as C
    from oracle import oracle as orc
    corners = [int(c) for c in mesh.indices[3 * triangle: 3 * triangle + 3]]
    v = np.float32([mesh.positions[c] for c in corners])
    n = (np.float32([mesh.normals[c] for c in corners]) if mesh.normals is not None
         else np.tile(np.float32([0, 1, 0]), (3, 1)))
    uv = np.float32([mesh.uv1[c] for c in corners])
    if face is None:
        c = np.cross(v[1] - v[0], v[2] - v[0]).astype(np.float32)
        face = c / np.float32(np.linalg.norm(c))
    face = np.ascontiguousarray(face, np.float32)
    cap = size * size
    xy = np.zeros(2 * cap, np.uint32)
    pos = np.zeros(3 * cap, np.float32)
    nrm = np.zeros(3 * cap, np.float32)
    args = [np.ascontiguousarray(a.reshape(-1)) for a in (v, n, uv)]
    count = orc.lib().oracle_texels(0, *(a.ctypes.data_as(C.c_void_p) for a in args),
                                    face.ctypes.data_as(C.c_void_p), size, None, cap,
                                    xy.ctypes.data_as(C.c_void_p), pos.ctypes.data_as(C.c_void_p),
                                    nrm.ctypes.data_as(C.c_void_p))
    assert count <= cap
    xy, pos = xy[:2 * count].reshape(-1, 2), pos[:3 * count].reshape(-1, 3)
    return [(int(a), int(b), p) for (a, b), p in zip(xy, pos)]
