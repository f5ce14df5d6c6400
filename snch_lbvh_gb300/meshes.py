"""Seeded synthetic triangle meshes and query batches for the SNCH-LBVH workloads.

The reference ships no meshes (its benchmark loads .obj files that are not in
the repository, benchmark.cu:319-324), so every workload here is generated
from a seed:

* ``noisy_icosphere`` -- subdivided icosahedron on a sphere, each vertex
  displaced along its (pre-noise) normal by N(0, sigma^2).
* ``noisy_torus`` -- (nu x nv) parametric torus, same displacement.
* ``wost_scene`` -- 64 placed meshes (icospheres and tori alternating) with a
  total of about two million triangles in the unit cube, plus per-face
  Dirichlet/Neumann flags.

Vertices are float32 x 3, faces int32 x 3 (counter-clockwise seen from outside).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_T = (1.0 + math.sqrt(5.0)) / 2.0
_ICO_VERTS = np.array(
    [(-1, _T, 0), (1, _T, 0), (-1, -_T, 0), (1, -_T, 0), (0, -1, _T), (0, 1, _T),
     (0, -1, -_T), (0, 1, -_T), (_T, 0, -1), (_T, 0, 1), (-_T, 0, -1), (-_T, 0, 1)],
    dtype=np.float64)
_ICO_FACES = np.array(
    [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
     (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
     (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], dtype=np.int64)


def _normalize(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def icosphere(level: int, radius: float = 1.0):
    """Unit icosahedron subdivided ``level`` times: 20*4^level faces, 10*4^level+2 vertices."""
    verts = _normalize(_ICO_VERTS.copy())
    faces = _ICO_FACES.copy()
    for _ in range(level):
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        e = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mids = _normalize(0.5 * (verts[uniq[:, 0]] + verts[uniq[:, 1]]))
        m = len(verts) + inv.reshape(3, -1)
        ab, bc, ca = m[0], m[1], m[2]
        faces = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                                np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)], 0)
        verts = np.concatenate([verts, mids], 0)
    return verts * radius, faces.astype(np.int32), _normalize(verts)


def torus(major: float, minor: float, nu: int, nv: int):
    """Parametric torus around z: 2*nu*nv faces, nu*nv vertices, outward normals."""
    u = 2.0 * np.pi * np.arange(nu) / nu
    v = 2.0 * np.pi * np.arange(nv) / nv
    uu, vv = np.meshgrid(u, v, indexing="ij")
    cu, su, cv, sv = np.cos(uu), np.sin(uu), np.cos(vv), np.sin(vv)
    verts = np.stack([(major + minor * cv) * cu, (major + minor * cv) * su, minor * sv], -1).reshape(-1, 3)
    normals = np.stack([cv * cu, cv * su, sv], -1).reshape(-1, 3)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    p00 = (i * nv + j)
    p10 = (((i + 1) % nu) * nv + j)
    p11 = (((i + 1) % nu) * nv + (j + 1) % nv)
    p01 = (i * nv + (j + 1) % nv)
    t0 = np.stack([p00, p10, p11], -1).reshape(-1, 3)
    t1 = np.stack([p00, p11, p01], -1).reshape(-1, 3)
    faces = np.concatenate([t0, t1], 0)
    # orient counter-clockwise seen from outside
    a, b, c = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
    n = np.cross(b - a, c - a)
    outward = (n * normals[faces[:, 0]]).sum(1) > 0
    faces[~outward] = faces[~outward][:, [0, 2, 1]]
    return verts, faces.astype(np.int32), normals


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform rotation from a normalised Gaussian quaternion."""
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def noisy_icosphere(level: int = 5, radius: float = 1.0, sigma: float = 0.01, seed: int = 0):
    """Level-``level`` icosphere, vertices displaced along the sphere normal by N(0, sigma^2)."""
    rng = np.random.default_rng(seed)
    verts, faces, normals = icosphere(level, radius)
    verts = verts + normals * rng.standard_normal((len(verts), 1)) * sigma
    return verts.astype(np.float32), faces


def noisy_torus(major: float, minor: float, nu: int, nv: int, sigma: float, seed: int = 0):
    rng = np.random.default_rng(seed)
    verts, faces, normals = torus(major, minor, nu, nv)
    verts = verts + normals * rng.standard_normal((len(verts), 1)) * sigma
    return verts.astype(np.float32), faces


def box_queries(verts: np.ndarray, n: int, scale: float = 1.2, seed: int = 1) -> np.ndarray:
    """n points uniform in the mesh AABB scaled by ``scale`` about its centre."""
    rng = np.random.default_rng(seed)
    lo, hi = verts.min(0).astype(np.float64), verts.max(0).astype(np.float64)
    c, h = 0.5 * (lo + hi), 0.5 * (hi - lo) * scale
    return (c + (rng.random((n, 3)) * 2.0 - 1.0) * h).astype(np.float32)


@dataclass
class Scene:
    verts: np.ndarray        # float32 [V, 3]
    faces: np.ndarray        # int32 [F, 3]
    face_flags: np.ndarray   # uint8 [F]: 1 = Neumann, 0 = Dirichlet
    mesh_offsets: np.ndarray  # int64 [M+1] face offsets of the placed meshes


# Tessellation of the two-million-triangle scene: 32 level-5 icospheres
# (20,480 faces) and 32 tori of 205 x 102 quads (41,820 faces): 1,993,600 faces.
WOST_MESHES = 64
WOST_TORUS_NU, WOST_TORUS_NV = 205, 102
WOST_ICO_LEVEL = 5


def place_in_unit_cube(verts: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """Random rotation about the centroid, then a translation that keeps the
    mesh inside [0,1]^3 where it fits (meshes wider than the cube are centred)."""
    v = verts.astype(np.float64)
    v = (v - v.mean(0)) @ random_rotation(rng).T
    lo_t, hi_t = -v.min(0), 1.0 - v.max(0)
    t = np.where(lo_t <= hi_t, lo_t + rng.random(3) * (hi_t - lo_t), 0.5 * (lo_t + hi_t))
    return v + t


def wost_scene(seed: int = 0, n_meshes: int = WOST_MESHES, torus_nu: int = WOST_TORUS_NU,
               torus_nv: int = WOST_TORUS_NV, ico_level: int = WOST_ICO_LEVEL) -> Scene:
    """Noisy tori and icospheres (alternating), major radius U[0.1, 0.5], torus
    minor radius 0.25 x major, rigid random placement in the unit cube, vertex
    noise sigma = 0.5 % of the mesh's size, per-face Neumann flag Bernoulli(0.5)."""
    rng = np.random.default_rng(seed)
    vs, fs, offs = [], [], [0]
    nv = 0
    for k in range(n_meshes):
        major = rng.uniform(0.1, 0.5)
        sub = int(rng.integers(0, 2**31 - 1))
        if k % 2 == 0:
            size = 2.0 * major
            v, f = noisy_icosphere(ico_level, major, 0.005 * size, sub)
        else:
            minor = 0.25 * major
            size = 2.0 * (major + minor)
            v, f = noisy_torus(major, minor, torus_nu, torus_nv, 0.005 * size, sub)
        v = place_in_unit_cube(v, rng)
        vs.append(v.astype(np.float32))
        fs.append(f + nv)
        nv += len(v)
        offs.append(offs[-1] + len(f))
    faces = np.concatenate(fs, 0).astype(np.int32)
    flags = (rng.random(len(faces)) < 0.5).astype(np.uint8)
    return Scene(np.concatenate(vs, 0), faces, flags, np.asarray(offs, dtype=np.int64))


def wost_queries(n_near: int, n_sil: int, n_ray: int, n_smp: int, seed: int = 1) -> dict:
    """Query batches of the walk-on-stars set in the unit cube: nearest and
    silhouette points U([0,1]^3) (flip = false); rays with U([0,1]^3) origins,
    uniform unit directions and tmax log-uniform in [1e-3, 1]; sphere draws with
    centres U([0,1]^3), radii log-uniform in [1e-3, 0.5] and u ~ U[0,1)."""
    rng = np.random.default_rng(seed)
    q = {}
    q["near_pts"] = rng.random((n_near, 3), dtype=np.float32)
    q["sil_pts"] = rng.random((n_sil, 3), dtype=np.float32)
    q["sil_flip"] = np.zeros(n_sil, dtype=np.uint8)
    q["ray_o"] = rng.random((n_ray, 3), dtype=np.float32)
    d = rng.standard_normal((n_ray, 3), dtype=np.float32)
    q["ray_d"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    q["ray_tmax"] = np.exp(rng.uniform(math.log(1e-3), 0.0, n_ray)).astype(np.float32)
    q["smp_c"] = rng.random((n_smp, 3), dtype=np.float32)
    q["smp_r"] = np.exp(rng.uniform(math.log(1e-3), math.log(0.5), n_smp)).astype(np.float32)
    q["smp_u"] = rng.random(n_smp, dtype=np.float32)
    return q


def batched_meshes(seed: int = 5, count: int = 256, lo: float = 1e3, hi: float = 5e5):
    """Independent meshes of the batched workload: alternating noisy icospheres
    and tori, triangle counts log-uniform in [lo, hi] (icospheres: the nearest
    subdivision level, 20 * 4^L faces; tori: nu x nv quads with nv = nu / 2),
    noise sigma = 0.5 % of the mesh's size, each placed in the unit cube.
    Returns a list of (float32 vertices, int32 faces)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        major = rng.uniform(0.1, 0.5)
        sub = int(rng.integers(0, 2**31 - 1))
        if k % 2 == 0:
            level = int(np.clip(np.rint(np.log(target / 20.0) / np.log(4.0)), 1, 7))
            v, f = noisy_icosphere(level, major, 0.005 * 2.0 * major, sub)
        else:
            nu = max(6, int(round(np.sqrt(target))))
            nv = max(3, int(round(target / (2.0 * nu))))
            minor = 0.25 * major
            v, f = noisy_torus(major, minor, nu, nv, 0.005 * 2.0 * (major + minor), sub)
        out.append((place_in_unit_cube(v, rng).astype(np.float32), f.astype(np.int32)))
    return out
