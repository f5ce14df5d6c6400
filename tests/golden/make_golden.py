"""Generate the golden vectors under tests/golden/ from the reference's own code.

Runs oracle/_ref/ref_harness -- the unmodified tyanyuy3125/snch-lbvh headers
compiled as host C++ (oracle/Makefile) -- on seeded inputs and stores inputs
and outputs as compressed .npz fixtures. Needs the reference checkout, so it
runs only where the reference exists; the fixtures it writes are committed.

    python tests/golden/make_golden.py

Harness file layout (little endian):
  in : int64[7] {nv, nt, n_near, n_sil, n_ray, n_smp, n_obj}, verts f32[nv*3],
       tris i32[nt*3], near f32[*3], sil f32[*3], sil_flip u8[], ray_o f32[*3],
       ray_d f32[*3], ray_tmax f32[], smp_c f32[*3], smp_r f32[], smp_u f32[],
       obj_idx i32[], obj_u f32[], obj_v f32[]
  out: int64[2] {E, NN}, tri_edges i32[nt*3], tri_owned i32[nt*3],
       edge_verts i32[E*4], morton u32[nt], nodes u32[NN*4], aabbs f32[NN*6],
       cones f32[NN*5], near {u32 idx, f32 dist}, sil f32, ray {u8 hit, f32 t,
       f32 u, f32 v, u32 idx}, smp {i32 idx, f32 pdf}, obj f32[*3]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from snch_lbvh_gb300 import meshes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def run_harness(verts, tris, q):
    nv, nt = len(verts), len(tris)
    n_near, n_sil, n_ray = len(q["near_pts"]), len(q["sil_pts"]), len(q["ray_o"])
    n_smp, n_obj = len(q["smp_c"]), len(q["obj_idx"])
    n_box, n_line = len(q["box_q"]), len(q["line_o"])
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([nv, nt, n_near, n_sil, n_ray, n_smp, n_obj, n_box, n_line, MAX_OUT], np.int64).tofile(f)
            for a, dt in [(verts, np.float32), (tris, np.int32), (q["near_pts"], np.float32),
                          (q["sil_pts"], np.float32), (q["sil_flip"], np.uint8), (q["ray_o"], np.float32),
                          (q["ray_d"], np.float32), (q["ray_tmax"], np.float32), (q["smp_c"], np.float32),
                          (q["smp_r"], np.float32), (q["smp_u"], np.float32), (q["obj_idx"], np.int32),
                          (q["obj_u"], np.float32), (q["obj_v"], np.float32), (q["box_q"], np.float32),
                          (q["line_o"], np.float32), (q["line_d"], np.float32)]:
                np.ascontiguousarray(a, dtype=dt).tofile(f)
        subprocess.run([oracle.REF_HARNESS, fin, fout], check=True, stdout=subprocess.DEVNULL)
        buf = open(fout, "rb").read()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(buf, dtype=dt, count=n, offset=off)
        off += a.nbytes
        return a.copy()

    E, NN = take(np.int64, 2)
    r = {}
    r["ref_tri_edges"] = take(np.int32, nt * 3).reshape(nt, 3)
    r["ref_tri_owned"] = take(np.int32, nt * 3).reshape(nt, 3)
    r["ref_edge_verts"] = take(np.int32, E * 4).reshape(E, 4)
    r["ref_morton"] = take(np.uint32, nt)
    r["ref_nodes"] = take(np.uint32, NN * 4).reshape(NN, 4)
    r["ref_aabbs"] = take(np.float32, NN * 6).reshape(NN, 6)
    r["ref_cones"] = take(np.float32, NN * 5).reshape(NN, 5)
    tree_ok = nt >= 2
    nn_, ns_ = (n_near, n_sil) if tree_ok else (0, 0)
    rec = take(np.uint8, nn_ * 8).reshape(-1, 8)
    r["ref_near_idx"] = rec[:, :4].copy().view(np.uint32).reshape(-1)
    r["ref_near_dist"] = rec[:, 4:].copy().view(np.float32).reshape(-1)
    r["ref_sil_dist"] = take(np.float32, ns_)
    rec = take(np.uint8, n_ray * 17).reshape(-1, 17)
    r["ref_ray_hit"] = rec[:, 0].copy()
    r["ref_ray_t"] = rec[:, 1:5].copy().view(np.float32).reshape(-1)
    r["ref_ray_uv"] = rec[:, 5:13].copy().view(np.float32).reshape(-1, 2)
    r["ref_ray_idx"] = rec[:, 13:17].copy().view(np.uint32).reshape(-1)
    rec = take(np.uint8, n_smp * 8).reshape(-1, 8)
    r["ref_smp_idx"] = rec[:, :4].copy().view(np.int32).reshape(-1)
    r["ref_smp_pdf"] = rec[:, 4:].copy().view(np.float32).reshape(-1)
    r["ref_obj_pts"] = take(np.float32, n_obj * 3).reshape(-1, 3)
    # overlap / line enumerations: count per query and the first MAX_OUT results,
    # stored padded (0xFFFFFFFF / NaN beyond min(count, MAX_OUT))
    nb, nl = (n_box, n_line) if tree_ok else (0, 0)
    r["ref_box_count"] = np.zeros(nb, np.uint32)
    r["ref_box_idx"] = np.full((nb, MAX_OUT), 0xFFFFFFFF, np.uint32)
    for k in range(nb):
        c = int(take(np.uint32, 1)[0])
        r["ref_box_count"][k] = c
        r["ref_box_idx"][k, :min(c, MAX_OUT)] = take(np.uint32, min(c, MAX_OUT))
    r["ref_line_count"] = np.zeros(nl, np.uint32)
    r["ref_line_idx"] = np.full((nl, MAX_OUT), 0xFFFFFFFF, np.uint32)
    r["ref_line_t"] = np.full((nl, MAX_OUT), np.nan, np.float32)
    for k in range(nl):
        c = int(take(np.uint32, 1)[0])
        r["ref_line_count"][k] = c
        rec = take(np.uint8, 8 * min(c, MAX_OUT)).reshape(-1, 8)
        r["ref_line_idx"][k, :len(rec)] = rec[:, :4].copy().view(np.uint32).reshape(-1)
        r["ref_line_t"][k, :len(rec)] = rec[:, 4:].copy().view(np.float32).reshape(-1)
    assert off == len(buf), (off, len(buf))
    return r


MAX_OUT = 64  # results kept per overlap / line query (the count is the full one)


def make_region_queries(verts, seed, n=256):
    """AABB-overlap and line queries from their own generator (the point / ray
    queries above keep their values): boxes of random centre and log-uniform
    size, point boxes, a box holding everything and an empty one; lines through
    random points with random and axis-aligned directions (zero components make
    the slab test meet 0 * inf)."""
    rng = np.random.default_rng(seed + 1000)
    v = verts.astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    c, h = 0.5 * (lo + hi), 0.5 * np.maximum(hi - lo, 1e-3) * 1.5
    cen = c + (rng.random((n, 3)) * 2 - 1) * h
    half = np.exp(rng.uniform(np.log(1e-3), np.log(h.max()), (n, 3)))
    half[: n // 16] = 0.0  # point boxes
    boxes = np.concatenate([cen - half, cen + half], 1)
    boxes[-1] = np.concatenate([lo - 1, hi + 1])  # everything
    boxes[-2] = np.concatenate([hi + 1, hi + 2])  # nothing
    o = c + (rng.random((n, 3)) * 2 - 1) * h
    d = rng.standard_normal((n, 3))
    axis = rng.integers(0, 3, n)
    axial = rng.random(n) < 0.2
    d[axial] = 0.0
    d[axial, axis[axial]] = 1.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return {"box_q": boxes.astype(np.float32), "line_o": o.astype(np.float32), "line_d": d.astype(np.float32)}


def make_queries(verts, tris, seed, n_rand=512, extra=True):
    """Random points in the AABB x 1.5 plus exact-tie probes (vertices, edge
    midpoints, face centroids, offset along face normals), rays (random and
    axis-aligned), sphere draws and on-object samples."""
    rng = np.random.default_rng(seed)
    v = verts.astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    c, h = 0.5 * (lo + hi), 0.5 * np.maximum(hi - lo, 1e-3) * 1.5
    pts = [c + (rng.random((n_rand, 3)) * 2 - 1) * h]
    if extra:
        k = min(len(tris), 64)
        sel = rng.choice(len(tris), k, replace=False)
        a, b, cc = v[tris[sel, 0]], v[tris[sel, 1]], v[tris[sel, 2]]
        n = np.cross(b - a, cc - a)
        nn = np.linalg.norm(n, axis=1, keepdims=True)
        n = np.where(nn > 0, n / np.where(nn > 0, nn, 1), 0)
        pts += [a, 0.5 * (a + b), (a + b + cc) / 3, (a + b + cc) / 3 + 0.01 * n, 0.5 * (a + b) - 0.02 * n]
    pts = np.concatenate(pts, 0).astype(np.float32)
    q = {"near_pts": pts, "sil_pts": pts, "sil_flip": (rng.random(len(pts)) < 0.5).astype(np.uint8)}
    nr = len(pts)
    d = rng.standard_normal((nr, 3))
    axis = rng.integers(0, 3, nr)
    axial = rng.random(nr) < 0.15
    d[axial] = 0.0
    d[axial, axis[axial]] = np.where(rng.random(axial.sum()) < 0.5, -1.0, 1.0)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    q["ray_o"] = pts
    q["ray_d"] = d.astype(np.float32)
    q["ray_tmax"] = np.where(rng.random(nr) < 0.2, np.float32(np.inf),
                             np.exp(rng.uniform(np.log(1e-3), np.log(4 * h.max()), nr))).astype(np.float32)
    q["smp_c"] = pts
    q["smp_r"] = np.exp(rng.uniform(np.log(1e-3), np.log(2 * h.max()), nr)).astype(np.float32)
    q["smp_u"] = rng.random(nr).astype(np.float32)
    m = min(256, 4 * len(tris))
    q["obj_idx"] = rng.integers(0, len(tris), m).astype(np.int32)
    q["obj_u"] = rng.random(m).astype(np.float32)
    q["obj_v"] = rng.random(m).astype(np.float32)
    return q


def cases():
    tet_v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    tet_f = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]], np.int32)
    yield "tetra", tet_v, tet_f, 11
    yield "single_tri", np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]], np.int32), 12
    yield "two_tri", np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32), \
        np.array([[0, 1, 2], [0, 2, 3]], np.int32), 13
    # open flat grid: coplanar neighbours (dihedral branch of is_silhouette_edge) and boundary edges
    g = 12
    xs, ys = np.meshgrid(np.arange(g + 1), np.arange(g + 1), indexing="ij")
    gv = np.stack([xs.ravel() / g, ys.ravel() / g, np.zeros(xs.size)], 1).astype(np.float32)
    gi = np.arange(g)[:, None] * (g + 1) + np.arange(g)[None, :]
    gf = np.concatenate([np.stack([gi, gi + g + 1, gi + g + 2], -1).reshape(-1, 3),
                         np.stack([gi, gi + g + 2, gi + 1], -1).reshape(-1, 3)]).astype(np.int32)
    yield "open_grid", gv, gf, 14
    v, f = meshes.noisy_icosphere(3, 1.0, 0.01, seed=5)
    yield "ico3", v, f, 15
    v, f = meshes.noisy_torus(0.4, 0.1, 24, 12, 0.004, seed=6)
    yield "torus_small", v, f, 16
    # every triangle twice (and some three times): duplicated Morton codes force
    # the 64-bit key path (bvh.cuh:459-476); edges with 4-6 faces exercise the
    # overwrite order of compute_silhouettes
    v, f = meshes.noisy_icosphere(2, 1.0, 0.02, seed=7)
    f = np.concatenate([f, f[::-1], f[:40]]).astype(np.int32)
    yield "duplicated", v, f, 17
    # degenerate triangles: a repeated vertex id and collinear vertices
    v, f = meshes.noisy_icosphere(1, 1.0, 0.0, seed=8)
    extra_v = np.array([[2, 0, 0], [2.5, 0, 0], [3, 0, 0]], np.float32)
    v = np.concatenate([v, extra_v]).astype(np.float32)
    n0 = len(v) - 3
    f = np.concatenate([f, [[n0, n0 + 1, n0 + 2], [n0, n0, n0 + 1]]]).astype(np.int32)
    yield "degenerate", v, f, 18
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    yield "cfg1_icosphere_l5", v, f, 19


def write_obj_case(path, verts, tris):
    """An OBJ file of a golden mesh in the forms the reference's reader handles:
    comments, object / group / smoothing / normal / texture lines (ignored),
    varied number formats and spacing, a 4th vertex coordinate, CRLF line ends,
    quads (the first three indices count) and blank lines."""
    rng = np.random.default_rng(99)
    lines = ["# golden OBJ case", "o torus", "g part0", "s off", ""]
    for k, p in enumerate(verts):
        xs = [repr(float(x)) for x in p]
        if k % 7 == 1:
            xs = [f"{float(x):.9e}" for x in p]
        sep = "\t" if k % 5 == 2 else "  " if k % 5 == 3 else " "
        extra = " 1.0" if k % 11 == 4 else ""
        lines.append("v" + sep + sep.join(xs) + extra + ("\r" if k % 13 == 6 else ""))
        if k % 17 == 0:
            lines.append(f"vn 0 0 1\nvt {rng.random():.3f} {rng.random():.3f}")
    for k, t in enumerate(tris):
        ids = [str(int(i) + 1) for i in t]
        if k % 9 == 3:
            ids.append(str(int(t[0]) + 1))  # a quad: the reader keeps the first three
        lines.append("f " + " ".join(ids) + ("\r" if k % 10 == 7 else ""))
        if k % 50 == 0:
            lines.append("")
    with open(path, "w", newline="") as f:
        f.write("\n".join(lines) + "\n")


def obj_case():
    d = os.path.join(OUT, "obj")
    os.makedirs(d, exist_ok=True)
    v, f = meshes.noisy_torus(0.4, 0.1, 24, 12, 0.004, seed=6)
    path = os.path.join(d, "torus.obj")
    write_obj_case(path, v.astype(np.float32), f)
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.bin")
        subprocess.run([oracle.REF_HARNESS, "--obj", path, out], check=True)
        buf = open(out, "rb").read()
    nv, nt = np.frombuffer(buf, np.int64, 2)
    rv = np.frombuffer(buf, np.float32, 3 * nv, 16).reshape(-1, 3)
    rt = np.frombuffer(buf, np.int32, 3 * nt, 16 + 12 * nv).reshape(-1, 3)
    np.savez_compressed(os.path.join(d, "torus_ref.npz"), ref_verts=rv, ref_tris=rt)
    print(f"obj/torus.obj          verts={nv} tris={nt}")


# ---------------------------------------------------------------- 2D scenes
def polygon(n, r=1.0, c=(0.0, 0.0), noise=0.0, seed=0, reverse=False):
    rng = np.random.default_rng(seed)
    a = np.linspace(0, 2 * np.pi, n, endpoint=False)
    rr = r * (1 + noise * rng.standard_normal(n))
    v = np.stack([c[0] + rr * np.cos(a), c[1] + rr * np.sin(a)], 1)
    s = np.stack([np.arange(n), (np.arange(n) + 1) % n], 1)
    if reverse:
        s = s[:, ::-1]
    return v, s


def cases_2d():
    yield "square", np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32), \
        np.array([[0, 1], [1, 2], [2, 3], [3, 0]], np.int32), 31
    yield "single_seg", np.array([[0, 0], [1, 0.5]], np.float32), np.array([[0, 1]], np.int32), 32
    yield "two_seg", np.array([[0, 0], [1, 0], [1, 1]], np.float32), np.array([[0, 1], [1, 2]], np.int32), 33
    v, s = polygon(64, noise=0.02, seed=1)
    yield "circle64", v.astype(np.float32), s.astype(np.int32), 34
    # a domain with a hole: outer loop counter-clockwise, inner loop clockwise
    vo, so = polygon(48, 1.0, noise=0.01, seed=2)
    vi, si = polygon(24, 0.4, c=(0.1, -0.05), noise=0.01, seed=3, reverse=True)
    yield "two_loops", np.concatenate([vo, vi]).astype(np.float32), \
        np.concatenate([so, si + len(vo)]).astype(np.int32), 35
    # open zig-zag polyline: end vertices have one segment
    x = np.linspace(0, 2, 41)
    v = np.stack([x, 0.2 * (np.arange(41) % 2)], 1)
    yield "open_polyline", v.astype(np.float32), np.stack([np.arange(40), np.arange(1, 41)], 1).astype(np.int32), 36
    # independent random segments (every vertex is an end point)
    rng = np.random.default_rng(7)
    a = rng.random((150, 2))
    b = a + 0.05 * rng.standard_normal((150, 2))
    v = np.concatenate([a, b]).astype(np.float32)
    yield "random_segments", v, np.stack([np.arange(150), np.arange(150, 300)], 1).astype(np.int32), 37
    # every segment twice: equal Morton codes (the 64-bit key path) and shared vertices
    v, s = polygon(32, noise=0.03, seed=4)
    yield "duplicated_2d", v.astype(np.float32), np.concatenate([s, s]).astype(np.int32), 38
    v, s = polygon(4096, noise=0.005, seed=5)
    yield "circle4096", v.astype(np.float32), s.astype(np.int32), 39


def make_queries_2d(verts, segs, seed, n_rand=512):
    """Points in the box x 1.5 plus vertex, midpoint and offset probes; rays
    (random and axis-aligned); circles with log-uniform radii."""
    rng = np.random.default_rng(seed)
    v = verts.astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    c, h = 0.5 * (lo + hi), 0.5 * np.maximum(hi - lo, 1e-3) * 1.5
    k = min(len(segs), 64)
    sel = rng.choice(len(segs), k, replace=False)
    a, b = v[segs[sel, 0]], v[segs[sel, 1]]
    d = b - a
    nrm = np.stack([d[:, 1], -d[:, 0]], 1)
    nn = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(nn > 0, nrm / np.where(nn > 0, nn, 1), 0)
    pts = np.concatenate([c + (rng.random((n_rand, 2)) * 2 - 1) * h, a, 0.5 * (a + b),
                          0.5 * (a + b) + 0.01 * nrm, a - 0.02 * nrm]).astype(np.float32)
    nr = len(pts)
    dd = rng.standard_normal((nr, 2))
    axial = rng.random(nr) < 0.15
    ax = rng.integers(0, 2, nr)
    dd[axial] = 0.0
    dd[axial, ax[axial]] = np.where(rng.random(axial.sum()) < 0.5, -1.0, 1.0)
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    return {"near_pts": pts, "sil_pts": pts, "sil_flip": (rng.random(nr) < 0.5).astype(np.uint8),
            "ray_o": pts, "ray_d": dd.astype(np.float32),
            "ray_tmax": np.where(rng.random(nr) < 0.2, np.float32(np.inf),
                                 np.exp(rng.uniform(np.log(1e-3), np.log(4 * h.max()), nr))).astype(np.float32),
            "smp_c": pts, "smp_r": np.exp(rng.uniform(np.log(1e-3), np.log(2 * h.max()), nr)).astype(np.float32),
            "smp_u": rng.random(nr).astype(np.float32)}


def run_harness_2d(verts, segs, q):
    nv, nt = len(verts), len(segs)
    nq = len(q["near_pts"])
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([nv, nt, nq, nq, nq, nq], np.int64).tofile(f)
            for a, dt in [(verts, np.float32), (segs, np.int32), (q["near_pts"], np.float32),
                          (q["sil_pts"], np.float32), (q["sil_flip"], np.uint8), (q["ray_o"], np.float32),
                          (q["ray_d"], np.float32), (q["ray_tmax"], np.float32), (q["smp_c"], np.float32),
                          (q["smp_r"], np.float32), (q["smp_u"], np.float32)]:
                np.ascontiguousarray(a, dtype=dt).tofile(f)
        subprocess.run([oracle.REF_HARNESS, "--2d", fin, fout], check=True, stdout=subprocess.DEVNULL)
        buf = open(fout, "rb").read()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(buf, dtype=dt, count=n, offset=off)
        off += a.nbytes
        return a.copy()

    nn = 2 * nt - 1
    r = {"ref_sv": take(np.int32, 4 * nv).reshape(nv, 4), "ref_seg_owned": take(np.int32, 2 * nt).reshape(nt, 2),
         "ref_morton": take(np.uint32, nt), "ref_nodes": take(np.uint32, 4 * nn).reshape(nn, 4),
         "ref_aabbs": take(np.float32, 4 * nn).reshape(nn, 4), "ref_cones": take(np.float32, 4 * nn).reshape(nn, 4)}
    m = nq if nt >= 2 else 0
    rec = take(np.uint8, 8 * m).reshape(-1, 8)
    r["ref_near_idx"] = rec[:, :4].copy().view(np.uint32).reshape(-1)
    r["ref_near_dist"] = rec[:, 4:].copy().view(np.float32).reshape(-1)
    r["ref_sil_dist"] = take(np.float32, m)
    rec = take(np.uint8, 13 * m).reshape(-1, 13)
    r["ref_ray_hit"] = rec[:, 0].copy()
    r["ref_ray_t"] = rec[:, 1:5].copy().view(np.float32).reshape(-1)
    r["ref_ray_s"] = rec[:, 5:9].copy().view(np.float32).reshape(-1)
    r["ref_ray_idx"] = rec[:, 9:13].copy().view(np.uint32).reshape(-1)
    rec = take(np.uint8, 8 * m).reshape(-1, 8)
    r["ref_smp_idx"] = rec[:, :4].copy().view(np.int32).reshape(-1)
    r["ref_smp_pdf"] = rec[:, 4:].copy().view(np.float32).reshape(-1)
    assert off == len(buf), (off, len(buf))
    return r


def main_2d():
    d = os.path.join(OUT, "2d")
    os.makedirs(d, exist_ok=True)
    for name, v, sg, seed in cases_2d():
        q = make_queries_2d(v, sg, seed, n_rand=2048 if name == "circle4096" else 512)
        r = run_harness_2d(v, sg, q)
        path = os.path.join(d, f"{name}.npz")
        np.savez_compressed(path, verts=v, segs=sg, **q, **r)
        print(f"2d/{name:20s} segs={len(sg):6d} -> {os.path.getsize(path)/1024:.0f} KiB")


def main():
    oracle.build()
    main_2d()
    obj_case()
    for name, v, f, seed in cases():
        q = make_queries(v, f, seed, n_rand=2048 if name.startswith("cfg1") else 512)
        q.update(make_region_queries(v, seed))
        tree = oracle.Tree(v, f)
        depth = tree.max_depth()
        assert depth < 60, f"{name}: tree depth {depth} would overflow the reference's 64-entry stacks"
        r = run_harness(v, f, q)
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, verts=v, tris=f, **q, **r)
        print(f"{name:22s} tris={len(f):6d} depth={depth:3d} unique={tree.unique} -> {os.path.getsize(path)/1024:.0f} KiB")


if __name__ == "__main__":
    main()
