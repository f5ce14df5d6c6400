#!/usr/bin/env python
"""Throughput of the SNCH-LBVH hot path on GB300 (queries/s, walk-on-stars query set).

Workload (one "step"): on the seeded two-million-triangle scene (64 noisy tori
and icospheres in the unit cube, 1,993,600 triangles), rebuild the silhouette
topology and the LBVH, then run 16M nearest-primitive, 16M nearest-silhouette
and 16M ray queries and 4M SampleTriangleInSphere draws.

  value  = queries per second of the whole step, device-timed with CUDA events
           on the launching stream, inputs resident in HBM (N ranks: sum over
           ranks / max rank time; each rank runs the full step: weak scaling);
  e2e    = the same through the host-buffer C-ABI calls (scene upload, build,
           snch_*_host queries with their H2D/D2H copies) on pinned host memory;
  roofline = algorithmic bytes of the dominant query kernel (reference record
           sizes x the kernel's own per-query visit counts) / its event time;
  cpu_baseline = the CPU restatement (oracle/) on the host cores, bounded sample.

Outside the timed step (single GPU): the learned radius on the same batches,
the 20,480-triangle icosphere (1M nearest queries; learned radius on 16M
points), 256 batched meshes (autotuned, graph-captured) and a 1M-walker
walk-on-stars trace.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--scale F]
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("queries/sec (walk-on-stars query set: nearest, silhouette, ray, sphere sample) on the 2M-triangle "
          "scene")
FULL = {"near": 16_000_000, "sil": 16_000_000, "ray": 16_000_000, "smp": 4_000_000}
# kernels the default configuration runs for each query type (Morton-ordered
# 16M-query batches, 8 queries per triangle: nearest and silhouette batches
# run as persistent warp packets, rays as warps taking 32 rays at a time)
KERNEL_OF = {"near": "nearest_packet_persistent_kernel", "sil": "silhouette_packet_persistent_kernel",
             "ray": "ray_pool_kernel", "smp": "sample_kernel"}
# algorithmic bytes per query, reference record sizes: input + output + per
# expanded internal node (2 child boxes + 2 child refs [+ 2 cones]) + per leaf
# (vertex ids + vertices [silhouette: owned-edge ids]) + per silhouette edge
# (4 vertex ids + 4 vertices); multiplied by the visits the measured kernel makes
BYTES_IO = {"near": 12 + 8, "sil": 13 + 8, "ray": 28 + 20, "smp": 20 + 8}
BYTES_NODE = {"near": 56, "sil": 96, "ray": 56, "smp": 56}
BYTES_LEAF = {"near": 48, "sil": 12, "ray": 48, "smp": 52}
BYTES_EDGE = 64


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the query batches (1.0 = full workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-radius leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-meshes leg")
    ap.add_argument("--no-wost", action="store_true", help="skip the walk-on-stars leg")
    ap.add_argument("--no-icosphere", action="store_true", help="skip the 20,480-triangle icosphere leg")
    ap.add_argument("--no-sort", action="store_true", help="skip the radix-sort leg")
    ap.add_argument("--sort-only", action="store_true",
                    help="run only the radix-sort leg (16M pairs) and print its object (for profiling)")
    ap.add_argument("--output-scatter", type=int, default=-1, choices=[-1, 0, 1],
                    help="SNCH_OPT_OUTPUT_SCATTER of the step's scene (-1: the library default)")
    ap.add_argument("--top-levels", type=int, default=-1,
                    help="SNCH_OPT_TOP_LEVELS of the step's scene (-1: the library default)")
    ap.add_argument("--ray-order", type=int, default=-1, choices=[-1, 0, 1],
                    help="SNCH_OPT_RAY_ORDER of the step's scene (-1: the library default)")
    ap.add_argument("--order-bits", type=int, default=0,
                    help="SNCH_OPT_ORDER_BITS of the step's scene (0: the library default)")
    ap.add_argument("--host-chunk", type=int, default=0,
                    help="SNCH_OPT_HOST_CHUNK of the end-to-end leg's scenes (0: the library default)")
    ap.add_argument("--persistent-min", type=int, default=0,
                    help="SNCH_OPT_PACKET_PERSISTENT_MIN of the step's scene (0: the library default, 2^23); "
                         "lets a reduced --scale run the persistent packet kernels of the full workload")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return ws, int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank scalar (a step time) over the default process group.
    The multi-GPU form runs replicas: every rank builds its own scene and answers
    its own full batches (queries are independent), so this and the barrier are
    the only collectives."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_name(counts, ntri):
    return (f"wost_2m: {ntri:,} triangles (64 noisy tori + icospheres in the unit cube); step = silhouette "
            f"topology + LBVH build + {counts['near']:,} nearest + {counts['sil']:,} silhouette + "
            f"{counts['ray']:,} ray + {counts['smp']:,} sphere-sample queries")


def bit_mismatches(a, b):
    """Number of entries of a and b (same shape and dtype) whose bits differ."""
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    if a.shape != b.shape or a.dtype.itemsize != b.dtype.itemsize:
        return -1
    w = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
    return int(np.count_nonzero(a.view(w) != b.view(w)))


def bench_config(counts, ntri, ws):
    """The `config` of both arms' JSON lines (the same workload)."""
    return {"workload": workload_name(counts, ntri),
            "l2": "inputs larger than L2: 192 MB per 16M-query array, >1 GB of tree records",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}


def make_workload(scale, seed):
    from snch_lbvh_gb300 import meshes
    sc = meshes.wost_scene(seed=0)
    counts = {k: max(1, int(v * scale)) for k, v in FULL.items()}
    q = meshes.wost_queries(counts["near"], counts["sil"], counts["ray"], counts["smp"], seed=seed)
    return sc, counts, q


# --------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.rows, self.proc, self.device_index = [], None, device_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


# --------------------------------------------------------------------- radix sort
def sort_leg(reps=6):
    """The onesweep radix sort alone (row a3: the build's Morton sort and each
    query batch's Morton ordering), through snch_sort_pairs on 16M random
    (key, value) uint32 pairs: 24-bit keys (the query-order width, 3 passes) and
    30-bit keys (the build's Morton codes, 4 passes); event-timed median. Bytes
    counted: the histogram pass reads the keys (4 B per pair), each digit pass
    reads and writes key and value (16 B per pair), and a sort with an odd pass
    count copies the pairs back (16 B per pair)."""
    import ctypes as C
    import torch
    import snch_lbvh_gb300 as snch
    L = snch.lib()
    n = 16_000_000
    peak, _ = hbm_peak()
    gen = torch.Generator(device="cuda").manual_seed(11)
    raw = torch.randint(0, 2**31 - 1, (n,), dtype=torch.int64, device="cuda", generator=gen)
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    kt, vt = torch.empty_like(vals), torch.empty_like(vals)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    res = {"pairs": n}
    for bits in (24, 30):
        keys = (raw & ((1 << bits) - 1)).to(torch.int32)
        scratch = torch.empty(L.snch_sort_scratch_bytes(n, bits), dtype=torch.uint8, device="cuda")
        ts = []
        for _ in range(reps + 2):
            kk, vv = keys.clone(), vals.clone()
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            snch.check(L.snch_sort_pairs(C.c_void_p(kk.data_ptr()), C.c_void_p(vv.data_ptr()),
                                         C.c_void_p(kt.data_ptr()), C.c_void_p(vt.data_ptr()), n, bits,
                                         C.c_void_p(scratch.data_ptr()), C.c_void_p(status.data_ptr()), None))
            z.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(z))
        ms = float(np.median(ts[2:]))
        passes = (bits + 7) // 8
        byts = n * (4 + 16 * passes + (16 if passes % 2 else 0))
        ok = bool((kk[1:].to(torch.int64) >= kk[:-1].to(torch.int64)).all()) and int(status.item()) == 0
        res[f"bits{bits}"] = {"ms": ms, "passes": passes, "GB/s": byts / ms / 1e6, "frac": byts / ms / 1e6 / peak,
                              "sorted": ok}
    return res


# --------------------------------------------------------------------- peaks
def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "of measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback"


def traffic_of(kernel, workload_key):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel and parts[1] == workload_key:
            return float(parts[2])
    return None


def issue_of(kernel):
    """Issue-bound figures of `kernel` from the committed ncu summary, if any:
    issue slots busy, active lanes per warp instruction, warp instructions per
    query, DRAM % of peak (profiles/issue.txt)."""
    path = os.path.join(ROOT, "profiles", "issue.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 6 and not line.startswith("#") and parts[0] == kernel:
            return {"issue_slots_busy": float(parts[1]), "lanes_per_inst": float(parts[2]),
                    "warp_inst_per_query": float(parts[3]), "dram_pct_of_peak": float(parts[4]),
                    "profile": parts[5]}
    return None


# --------------------------------------------------------------------- CPU restatement
def cpu_sample_counts(counts, frac):
    return {k: max(256, int(v * frac)) for k, v in counts.items()}


def run_cpu(sc, q, counts, frac, nthreads):
    """Times the CPU restatement on one bounded sample of the step: the
    single-threaded build of the whole scene + the first `frac` of each query
    batch on nthreads threads. value = sample queries / the wall time of that
    sample (build included, so the build weighs 1/frac times more than in the
    full step: a conservative figure). Also returns per-type q/s, the mean visit
    counts (for the algorithmic-bytes roofline) and the tree."""
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    tree = oracle.Tree(sc.verts, sc.faces)
    build_s = time.perf_counter() - t0
    sc_n = cpu_sample_counts(counts, frac)
    out, stats, secs = {}, {}, {}
    t0 = time.perf_counter()
    _, _, st = tree.nearest(q["near_pts"][:sc_n["near"]], stats=True, nthreads=nthreads)
    secs["near"] = time.perf_counter() - t0
    stats["near"] = st.mean(0)
    t0 = time.perf_counter()
    _, _, st = tree.silhouette(q["sil_pts"][:sc_n["sil"]], q["sil_flip"][:sc_n["sil"]], stats=True, nthreads=nthreads)
    secs["sil"] = time.perf_counter() - t0
    stats["sil"] = st.mean(0)
    t0 = time.perf_counter()
    *_, st = tree.ray(q["ray_o"][:sc_n["ray"]], q["ray_d"][:sc_n["ray"]], q["ray_tmax"][:sc_n["ray"]], stats=True,
                      nthreads=nthreads)
    secs["ray"] = time.perf_counter() - t0
    stats["ray"] = st.mean(0)
    t0 = time.perf_counter()
    *_, st = tree.sample(q["smp_c"][:sc_n["smp"]], q["smp_r"][:sc_n["smp"]], q["smp_u"][:sc_n["smp"]], stats=True,
                         nthreads=nthreads)
    secs["smp"] = time.perf_counter() - t0
    stats["smp"] = st.mean(0)
    out = {k: sc_n[k] / secs[k] for k in secs}
    wall_s = build_s + sum(secs.values())
    n_sample = sum(sc_n.values())
    return {"qps": out, "build_s": build_s, "wall_s": wall_s, "queries": n_sample, "value": n_sample / wall_s,
            "stats": stats, "sample": sc_n, "tree": tree}


def algorithmic_bytes(kind, st):
    b = BYTES_IO[kind] + BYTES_NODE[kind] * st[0] + BYTES_LEAF[kind] * st[1]
    if kind == "sil":
        b += BYTES_EDGE * st[2]
    return float(b)


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# --------------------------------------------------------------------- learned radius
LEARNED_TRAIN = {"uniform": 4_000_000, "surface": 4_000_000, "band": 0.05, "epochs": 6, "batch": 65536,
                 "lr": 2e-3, "tau": 0.9}
MLP_FLOP_PER_QUERY = 2 * (192 * 64 + 3 * 64 * 64) + 2 * 2 * 64  # tensor-core layers + head


def learned_leg(scene, sc, dev, counts, out, steps, scale):
    """Nearest and silhouette queries seeded by the learned radius vs plain, on the
    same batches: per-type q/s including the MLP inference, fallback fractions,
    and a bit-for-bit comparison with the plain results. Training runs first and
    is reported separately (a model is trained once per scene)."""
    import torch
    from snch_lbvh_gb300.learned import LearnedRadius, targets_from_scene, training_points
    cfg = dict(LEARNED_TRAIN)
    nu, ns = max(4096, int(cfg["uniform"] * scale)), max(4096, int(cfg["surface"] * scale))
    pts = torch.from_numpy(training_points(sc.verts, sc.faces, nu, ns, cfg["band"], seed=77)).cuda()
    tgt = targets_from_scene(scene, pts)
    model = LearnedRadius(np.zeros(3), np.ones(3), seed=3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = model.train(pts, tgt, epochs=cfg["epochs"], batch=cfg["batch"], lr=cfg["lr"], tau=cfg["tau"])
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    nn, ns_ = counts["near"], counts["sil"]
    rn = torch.empty(nn, device="cuda")
    rs = torch.empty(ns_, device="cuda")
    o_near = (torch.empty(nn, dtype=torch.int32, device="cuda"), torch.empty(nn, device="cuda"))
    o_sil = (torch.empty(ns_, device="cuda"), torch.empty(ns_, dtype=torch.int32, device="cuda"))
    nf = torch.zeros(2, dtype=torch.int32, device="cuda")
    res = {"training": {**cfg, "uniform": nu, "surface": ns, "final_loss": loss, "train_s": train_s},
           "margins": {}}
    best = None
    for margin in (1.1, 1.25, 1.5):
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(steps + 1)]
        for k in range(steps + 1):  # the first round is a warm-up
            e = ev[k]
            e[0].record(stream)
            model.predict(dev["near_pts"], margin=margin, floor=1e-4, out=(rn, None), which="near")
            e[1].record(stream)
            scene.query_nearest_seeded(dev["near_pts"], rn, out=o_near, num_fallback=nf[0:1])
            e[2].record(stream)
            model.predict(dev["sil_pts"], margin=margin, floor=1e-4, out=(None, rs), which="sil")
            e[3].record(stream)
            scene.query_silhouette_seeded(dev["sil_pts"], rs, dev["sil_flip"], out=o_sil, num_fallback=nf[1:2])
            e[4].record(stream)
        torch.cuda.synchronize()
        ms = np.array([[e[i].elapsed_time(e[i + 1]) for i in range(4)] for e in ev[1:]]).mean(0)
        same = (torch.equal(o_near[0], out["near"][0]) and torch.equal(o_near[1].view(torch.int32),
                                                                          out["near"][1].view(torch.int32))
                and torch.equal(o_sil[0].view(torch.int32), out["sil"][0].view(torch.int32))
                and torch.equal(o_sil[1], out["sil"][1]))
        fb = nf.cpu().numpy()
        r = {"near_qps": nn / ((ms[0] + ms[1]) / 1e3), "sil_qps": ns_ / ((ms[2] + ms[3]) / 1e3),
             "mlp_ms": {"near": float(ms[0]), "sil": float(ms[2])},
             "seeded_ms": {"near": float(ms[1]), "sil": float(ms[3])},
             "fallback_frac": {"near": float(fb[0]) / nn, "sil": float(fb[1]) / ns_},
             "identical_to_plain": bool(same),
             "mlp_tflops": MLP_FLOP_PER_QUERY * nn / (ms[0] / 1e3) / 1e12}
        res["margins"][str(margin)] = r
        if best is None or r["near_qps"] + r["sil_qps"] > best[1]["near_qps"] + best[1]["sil_qps"]:
            best = (margin, r)
    res["best_margin"] = best[0]
    res["near_qps"], res["sil_qps"] = best[1]["near_qps"], best[1]["sil_qps"]
    res["ceiling"] = radius_ceiling(scene, dev, counts, out, steps)
    res["identical_to_plain"] = all(r["identical_to_plain"] for r in res["margins"].values())
    res["reference_order"] = learned_on_reference_order(scene, model, dev, best[0], best[1]["mlp_ms"], counts)
    model.close()
    return res


def radius_ceiling(scene, dev, counts, out, steps):
    """What radius seeding can buy at most on the default traversal: every query
    seeded with its own answer (the next float above the plain distance, so that
    no query falls back), no MLP time, against the plain search on the same
    batch. No predictor can prune more than the exact distance does."""
    import torch
    stream = torch.cuda.current_stream()
    rn = torch.from_numpy(np.nextafter(out["near"][1].cpu().numpy(), np.float32(np.inf))).cuda()
    rs = torch.from_numpy(np.nextafter(out["sil"][0].cpu().numpy(), np.float32(np.inf))).cuda()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(steps + 1)]
    for k in range(steps + 1):  # the first round is a warm-up
        e = ev[k]
        e[0].record(stream)
        scene.query_nearest(dev["near_pts"])
        e[1].record(stream)
        scene.query_nearest_seeded(dev["near_pts"], rn)
        e[2].record(stream)
        scene.query_silhouette(dev["sil_pts"], dev["sil_flip"])
        e[3].record(stream)
        scene.query_silhouette_seeded(dev["sil_pts"], rs, dev["sil_flip"])
        e[4].record(stream)
    torch.cuda.synchronize()
    ms = np.array([[e[i].elapsed_time(e[i + 1]) for i in range(4)] for e in ev[1:]]).mean(0)
    return {"what": "seeded with each query's own distance (next float up), no MLP: the upper bound of any "
                    "radius predictor on this traversal",
            "plain_ms": {"near": float(ms[0]), "sil": float(ms[2])},
            "exact_seeded_ms": {"near": float(ms[1]), "sil": float(ms[3])},
            "speedup": {"near": float(ms[0] / ms[1]), "sil": float(ms[2] / ms[3])}}


def learned_on_reference_order(scene, model, dev, margin, mlp_ms, counts, sub=2_000_000):
    """The same learned radius applied to the reference's own traversal order
    (TRAVERSAL_REFERENCE_ORDER): plain vs seeded on the first `sub` queries of
    each batch, one timed run each; the MLP time is the full batch's, scaled."""
    import torch
    import snch_lbvh_gb300 as snch
    stream = torch.cuda.current_stream()
    out = {"queries": {}}
    scene.set_traversal(snch.TRAVERSAL_REFERENCE_ORDER)
    try:
        for kind, key in (("near", "near_pts"), ("sil", "sil_pts")):
            m = min(counts[kind], sub)
            pts = dev[key][:m]
            rn, rs = model.predict(pts, margin=margin, floor=1e-4, which=kind)
            r = rn if kind == "near" else rs
            nf = torch.zeros(1, dtype=torch.int32, device="cuda")
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            if kind == "near":
                e[0].record(stream)
                a = scene.query_nearest(pts)
                e[1].record(stream)
                b = scene.query_nearest_seeded(pts, r, num_fallback=nf)
                e[2].record(stream)
            else:
                flip = dev["sil_flip"][:m]
                e[0].record(stream)
                a = scene.query_silhouette(pts, flip)
                e[1].record(stream)
                b = scene.query_silhouette_seeded(pts, r, flip, num_fallback=nf)
                e[2].record(stream)
            torch.cuda.synchronize()
            same = all(torch.equal(x.view(torch.int32), y.view(torch.int32)) for x, y in zip(a, b))
            plain_ms, seeded_ms = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
            mlp = mlp_ms[kind] * m / counts[kind]
            out["queries"][kind] = m
            out[f"{kind}_plain_qps"] = m / (plain_ms / 1e3)
            out[f"{kind}_learned_qps"] = m / ((seeded_ms + mlp) / 1e3)
            out[f"{kind}_speedup"] = plain_ms / (seeded_ms + mlp)
            out[f"{kind}_fallback_frac"] = float(nf.item()) / m
            out[f"{kind}_identical"] = bool(same)
    finally:
        scene.set_traversal(snch.TRAVERSAL_NEAR_FIRST)
    return out


# --------------------------------------------------------------------- icosphere (configs 1 and 4)
def time_events(fn, reps, stream):
    """Mean milliseconds of fn() over reps runs after one warm-up, CUDA events."""
    import torch
    fn()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(reps):
        fn()
    e[1].record(stream)
    torch.cuda.synchronize()
    return e[0].elapsed_time(e[1]) / reps


def l2_copy_gbs(stream, mb=24, reps=50):
    """Copy bandwidth of a buffer pair that stays in L2 (read + write bytes / time)."""
    import torch
    a = torch.empty(mb << 20, dtype=torch.uint8, device="cuda")
    b = torch.empty_like(a)
    ms = time_events(lambda: b.copy_(a), reps, stream)
    return 2 * a.numel() / (ms / 1e3) / 1e9


def icosphere_leg(scale, n_plain=1_000_000, n_eval=16_000_000, reps=5):
    """The 20,480-triangle noisy icosphere (level 5, radius 1, sigma 0.01): 1M
    nearest queries uniform in its box x 1.2, both traversal orders (config 1;
    the tree is L2-resident, so the algorithmic bytes are set against an L2 copy
    bandwidth measured here), and the learned radius trained on 8M (point, exact
    distance) pairs from the plain queries -- half uniform in the box, half within
    0.05 of the surface -- evaluated on 16M fresh points: learned vs plain, both
    traversal orders, identical results (config 4)."""
    import torch
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    from snch_lbvh_gb300.learned import LearnedRadius, targets_from_scene, training_points
    stream = torch.cuda.current_stream()
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    s = snch.Scene(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda())
    s.compute_silhouettes()
    s.build_bvh()
    n1 = max(1024, int(n_plain * scale))
    p1 = torch.from_numpy(meshes.box_queries(v, n1, 1.2, seed=1)).cuda()
    res = {"workload": f"{len(f):,}-triangle noisy icosphere; {n1:,} nearest queries uniform in its box x 1.2"}
    plain = {}
    for name, mode in (("near_first", snch.TRAVERSAL_NEAR_FIRST), ("reference_order", snch.TRAVERSAL_REFERENCE_ORDER)):
        s.set_traversal(mode)
        ms = time_events(lambda: s.query_nearest(p1), reps, stream)
        vis = s.query_visits("nearest", p1[: min(n1, 1_000_000)]).astype(np.float64).mean(0)
        alg = 20 + 56 * vis[0] + 48 * vis[1]  # in/out + per expanded node + per leaf triangle
        plain[name] = {"qps": n1 / (ms / 1e3), "ms": ms, "visits_per_query": vis[:2].tolist(),
                       "algorithmic_bytes_per_query": float(alg), "achieved_GBs": n1 * alg / (ms / 1e3) / 1e9}
    s.set_traversal(snch.TRAVERSAL_NEAR_FIRST)
    l2 = l2_copy_gbs(stream)
    for r in plain.values():
        r["l2_frac"] = r["achieved_GBs"] / l2
    res["nearest"] = plain
    res["l2_copy_GBs"] = l2

    # learned radius (config 4)
    cfg = dict(LEARNED_TRAIN)
    lo, hi = v.min(0), v.max(0)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.2
    nu, ns = max(4096, int(cfg["uniform"] * scale)), max(4096, int(cfg["surface"] * scale))
    tp = torch.from_numpy(training_points(v, f, nu, ns, cfg["band"], lo=c - h, hi=c + h, seed=78)).cuda()
    tgt = targets_from_scene(s, tp)
    model = LearnedRadius(c - h, c + h, seed=4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = model.train(tp, tgt, epochs=cfg["epochs"], batch=cfg["batch"], lr=cfg["lr"], tau=cfg["tau"])
    torch.cuda.synchronize()
    res["training"] = {**cfg, "uniform": nu, "surface": ns, "final_loss": loss,
                       "train_s": time.perf_counter() - t0}
    del tp, tgt
    ne = max(1024, int(n_eval * scale))
    pe = torch.from_numpy(meshes.box_queries(v, ne, 1.2, seed=2)).cuda()
    fe = (torch.arange(ne, device="cuda") % 2).to(torch.uint8)
    learned = {}
    for name, mode in (("near_first", snch.TRAVERSAL_NEAR_FIRST), ("reference_order", snch.TRAVERSAL_REFERENCE_ORDER)):
        s.set_traversal(mode)
        pn, ps = s.query_nearest(pe), s.query_silhouette(pe, fe)
        plain_ms = [time_events(lambda: s.query_nearest(pe), reps, stream),
                    time_events(lambda: s.query_silhouette(pe, fe), reps, stream)]
        best = None
        for margin in (1.1, 1.25, 1.5):
            rn, rs = model.predict(pe, margin=margin, floor=1e-4)
            nf = torch.zeros(2, dtype=torch.int32, device="cuda")
            sn = s.query_nearest_seeded(pe, rn, num_fallback=nf[0:1])
            ss = s.query_silhouette_seeded(pe, rs, fe, num_fallback=nf[1:2])
            same = (torch.equal(sn[0], pn[0]) and torch.equal(sn[1].view(torch.int32), pn[1].view(torch.int32))
                    and torch.equal(ss[0].view(torch.int32), ps[0].view(torch.int32)) and torch.equal(ss[1], ps[1]))
            mlp_ms = time_events(lambda: model.predict(pe, margin=margin, floor=1e-4, out=(rn, rs)), reps, stream)
            seeded_ms = [time_events(lambda: s.query_nearest_seeded(pe, rn), reps, stream),
                         time_events(lambda: s.query_silhouette_seeded(pe, rs, fe), reps, stream)]
            fb = nf.cpu().numpy() / ne
            # the model predicts both radii in one pass: half its time is charged to each type
            r = {"margin": margin, "near_qps": ne / ((seeded_ms[0] + mlp_ms / 2) / 1e3),
                 "sil_qps": ne / ((seeded_ms[1] + mlp_ms / 2) / 1e3), "mlp_ms_both": mlp_ms,
                 "fallback_frac": {"near": float(fb[0]), "sil": float(fb[1])}, "identical_to_plain": bool(same)}
            if best is None or r["near_qps"] + r["sil_qps"] > best["near_qps"] + best["sil_qps"]:
                best = r
        best["plain_qps"] = {"near": ne / (plain_ms[0] / 1e3), "sil": ne / (plain_ms[1] / 1e3)}
        best["speedup"] = {"near": best["near_qps"] / best["plain_qps"]["near"],
                           "sil": best["sil_qps"] / best["plain_qps"]["sil"]}
        learned[name] = best
    s.set_traversal(snch.TRAVERSAL_NEAR_FIRST)
    res["learned"] = {"eval_points": ne, **learned}
    res["device_status"] = int(s.device_status())
    model.close()
    s.close()
    return res


# --------------------------------------------------------------------- batched meshes
def batched_leg(scale, per_tri=8):
    """256 independent meshes (log-uniform 1k..500k triangles): one batched scene
    (one topology pass, one build, one launch per query type) vs one scene per
    mesh (a build and two query launches per mesh), same queries: per_tri x
    triangles nearest and silhouette points per mesh, uniform in the mesh's box
    scaled by 1.2. Device time with CUDA events; results compared bit for bit."""
    import torch
    import snch_lbvh_gb300 as snch
    from snch_lbvh_gb300 import meshes
    ms = meshes.batched_meshes(seed=5)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    counts = [max(1, int(per_tri * len(f) * scale)) for _, f in ms]
    dev = [(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda()) for v, f in ms]
    pts, mid = [], []
    for m, (v, _) in enumerate(dev):
        lo, hi = v.min(0).values, v.max(0).values
        c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.2
        pts.append(c + h * (2 * torch.rand((counts[m], 3), device="cuda", generator=gen) - 1))
        mid.append(torch.full((counts[m],), m, dtype=torch.int32, device="cuda"))
    P, M = torch.cat(pts), torch.cat(mid)
    n = len(P)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    b = snch.BatchedScene(dev)
    torch.cuda.synchronize()
    ev[0].record(stream)
    b.compute_silhouettes()
    b.build_bvh()
    ev[1].record(stream)
    bi, bd = b.query_nearest_batch(M, P)
    ev[2].record(stream)
    bs, be = b.query_silhouette_batch(M, P)
    ev[3].record(stream)
    torch.cuda.synchronize()
    batched = [ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2]), ev[2].elapsed_time(ev[3])]
    # one scene per mesh, on the first 1/128 of each mesh's queries (1/16 of its
    # triangle count; the per-mesh silhouette launches of the full set take minutes),
    # against the batched launches on the same subset
    sub = [p_[: max(1, len(p_) // 128)] for p_ in pts]
    Ps, Ms = torch.cat(sub), torch.cat([m_[: len(p_)] for m_, p_ in zip(mid, sub)])
    ns = len(Ps)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    e[0].record(stream)
    si, sd = b.query_nearest_batch(Ms, Ps)
    e[1].record(stream)
    ss, se = b.query_silhouette_batch(Ms, Ps)
    e[2].record(stream)
    scenes = [snch.Scene(v, f) for v, f in dev]
    torch.cuda.synchronize()
    e[3].record(stream)
    for s_ in scenes:
        s_.compute_silhouettes()
        s_.build_bvh()
    e[4].record(stream)
    outs = [s_.query_nearest(p_) for s_, p_ in zip(scenes, sub)]
    e5 = torch.cuda.Event(enable_timing=True)
    e5.record(stream)
    outs2 = [s_.query_silhouette(p_) for s_, p_ in zip(scenes, sub)]
    e[5].record(stream)
    torch.cuda.synchronize()
    single = [e[3].elapsed_time(e[4]), e[4].elapsed_time(e5), e5.elapsed_time(e[5])]
    bsub = [e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])]
    same = (torch.equal(si, torch.cat([o[0] for o in outs]).view(torch.int32))
            and torch.equal(sd.view(torch.int32), torch.cat([o[1] for o in outs]).view(torch.int32))
            and torch.equal(ss.view(torch.int32), torch.cat([o[0] for o in outs2]).view(torch.int32))
            and torch.equal(se, torch.cat([o[1] for o in outs2])))
    for s_ in scenes:
        s_.close()
    # autotuned (node width, threads per block, packets, persistent) on every query of
    # every 32nd mesh: the sample keeps the batch's query density, which decides
    # whether warp packets pay (a thin slice of every mesh's queries would not)
    tsel = range(0, len(pts), 32)
    Pt, Mt = torch.cat([pts[m_] for m_ in tsel]), torch.cat([mid[m_] for m_ in tsel])
    tuned = b.autotune(Pt, Pt, None, near_mesh=Mt, sil_mesh=Mt)

    def cfg_name(w, bk, pk, pers):
        return f"w{w}_b{bk}_" + ("packet" if pk else "persistent" if pers else "lane")

    chosen = {"near": cfg_name(*b.search_config("nearest")), "sil": cfg_name(*b.search_config("silhouette"))}
    # the full batches again in the chosen configurations
    te = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    te[0].record()
    b.query_nearest_batch(M, P)
    te[1].record()
    b.query_silhouette_batch(M, P)
    te[2].record()
    torch.cuda.synchronize()
    tuned_ms = [te[0].elapsed_time(te[1]), te[1].elapsed_time(te[2])]
    # the whole step (topology + build of all meshes + both query batches) as one
    # captured CUDA graph, launched once to warm up and once timed
    gst = torch.cuda.Stream()
    go = ((torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda")),
          (torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda")))
    torch.cuda.synchronize()
    g = b.capture(True, P, go[0], P, None, go[1], near_mesh=M, sil_mesh=M, stream=gst)
    g.launch(gst)
    ge = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ge[0].record(gst)
    g.launch(gst)
    ge[1].record(gst)
    gst.synchronize()
    graph_ms = ge[0].elapsed_time(ge[1])
    graph_same = (torch.equal(go[0][0], bi) and torch.equal(go[0][1].view(torch.int32), bd.view(torch.int32))
                  and torch.equal(go[1][0].view(torch.int32), bs.view(torch.int32)) and torch.equal(go[1][1], be))
    g.close()
    status = b.device_status()
    b.close()
    return {"workload": f"{len(ms)} meshes, {sum(len(f) for _, f in ms):,} triangles, {n:,} nearest + {n:,} "
                        f"silhouette queries ({per_tri * scale:g} x triangles per mesh, uniform in the mesh's box "
                        f"x 1.2)",
            "batched_ms": {"build": batched[0], "near": batched[1], "sil": batched[2]},
            "batched_qps": {"near": n / (batched[1] / 1e3), "sil": n / (batched[2] / 1e3)},
            "subset": f"{ns:,} queries per type (the first 1/128 of each mesh's)",
            "per_mesh_ms": {"build": single[0], "near": single[1], "sil": single[2]},
            "per_mesh_qps": {"near": ns / (single[1] / 1e3), "sil": ns / (single[2] / 1e3)},
            "batched_subset_qps": {"near": ns / (bsub[0] / 1e3), "sil": ns / (bsub[1] / 1e3)},
            "build_speedup": single[0] / batched[0],
            "identical_to_per_mesh": bool(same),
            "autotune_ms": {"sample": f"{len(Pt):,} queries per type (all queries of every 32nd mesh)",
                            "near": {cfg_name(*c): t for c, t in tuned["nearest"].items()},
                            "sil": {cfg_name(*c): t for c, t in tuned["silhouette"].items()},
                            "chosen": chosen},
            "tuned_qps": {"near": n / (tuned_ms[0] / 1e3), "sil": n / (tuned_ms[1] / 1e3)},
            "graph": {"step_ms": graph_ms, "qps": 2 * n / (graph_ms / 1e3),
                      "what": "one CUDA-graph launch: topology + build of all meshes + both query batches",
                      "identical": bool(graph_same)},
            "device_status": int(status)}


# --------------------------------------------------------------------- walk-on-stars
def wost_leg(scale, walkers=1_000_000, max_steps=128):
    """Wavefront walk-on-stars on the 20,480-triangle noisy icosphere with 50/50
    Dirichlet/Neumann faces: 1M walkers from the ball of radius 0.95, up to 128
    steps, one nearest + silhouette + ray + sphere-sample query per live walker
    and step; plain vs learned radius (trained on the walk's own distances).
    Per-step queries/s; estimates compared bit for bit."""
    import torch
    from snch_lbvh_gb300 import meshes, wost
    from snch_lbvh_gb300.learned import LearnedRadius, training_points
    v, f = meshes.noisy_icosphere(5, 1.0, 0.01, seed=0)
    flags = (np.random.default_rng(1).random(len(f)) < 0.5).astype(np.uint8)
    d, nsc = wost.split_boundary(v, f, flags)
    n = max(1024, int(walkers * scale))
    pts = torch.from_numpy(training_points(v, f, max(4096, int(4_000_000 * scale)), max(4096, int(4_000_000 * scale)),
                                           0.05, lo=(-1.2, -1.2, -1.2), hi=(1.2, 1.2, 1.2), seed=9)).cuda()
    _, dd = d.query_nearest(pts)
    ds, _ = nsc.query_silhouette(pts)
    t = torch.stack([dd, ds], 1)
    t = torch.log(torch.where(torch.isfinite(t) & (t > 0), t, torch.full_like(t, float("nan"))))
    model = LearnedRadius(np.full(3, -1.2), np.full(3, 1.2), seed=4)
    t0 = time.perf_counter()
    model.train(pts, t, epochs=6, batch=65536, lr=2e-3, tau=0.9)
    train_s = time.perf_counter() - t0
    wost.trace(d, nsc, min(n, 65536), max_steps=4, seed=1)  # warm-up
    e0, x0, s0 = wost.trace(d, nsc, n, max_steps=max_steps, seed=3)
    e1, _, s1 = wost.trace(d, nsc, n, max_steps=max_steps, seed=3, model=model, margin=1.5)
    err = (e0 - x0[:, 0]).double()
    q0, q1 = sum(s0["queries"]), sum(s1["queries"])
    res = {"workload": f"{n:,} walkers, <= {max_steps} steps, 20,480-triangle icosphere, 50/50 Dirichlet/Neumann faces",
           "steps": s0["steps"], "terminated_frac": s0["terminated"] / n, "queries": q0,
           "plain": {"query_qps": q0 / (sum(s0["query_ms"]) / 1e3), "step_qps": q0 / (sum(s0["step_ms"]) / 1e3)},
           "learned": {"query_qps": q1 / (sum(s1["query_ms"]) / 1e3), "step_qps": q1 / (sum(s1["step_ms"]) / 1e3),
                       "fallback_frac": sum(s1["fallback"]) / max(1, 2 * sum(s1["live"])), "train_s": train_s},
           "identical_estimates": bool(torch.equal(e0.view(torch.int32), e1.view(torch.int32))),
           "estimate_error": {"mean": float(err.mean()), "std": float(err.std())},
           "per_step_live": s0["live"][:8] + ["..."] + s0["live"][-3:],
           "per_step_qps_plain": [round(q / (m / 1e3)) for q, m in zip(s0["queries"][:8], s0["step_ms"][:8])]}
    model.close()
    return res


# --------------------------------------------------------------------- reference arm
def run_reference(args):
    """The reference's own implementation of the step on this machine: the CPU
    restatement of its build and queries (its documented CPU query path is
    broken, README.md:39) on all host cores, each step one bounded sample of the
    workload, timed as it runs; plus the reference's own CUDA queries (its
    headers compiled for sm_103a) over a tree the restatement built."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sc, counts, q = make_workload(args.scale, seed=1)
    nthreads = cpu_threads()
    frac, warm_frac = 0.01, 0.001
    rows = []
    for i in range(args.warmup + args.steps):
        r = run_cpu(sc, q, counts, frac if i >= args.warmup else warm_frac, nthreads)
        if i >= args.warmup:
            rows.append(r)
    wall = sum(r["wall_s"] for r in rows)
    value = sum(r["queries"] for r in rows) / wall
    smp = rows[-1]["sample"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / len(rows), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded meshes and queries)",
        "config": bench_config(counts, len(sc.faces), ws),
        "per_type_qps": {k: float(np.mean([r["qps"][k] for r in rows])) for k in counts},
        "build_s": float(np.mean([r["build_s"] for r in rows])),
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": nthreads, "kind": "port",
                         "sample": f"per step: single-thread build of the whole {len(sc.faces):,}-triangle scene + "
                                   f"the first {smp['near']:,} nearest, {smp['sil']:,} silhouette, {smp['ray']:,} "
                                   f"ray and {smp['smp']:,} sample queries ({frac:.0%} of each batch) on {nthreads} "
                                   f"threads; value = those queries / the step's wall time"},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line["reference_cuda"] = reference_cuda_leg(rows[-1]["tree"], q, counts)
    print(json.dumps(line), flush=True)


def reference_cuda_leg(tree, q, counts, sample=2_000_000):
    """The reference's own query_device kernels (its headers compiled for sm_103a
    with its flags, oracle/ref_gpu_kernels.cu), timed on this GPU over a tree the
    CPU restatement built (oracle/ref_gpu.py RefTree: the reference's device
    layout, no code of this library); queries only, a bounded sample of each
    batch. The reference's build runs Thrust from host code compiled with its
    headers, which this GPU machine cannot compile (they are not on it)."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA device"}
        from oracle import ref_gpu
        ok, why = ref_gpu.available()
        if not ok:
            return {"unavailable": why}
        R = ref_gpu.RefQueries(ref_gpu.RefTree(tree))
        m = {k: min(sample, counts[k]) for k in counts}
        kind = {"near_pts": "near", "sil_pts": "sil", "sil_flip": "sil", "ray_o": "ray", "ray_d": "ray",
                "ray_tmax": "ray", "smp_c": "smp", "smp_r": "smp", "smp_u": "smp"}
        d = {k: torch.from_numpy(np.ascontiguousarray(v[:m[kind[k]]])).cuda() for k, v in q.items()}
        calls = {"near": lambda: R.nearest(d["near_pts"]), "sil": lambda: R.silhouette(d["sil_pts"], d["sil_flip"]),
                 "ray": lambda: R.ray(d["ray_o"], d["ray_d"], d["ray_tmax"]),
                 "smp": lambda: R.sample(d["smp_c"], d["smp_r"], d["smp_u"])}
        qps = {}
        for k, f in calls.items():
            f()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            f()
            e1.record()
            torch.cuda.synchronize()
            qps[k] = m[k] / (e0.elapsed_time(e1) / 1e3)
        t = sum(counts[k] / qps[k] for k in counts)
        return {"value": sum(counts.values()) / t, "unit": "queries/s", "per_type_qps": qps,
                "tree": "built by the CPU restatement (oracle), reference device layout",
                "sample": f"{m['near']:,} nearest, {m['sil']:,} silhouette, {m['ray']:,} ray, {m['smp']:,} sample "
                          f"queries (input order), each extrapolated to its batch; queries only"}
    except Exception as exc:  # reported, never fatal for the CPU arm
        return {"unavailable": f"{type(exc).__name__}: {exc}"}


# --------------------------------------------------------------------- our arm
def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import snch_lbvh_gb300 as snch
    L = snch.lib()

    sc, counts, q = make_workload(args.scale, seed=1 + rank)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in q.items()}
    n = counts
    out = {
        "near": (torch.empty(n["near"], dtype=torch.int32, device="cuda"),
                 torch.empty(n["near"], dtype=torch.float32, device="cuda")),
        "sil": (torch.empty(n["sil"], dtype=torch.float32, device="cuda"),
                torch.empty(n["sil"], dtype=torch.int32, device="cuda")),
        "ray": (torch.empty(n["ray"], dtype=torch.uint8, device="cuda"),
                torch.empty(n["ray"], dtype=torch.float32, device="cuda"),
                torch.empty((n["ray"], 2), dtype=torch.float32, device="cuda"),
                torch.empty(n["ray"], dtype=torch.int32, device="cuda")),
        "smp": (torch.empty(n["smp"], dtype=torch.int32, device="cuda"),
                torch.empty(n["smp"], dtype=torch.float32, device="cuda")),
    }
    verts_d = torch.from_numpy(sc.verts).cuda()
    faces_d = torch.from_numpy(sc.faces).cuda()
    scene = snch.Scene(verts_d, faces_d)
    if args.persistent_min > 0:
        scene.set_option(snch.OPT_PACKET_PERSISTENT_MIN, args.persistent_min)
    if args.output_scatter >= 0:
        scene.set_option(snch.OPT_OUTPUT_SCATTER, args.output_scatter)
    if args.top_levels >= 0:
        scene.set_option(snch.OPT_TOP_LEVELS, args.top_levels)
    if args.ray_order >= 0:
        scene.set_option(snch.OPT_RAY_ORDER, args.ray_order)
    if args.order_bits > 0:
        scene.set_option(snch.OPT_ORDER_BITS, args.order_bits)
    stream = torch.cuda.current_stream()

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        scene.compute_silhouettes()
        scene.build_bvh()
        if ev:
            ev[1].record(stream)
        scene.query_nearest(dev["near_pts"], out=out["near"])
        if ev:
            ev[2].record(stream)
        scene.query_silhouette(dev["sil_pts"], dev["sil_flip"], out=out["sil"])
        if ev:
            ev[3].record(stream)
        scene.query_ray(dev["ray_o"], dev["ray_d"], dev["ray_tmax"], out=out["ray"])
        if ev:
            ev[4].record(stream)
        scene.sample_in_sphere(dev["smp_c"], dev["smp_r"], dev["smp_u"], out=out["smp"])
        if ev:
            ev[5].record(stream)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 0)):
        step()
    barrier()
    status = scene.device_status()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(args.steps)]
    clocks = ClockSampler(torch.cuda.current_device() if "CUDA_VISIBLE_DEVICES" not in os.environ
                          else os.environ["CUDA_VISIBLE_DEVICES"].split(",")[local])
    clocks.start()
    time.sleep(0.3)
    launches0 = L.snch_kernel_launch_count()
    barrier()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t_end.record(stream)
    barrier()
    launches = L.snch_kernel_launch_count() - launches0
    clk = clocks.stop()
    # answers of the last timed step; the e2e leg's host-buffer answers must equal them
    device_answers = {"near_dist": out["near"][1].cpu().numpy(), "sil_dist": out["sil"][0].cpu().numpy(),
                      "ray_hit": out["ray"][0].cpu().numpy(), "ray_t": out["ray"][1].cpu().numpy(),
                      "smp_idx": out["smp"][0].cpu().numpy(), "smp_pdf": out["smp"][1].cpu().numpy()}
    status |= scene.device_status()
    elapsed_ms = t_start.elapsed_time(t_end)
    elapsed_ms = max_over_ranks(elapsed_ms, "cuda")
    phase_ms = np.array([[e[i].elapsed_time(e[i + 1]) for i in range(5)] for e in evs]).mean(0)
    total_q = sum(counts.values())
    value = total_q * ws * args.steps / (elapsed_ms / 1e3)
    per_type = {k: counts[k] / (phase_ms[i + 1] / 1e3) for i, k in enumerate(["near", "sil", "ray", "smp"])}

    # ---- work counters of the timed kernels on the full batches (outside the timed
    # region; the batch size decides whether nearest searches run as warp packets)
    m = dict(counts)
    visits = {
        "near": scene.query_visits("nearest", dev["near_pts"][:m["near"]]).mean(0),
        "sil": scene.query_visits("silhouette", dev["sil_pts"][:m["sil"]], flip=dev["sil_flip"][:m["sil"]]).mean(0),
        "ray": scene.query_visits("ray", dev["ray_o"][:m["ray"]], dev["ray_d"][:m["ray"]],
                                  dev["ray_tmax"][:m["ray"]]).mean(0),
        "smp": scene.query_visits("sample", dev["smp_c"][:m["smp"]], dev["smp_r"][:m["smp"]],
                                  dev["smp_u"][:m["smp"]]).mean(0),
    }

    # ---- stack depth: a search pushes at most one entry per level it descends, so
    # the tree's depth bounds every stack (64 entries binary); no tuning needed
    nodes = scene.export_tree()["nodes"].astype(np.int64)
    depth = np.zeros(len(nodes), np.int64)
    frontier = np.array([0])
    ni = (len(nodes) + 1) // 2 - 1
    while len(frontier):
        inner = frontier[frontier < ni]
        kids = np.concatenate([nodes[inner, 1], nodes[inner, 2]])
        depth[kids] = np.concatenate([depth[inner], depth[inner]]) + 1
        frontier = kids
    stack = {"tree_depth": int(depth.max()), "stack_entries": 64,
             "overflowed": bool(status & 1), "note": "a search's stack holds at most one entry per level below "
             "its current node, so the tree depth bounds it; the autotuner has no stack dimension"}

    # ---- the occlusion form of the ray query (ray_intersect<TestOnly = true>) on the
    # same rays, outside the timed step; its hit flags equal the timed step's
    ray_test_ms = time_events(lambda: scene.query_ray_test(dev["ray_o"], dev["ray_d"], dev["ray_tmax"]), 3, stream)
    ray_test = {"qps": counts["ray"] / (ray_test_ms / 1e3), "ms": ray_test_ms,
                "same_hits": bool(torch.equal(scene.query_ray_test(dev["ray_o"], dev["ray_d"], dev["ray_tmax"]),
                                              out["ray"][0]))}

    # ---- learned radius vs plain on the same batches (outside the timed step)
    learned = None
    if not args.no_learned:
        learned = learned_leg(scene, sc, dev, counts, out, max(1, min(args.steps, 3)), args.scale)
        learned["plain_qps"] = {"near": float(per_type["near"]), "sil": float(per_type["sil"])}
        learned["speedup"] = {"near": learned["near_qps"] / per_type["near"],
                              "sil": learned["sil_qps"] / per_type["sil"]}
        learned["status"] = int(scene.device_status())

    # ---- icosphere, batched meshes and walk-on-stars (single GPU only; outside the timed step)
    batched = wost_res = ico = sort_res = None
    if ws == 1 and not args.no_sort:
        sort_res = sort_leg()
    if ws == 1 and not args.no_icosphere:
        ico = icosphere_leg(args.scale)
    if ws == 1 and not args.no_batched:
        batched = batched_leg(args.scale)
    if ws == 1 and not args.no_wost:
        wost_res = wost_leg(args.scale)

    # ---- e2e through the host-buffer C ABI
    e2e = None
    if not args.no_e2e:
        pin = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy() for k, v in q.items()}
        pin_v = torch.from_numpy(sc.verts).pin_memory().numpy()
        pin_f = torch.from_numpy(sc.faces).pin_memory().numpy()
        hout = {
            "near": (torch.empty(n["near"], dtype=torch.int32).pin_memory().numpy().view(np.uint32),
                     torch.empty(n["near"], dtype=torch.float32).pin_memory().numpy()),
            "sil": (torch.empty(n["sil"], dtype=torch.float32).pin_memory().numpy(),
                    torch.empty(n["sil"], dtype=torch.int32).pin_memory().numpy()),
            "ray": (torch.empty(n["ray"], dtype=torch.uint8).pin_memory().numpy(),
                    torch.empty(n["ray"], dtype=torch.float32).pin_memory().numpy(),
                    torch.empty((n["ray"], 2), dtype=torch.float32).pin_memory().numpy(),
                    torch.empty(n["ray"], dtype=torch.int32).pin_memory().numpy().view(np.uint32)),
            "smp": (torch.empty(n["smp"], dtype=torch.int32).pin_memory().numpy(),
                    torch.empty(n["smp"], dtype=torch.float32).pin_memory().numpy()),
        }

        e2e_parts = []

        def e2e_step():
            t = [time.perf_counter()]
            s = snch.Scene(pin_v, pin_f)
            if args.host_chunk > 0:
                s.set_option(snch.OPT_HOST_CHUNK, args.host_chunk)
            s.compute_silhouettes()
            s.build_bvh()
            t.append(time.perf_counter())
            s.query_nearest_host(pin["near_pts"], out=hout["near"])
            t.append(time.perf_counter())
            s.query_silhouette_host(pin["sil_pts"], pin["sil_flip"], out=hout["sil"])
            t.append(time.perf_counter())
            s.query_ray_host(pin["ray_o"], pin["ray_d"], pin["ray_tmax"], out=hout["ray"])
            t.append(time.perf_counter())
            s.sample_in_sphere_host(pin["smp_c"], pin["smp_r"], pin["smp_u"], out=hout["smp"])
            t.append(time.perf_counter())
            s.close()
            t.append(time.perf_counter())
            e2e_parts.append([1e3 * (b_ - a_) for a_, b_ in zip(t, t[1:])])

        # what the host link delivers on this machine (other tenants share it): one pinned
        # 192 MB input array each way, event-timed
        probe = torch.empty(pin["near_pts"].shape, dtype=torch.float32, device="cuda")
        src = torch.from_numpy(pin["near_pts"])
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        probe.copy_(src, non_blocking=True)
        e0.record()
        probe.copy_(src, non_blocking=True)
        e1.record()
        src.copy_(probe, non_blocking=True)
        e2.record()
        torch.cuda.synchronize()
        link = {"h2d_gbs": src.numel() * 4 / (e0.elapsed_time(e1) / 1e3) / 1e9,
                "d2h_gbs": src.numel() * 4 / (e1.elapsed_time(e2) / 1e3) / 1e9}
        del probe
        e2e_steps = max(1, min(args.steps, 5))
        e2e_step()
        # Python's cyclic garbage collector off while the host-form calls are timed
        # (as timeit does): a full collection over this process's objects can pause
        # the calling thread for milliseconds between two enqueues
        gc.collect()
        gc.disable()
        barrier()
        t0 = time.perf_counter()
        try:
            for _ in range(e2e_steps):
                e2e_step()
            barrier()
        finally:
            gc.enable()
        e2e_s = time.perf_counter() - t0
        e2e_s = max_over_ranks(e2e_s, "cuda")
        h2d = sc.verts.nbytes + sc.faces.nbytes + sum(v.nbytes for v in q.values())
        d2h = sum(a.nbytes for v in hout.values() for a in v)
        host_answers = {"near_dist": hout["near"][1], "sil_dist": hout["sil"][0], "ray_hit": hout["ray"][0],
                        "ray_t": hout["ray"][1], "smp_idx": hout["smp"][0], "smp_pdf": hout["smp"][1]}
        mismatch = {k: bit_mismatches(v, device_answers[k]) for k, v in host_answers.items()}
        e2e = {"value": total_q * ws * e2e_steps / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
               "mismatches_vs_device_forms": mismatch, "pinned_link": link,
               "phase_ms": dict(zip(["create+build", "near", "sil", "ray", "smp", "close"],
                                    np.round(np.mean(e2e_parts[1:], 0), 2).tolist())),
               "step_phase_ms": [np.round(p, 2).tolist() for p in e2e_parts[1:]],
               "note": "scene upload + build + snch_*_host queries from pinned host memory, wall clock, "
                       "Python's garbage collector off while timed; answers compared bit for bit with the "
                       "device forms' answers of the timed step"}

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    # ---- CPU baseline (rank 0, N = 1): also yields the visit counts of the roofline
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        cpu = run_cpu(sc, q, counts, 0.005, cpu_threads())
        cpu.pop("tree")
    kinds = ["near", "sil", "ray", "smp"]
    dom = kinds[int(np.argmax(phase_ms[1:]))]
    peak, peak_src = hbm_peak()
    per_kernel = {}
    for i, k in enumerate(kinds):
        bq = algorithmic_bytes(k, visits[k])
        ms = float(phase_ms[1 + i])
        per_kernel[KERNEL_OF[k]] = {"ms": ms, "queries": counts[k], "visits_per_query": [float(x) for x in visits[k]],
                                    "bytes_per_query": bq, "GB/s": bq * counts[k] / (ms / 1e3) / 1e9}
        if cpu is not None:
            # the reference's own visit order (oracle sample): what the same
            # answers cost the reference's traversal, per second of ours
            bref = algorithmic_bytes(k, cpu["stats"][k])
            per_kernel[KERNEL_OF[k]]["reference_order_bytes_per_query"] = bref
            per_kernel[KERNEL_OF[k]]["effective_GB/s"] = bref * counts[k] / (ms / 1e3) / 1e9
    dk = per_kernel[KERNEL_OF[dom]]
    dom_ms = float(phase_ms[1 + kinds.index(dom)])
    traffic = traffic_of(KERNEL_OF[dom], "wost_2m")
    issue = issue_of(KERNEL_OF[dom])
    dram_gbs = traffic / (dom_ms / 1e3) / 1e9 if traffic else None
    roof = {"bound": "issue" if issue else "hbm", "kernel": KERNEL_OF[dom],
            "achieved": dram_gbs, "peak": peak, "unit": "GB/s",
            "frac": dram_gbs / peak if dram_gbs else None, "peak_source": peak_src, "traffic": traffic,
            "basis": "achieved = the kernel's measured DRAM bytes per launch (ncu, profiles/traffic.txt) / its "
                     "event time; the warp-packet searches are bound by instruction issue, not by HBM",
            "issue": issue,
            "effective": {"achieved": dk.get("effective_GB/s"),
                          "frac": dk["effective_GB/s"] / peak if "effective_GB/s" in dk else None,
                          "algorithmic_bytes_per_query": dk.get("reference_order_bytes_per_query"),
                          "basis": "reference record sizes x the visits of the reference's own traversal order "
                                   "(CPU restatement on a sample) / this kernel's time: what the same answers "
                                   "cost the reference's algorithm, per second of this kernel"},
            "own_visits": {"achieved": dk["GB/s"], "frac": dk["GB/s"] / peak,
                           "algorithmic_bytes_per_query": dk["bytes_per_query"],
                           "basis": "reference record sizes x this kernel's own per-lane visits / its time; a "
                                    "warp packet loads a shared record once for all its lanes, so this exceeds "
                                    "the bytes it moves"},
            "per_kernel": per_kernel}
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded meshes and queries)",
        "config": bench_config(counts, len(sc.faces), ws),
        "per_type_qps": {k: float(v) for k, v in per_type.items()},
        "ray_test": ray_test,
        "phase_ms": {"build": float(phase_ms[0]), **{k: float(phase_ms[1 + i]) for i, k in enumerate(kinds)}},
        "gpu_launches": int(launches),
        "stack": stack,
        "device_status": int(status),
        "clocks": clk,
        "roofline": roof,
        "e2e": e2e,
        "learned": learned,
        "icosphere": ico,
        "sort": sort_res,
        "batched": batched,
        "wost": wost_res,
    }
    if cpu is not None:
        smp = cpu["sample"]
        line["cpu_baseline"] = {"value": cpu["value"], "unit": "queries/s", "cores": cpu_threads(), "kind": "port",
                                "sample": f"single-thread build of the whole {len(sc.faces):,}-triangle scene + "
                                          f"the first {smp['near']:,} nearest, {smp['sil']:,} silhouette, "
                                          f"{smp['ray']:,} ray, {smp['smp']:,} sample queries (0.5 % of each batch); "
                                          f"value = those queries / the wall time",
                                "per_type_qps": {k: float(v) for k, v in cpu["qps"].items()},
                                "build_s": cpu["build_s"]}
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.sort_only:
        print(json.dumps({"sort": sort_leg()}), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
