#!/usr/bin/env python
"""Benchmark of the ray-cast hot path: batched TriMesh::cast_ray_and_get_normal on the
65,536-triangle terrain (256 x 128 height field) with 1,048,576 rays, max_toi = 100, solid.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one pass of the path over the whole ray batch (Morton sort of the rays + LBVH traversal
+ ray/triangle tests + result write), through the library's C ABI on device-resident buffers.
`e2e` is the same call with pinned host buffers (host->device rays and device->host hits inside
the timed region). L2 is flushed (256 MiB write) before every timed step, outside the step's
events. Under torchrun each rank runs its own replica of the workload on its GPU (no collective in
the data path); value = rays of all ranks / the slowest rank's time.

--impl reference times the oracle (the C++ restatement of parry3d's f32 path, the only CPU
implementation of the reference that builds here: no Rust toolchain) on all host threads, on the
same workload, metric and unit; under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_RAYS = 1 << 20
MAX_TOI = 100.0
METRIC = "Mrays/s"
WORKLOAD = "terrain_trimesh_rays"


def config(world: int, n_rays: int) -> dict:
    return {"workload": WORKLOAD, "triangles": 65536, "grid": "256x128", "rays": n_rays, "max_toi": MAX_TOI,
            "solid": True, "ray_dirs": "uniform downward hemisphere", "l2": "flushed before each step (256 MiB write)",
            "parallelism": f"shards{world}" if world > 1 else "single",
            "sharding": "one batch of rays_per_rank x ranks rays, each rank casting its contiguous range against its "
                        "replica of the mesh (no data exchange)" if world > 1 else None,
            "rays_per_rank": n_rays}


def reduce_max(x: float, world: int) -> float:
    """The largest x over the job's ranks (the slowest rank's time): one all_reduce of a float64 on
    the process group's device (CUDA for NCCL, CPU for gloo); the value itself when alone."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """Samples nvidia-smi clocks / throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names[1:], parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def measured_peak_bf16() -> tuple[float, str]:
    """Dense BF16 tensor peak (TFLOP/s) for a kernel timed alone: the driver's measured burst figure,
    else the earlier GB300 measurement."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["bf16_tflops"]), "measured"
        except Exception:
            pass
    return 1900.0, "fallback"


def measured_fp32_peak(n: int = 8192, reps: int = 3) -> float:
    """FP32 (FFMA) throughput measured in this process: cuBLAS SGEMM with TF32 off, n x n x n, best
    of `reps` (TFLOP/s). The denominator of the FP32-bound kernels' roofline."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn((n, n), device="cuda", dtype=torch.float32)
        b = torch.randn((n, n), device="cuda", dtype=torch.float32)
        c = a @ b
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b, c
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def profiled_traffic(name: str, key: str = "dram_bytes_per_launch_full_size") -> float | None:
    """A figure recorded from an ncu capture (profiles/<name>.txt, line `<key>: <value> ...`):
    by default the dram read+write bytes per launch at the full size."""
    p = ROOT / "profiles" / f"{name}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def cpu_oracle_rays(v, i, rays, reps: int):
    """Times the oracle (f32 restatement of parry3d) over all host threads; returns (Mrays/s, stats, threads)."""
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    m = O.TriMesh(v, i, "f32")
    _, _, _, stats = m.cast_rays_and_get_normal(rays, MAX_TOI, threads=threads, want_stats=True)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        m.cast_rays_and_get_normal(rays, MAX_TOI, threads=threads)
        times.append(time.perf_counter() - t0)
    return len(rays) / statistics.median(times) / 1e6, stats, threads


def rays_f64_error(v, i, rays, feat, toi, nrm, sample: int = 131072) -> dict:
    """Error of the device results against the f64 oracle (parry3d-f64 restated) on the first
    `sample` rays: hit agreement, relative toi error and normal error where both hit the same triangle."""
    import numpy as np
    from oracle import oracle as O
    k = min(sample, len(rays))
    f64, t64, n64 = O.TriMesh(v, i, "f64").cast_rays_and_get_normal(rays[:k], MAX_TOI)
    f32 = np.asarray(feat[:k]).view(np.uint32)
    both = (f32 == f64) & (f64 != 0xFFFFFFFF)
    rel = np.abs(np.asarray(toi[:k], np.float64)[both] - t64[both]) / np.maximum(np.abs(t64[both]), 1e-30)
    nerr = np.linalg.norm(np.asarray(nrm[:k], np.float64)[both] - n64[both], axis=1)
    return {"sample_rays": k, "same_hit_triangle": round(float(np.mean(f32 == f64)), 7),
            "toi_rel_err_max": float(rel.max(initial=0.0)), "toi_rel_err_p99": float(np.quantile(rel, 0.99)) if rel.size else 0.0,
            "normal_err_max": float(nerr.max(initial=0.0))}


def contacts_f64_error(s, pairs, has, res, sample: int = 16384) -> dict:
    """Error of the device contacts against the f64 oracle on the first `sample` pairs: has-contact
    agreement, and where both report a contact the depth, normal and contact-point errors."""
    import numpy as np
    from oracle import oracle as O
    k = min(sample, len(pairs))
    h64, o64, _ = O.contacts(s, pairs[:k], 0.0, precision="f64", threads=os.cpu_count() or 1)
    h32 = np.asarray(has[:k])
    r32 = np.asarray(res[:k], np.float64)
    both = (h32 != 0) & (h64 != 0)
    dist = np.abs(r32[both, 12] - o64[both, 12])
    nerr = np.linalg.norm(r32[both, 6:9] - o64[both, 6:9], axis=1)
    perr = np.maximum(np.linalg.norm(r32[both, 0:3] - o64[both, 0:3], axis=1),
                      np.linalg.norm(r32[both, 3:6] - o64[both, 3:6], axis=1))
    q = lambda a: float(np.quantile(a, 0.99)) if a.size else 0.0  # noqa: E731
    return {"sample_pairs": k, "has_contact_agreement": round(float(np.mean(h32 == h64)), 7),
            "depth_abs_err_max": float(dist.max(initial=0.0)), "depth_abs_err_p99": q(dist),
            "normal_err_max": float(nerr.max(initial=0.0)), "normal_err_p99": q(nerr),
            "point_err_max": float(perr.max(initial=0.0)), "point_err_p99": q(perr)}


def host_link_rates(stream, mb: int = 512, reps: int = 3) -> dict:
    """Pinned host <-> device copy rates of this process (one buffer of `mb` MB each way, best of
    `reps`): the ceiling the end-to-end figures' copies run against."""
    import torch
    h = torch.empty(mb << 20, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(mb << 20, dtype=torch.uint8, device="cuda")
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        best = float("inf")
        for _ in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            dst.copy_(src, non_blocking=True)
            b.record(stream)
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        out[name] = round((mb << 20) / (best / 1e3) / 1e9, 1)
    out["bytes"] = mb << 20
    del h, d
    return out


def broadphase_section(ctx, stream, steps: int, warmup: int, n_shapes: int, flush) -> dict:
    """Broadphase + narrow phase on 131,072 balls and cuboids (50/50) in a cube of side 400: shape
    AABBs loosened by prediction/2, LBVH build, all overlapping pairs (traverse_bvtt_single_tree),
    query::contact(prediction 0.1) on every pair. A step is the whole sequence on device-resident
    shapes; the pair count comes back to the host to size the contact call. Checked against the
    oracle's sorted pair set and contacts; the oracle runs the same sequence as the CPU baseline."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O

    pred = 0.1
    s = W.broadphase_shapes(n_shapes)
    t, prm, pos, pool = s.arrays()
    dev = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (t.view(np.int32), prm, pos, pool))
    aabbs = torch.empty((n_shapes, 6), dtype=torch.float32, device="cuda")
    pg.shape_aabbs(ctx, dev, pred / 2, out=aabbs)
    bvh = pg.Bvh.from_leaves(ctx, aabbs)
    cap = 8 * n_shapes
    pairs = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    has = torch.empty(cap, dtype=torch.uint8, device="cuda")
    res = torch.empty((cap, 13), dtype=torch.float32, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    split = np.zeros(3)

    def step(record: bool):
        if record:
            ev[0].record(stream)
        pg.shape_aabbs(ctx, dev, pred / 2, out=aabbs)
        bvh.rebuild(aabbs)
        if record:
            ev[1].record(stream)
        m = bvh.traverse_bvtt_single_tree_into(pairs)
        if record:
            ev[2].record(stream)
        pg.contacts(ctx, dev, pairs[:m], pred, out=(has[:m], res[:m]))
        if record:
            ev[3].record(stream)
        return m

    for _ in range(max(1, warmup)):
        m = step(False)
    torch.cuda.synchronize()
    l0 = ctx.kernel_launches
    times = []
    for _ in range(steps):
        flush.zero_()
        m = step(True)
        torch.cuda.synchronize()
        times.append(ev[0].elapsed_time(ev[3]))
        split += [ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2]), ev[2].elapsed_time(ev[3])]
    launches = (ctx.kernel_launches - l0) // max(steps, 1)
    ms = statistics.mean(times)
    # oracle: the same sequence on the host cores (binned BVH, its own traversal), timed
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oa = O.shape_aabbs(s, pred / 2)
    opairs = O.canonical_sorted_pairs(O.Bvh(oa).traverse_bvtt_single_tree())
    oh, oo, _ = O.contacts(s, opairs, pred, threads=threads)
    cpu_s = time.perf_counter() - t0
    dev_pairs = pairs[:m].cpu().numpy().view(np.uint32)
    order = np.lexsort((dev_pairs[:, 1], dev_pairs[:, 0]))
    same_pairs = bool(np.array_equal(dev_pairs[order], opairs))
    same_has = same_pairs and bool(np.array_equal(has[:m].cpu().numpy()[order], oh))
    bvh.close()
    return {
        "workload": f"{n_shapes} balls and cuboids (50/50), radius / half extents log-uniform [0.25, 4], uniform rotations, "
                    "centres U([-200, 200)^3); AABBs loosened by 0.05; LBVH; all overlapping pairs; query::contact(prediction 0.1)",
        "metric": "broadphase+contact steps/s", "value": round(1e3 / ms, 2), "unit": "steps/s", "ms_per_step": round(ms, 4),
        "shapes_per_s": round(n_shapes / (ms / 1e3), 1), "pairs": int(m), "contacts": int(oh.sum()),
        "stage_ms": {"aabbs_and_build": round(split[0] / steps, 4), "pairs": round(split[1] / steps, 4),
                     "contacts": round(split[2] / steps, 4)},
        "gpu_launches": int(launches),
        "matches_oracle": {"pair_set": same_pairs, "has_contact": same_has},
        "cpu_baseline": {"value": round(1.0 / cpu_s, 3), "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": "one full step: oracle shape AABBs, parry binned BVH build, traversal, contacts over all threads"},
    }


def mixed_contacts(ctx, stream, steps: int, n_pairs: int, flush) -> dict:
    """query::contact on the uneven hull workload with balls, cuboids and capsules mixed in (a shape
    of each pair is any of the four kinds, hulls of 8-256 vertices): device-resident pairs/s, the
    oracle check and CPU baseline on a sample."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    from oracle import oracle as O

    s, pairs = W.mixed_contact_pairs(n_pairs)
    t, prm, pos, pool = s.arrays()
    dev = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (t.view(np.int32), prm, pos, pool))
    dpairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    has = torch.empty(n_pairs, dtype=torch.uint8, device="cuda")
    res = torch.empty((n_pairs, 13), dtype=torch.float32, device="cuda")
    pg.contacts(ctx, dev, dpairs, 0.0, out=(has, res))
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        pg.contacts(ctx, dev, dpairs, 0.0, out=(has, res))
        b.record(stream)
    torch.cuda.synchronize()
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    sample = min(n_pairs, 131072)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oh, oo, _ = O.contacts(s, pairs[:sample], 0.0, threads=threads)
    cpu_s = time.perf_counter() - t0
    return {"workload": "pairs of balls, cuboids, capsules and 8-256-vertex hulls (uniform kinds), random relative pose, prediction 0",
            "pairs": n_pairs, "value": round(n_pairs / (ms / 1e3), 1), "unit": "pairs/s", "ms_per_step": round(ms, 4),
            "contact_fraction": round(float(has.float().mean().item()), 4),
            "matches_oracle_on_sample": bool(np.array_equal(oh, has[:sample].cpu().numpy())),
            "cpu_baseline": {"value": round(sample / cpu_s, 1), "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": f"first {sample} pairs"}}


def hull_build_section(ctx, steps: int, n_hulls: int) -> dict:
    """ConvexPolyhedron::from_convex_hull for many clouds (16-64 points on ellipsoids, the hull
    workload of the manifold and contact sections) on the GPU, inputs resident on the device; the
    call is synchronous (it reads the output sizes back), so it is timed on the host clock. The
    host builder (the same algorithm on all host threads) is the CPU baseline on a sample, and the
    GPU output of that sample must equal the host's byte for byte."""
    import ctypes as C
    import numpy as np
    import torch
    from parry_gb300 import workloads as W
    from parry_gb300._capi import lib, check
    from parry_gb300.polyhedra import build_polyhedra

    cloud, first, count = W.ellipsoid_hulls(n_hulls, 66, 7, 16, 64)
    d_cloud, d_first, d_count = (torch.from_numpy(cloud).cuda(), torch.from_numpy(first.view(np.int32)).cuda(),
                                 torch.from_numpy(count.view(np.int32)).cuda())
    L = lib()

    def run():
        h = C.c_void_p()
        check(L.parrygpu_polyhedra_build_gpu(ctx.handle, C.c_void_p(d_cloud.data_ptr()), len(cloud), C.c_void_p(d_first.data_ptr()),
                                             C.c_void_p(d_count.data_ptr()), n_hulls, C.byref(h)), ctx.handle)
        sizes = np.zeros(5, np.uint64)
        check(L.parrygpu_polyhedra_gpu_sizes(h, C.c_void_p(sizes.ctypes.data)))
        L.parrygpu_polyhedra_gpu_destroy(h)
        return sizes

    sizes = run()
    torch.cuda.synchronize()
    times = []
    for _ in range(max(3, min(steps, 10))):
        t0 = time.perf_counter()
        run()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.median(times)
    # end to end: host clouds in, host arrays out - pinned buffers allocated once (the sizes of the
    # device run), and for comparison freshly allocated pageable arrays
    npts, nf, nfe, nve, ne = (int(x) for x in sizes)

    def pinned(shape, dt):
        return torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    p_in = (pinned(cloud.shape, torch.float32), pinned(first.shape, torch.int32).view(np.uint32),
            pinned(count.shape, torch.int32).view(np.uint32))
    for dst, src in zip(p_in, (cloud, first, count)):
        dst[...] = src
    p_out = {"points": pinned((npts, 3), torch.float32), "hulls": pinned((n_hulls, 8), torch.int32).view(np.uint32),
             "face_normals": pinned((nf, 3), torch.float32), "face_ranges": pinned((nf, 2), torch.int32).view(np.uint32),
             "face_vertices": pinned(nfe, torch.int32).view(np.uint32), "face_edges": pinned(nfe, torch.int32).view(np.uint32),
             "vertex_ranges": pinned((npts, 2), torch.int32).view(np.uint32), "vertex_faces": pinned(nve, torch.int32).view(np.uint32),
             "vertex_edges": pinned(nve, torch.int32).view(np.uint32), "edge_dirs": pinned((ne, 3), torch.float32)}
    out_bytes = sum(a.nbytes for a in p_out.values())
    build_polyhedra(*p_in, ctx=ctx, out=p_out)
    e2e_times = []
    for _ in range(3):
        t0 = time.perf_counter()
        build_polyhedra(*p_in, ctx=ctx, out=p_out)
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * statistics.median(e2e_times)
    t0 = time.perf_counter()
    build_polyhedra(cloud, first, count, ctx=ctx)
    e2e_pageable_ms = 1e3 * (time.perf_counter() - t0)
    del p_out, p_in
    sample = min(n_hulls, 65536)
    sc = cloud[: int(first[sample - 1] + count[sample - 1])]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    host = build_polyhedra(sc, first[:sample], count[:sample], threads=threads)
    cpu_s = time.perf_counter() - t0
    dev = build_polyhedra(sc, first[:sample], count[:sample], ctx=ctx)
    same = bool(all(np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in [(host[0], dev[0]), (host[1], dev[1])]) and
                all(np.array_equal(host[2][k].view(np.uint32), dev[2][k].view(np.uint32)) for k in host[2]))
    return {"workload": f"{n_hulls} clouds of 16-64 points on ellipsoids (log-uniform counts)", "metric": "hulls/s",
            "value": round(n_hulls / (ms / 1e3), 1), "unit": "hulls/s", "ms_per_step": round(ms, 3),
            "faces": int(sizes[1]), "edges": int(sizes[4]),
            "e2e": {"value": round(n_hulls / (e2e_ms / 1e3), 1), "unit": "hulls/s", "ms": round(e2e_ms, 2),
                    "h2d_bytes": int(cloud.nbytes + first.nbytes + count.nbytes), "d2h_bytes": int(out_bytes),
                    "note": "pinned host clouds in, pinned host arrays out (allocated once), median of 3",
                    "pageable": {"value": round(n_hulls / (e2e_pageable_ms / 1e3), 1), "unit": "hulls/s",
                                 "ms": round(e2e_pageable_ms, 2), "note": "numpy clouds in, freshly allocated numpy arrays out"}},
            "matches_host_builder_on_sample": same,
            "cpu_baseline": {"value": round(sample / cpu_s, 1), "unit": "hulls/s", "cores": threads, "kind": "port",
                             "sample": f"first {sample} clouds; the same hull + from_convex_mesh code on host threads"}}


def shape_cast_section(ctx, stream, steps: int, n_pairs: int, flush) -> dict:
    """query::cast_shapes on separated ball / cuboid / capsule / hull pairs closing at 0.5-2 units per
    unit time (W.shape_cast_pairs, max_toi 100): device-resident pairs/s, oracle check and CPU
    baseline on a sample."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    from oracle import oracle as O

    s, pairs, vels = W.shape_cast_pairs(n_pairs)
    t, prm, pos, pool = s.arrays()
    dev = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (t.view(np.int32), prm, pos, pool))
    dpairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    dvel = torch.from_numpy(vels).cuda()
    st = torch.empty(n_pairs, dtype=torch.uint8, device="cuda")
    res = torch.empty((n_pairs, 13), dtype=torch.float32, device="cuda")
    pg.cast_shapes(ctx, dev, dpairs, dvel, max_toi=100.0, out=(st, res))
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        pg.cast_shapes(ctx, dev, dpairs, dvel, max_toi=100.0, out=(st, res))
        b.record(stream)
    torch.cuda.synchronize()
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    sample = min(n_pairs, 131072)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    so, oo, _ = O.cast_shapes(s, pairs[:sample], vels, max_toi=100.0, threads=threads)
    cpu_s = time.perf_counter() - t0
    got = st[:sample].cpu().numpy()
    return {"workload": "separated ball/cuboid/capsule/hull(8-256) pairs closing at U[0.5, 2], max_toi 100",
            "metric": "shape casts/s", "pairs": n_pairs, "value": round(n_pairs / (ms / 1e3), 1), "unit": "pairs/s",
            "ms_per_step": round(ms, 4), "hit_fraction": round(float((st != 255).float().mean().item()), 4),
            "matches_oracle_on_sample": bool(np.array_equal(got, so)),
            "cpu_baseline": {"value": round(sample / cpu_s, 1), "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": f"first {sample} pairs"}}


def trimesh_contacts_section(ctx, stream, frames: int, warmup: int, n_shapes: int, flush, fix: bool = False,
                             sample: int = 2048) -> dict:
    """Contact manifolds of mixed shapes against the 65,536-triangle terrain, frame after frame
    (contact_manifolds_trimesh_shape with its workspace): ball / cuboid / capsule / hull(16-64)
    shapes drifting down onto the height field; a step is one frame's update on device-resident
    shapes. With `fix` the mesh has TriMeshFlags::FIX_INTERNAL_EDGES (pseudo-normal constraints).
    Interference lists and manifold records are checked bit-exact against the oracle's frame loop
    on a sample of shapes, which is also the CPU baseline."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    from parry_gb300.shapes import ShapeSet
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O

    v, i = W.terrain_mesh()
    t, prm, pos0, pool, poly, _ = W.primitive_pairs(n_shapes // 2, seed=0x9A77E7)
    n = len(t)
    rng = np.random.default_rng(7)
    pos0 = pos0.copy()
    pos0[:, 4] = rng.uniform(2, 254, n)
    pos0[:, 6] = rng.uniform(2, 126, n)
    pos0[:, 5] = rng.uniform(1.0, 6.0, n)
    vel = np.zeros((n, 3), np.float32)
    vel[:, 1] = -rng.uniform(0.01, 0.05, n).astype(np.float32)
    vel[:, 0] = rng.normal(0, 0.01, n).astype(np.float32)
    total = warmup + frames
    poses = np.repeat(pos0[None], total, 0)
    poses[:, :, 4:7] += vel[None] * np.arange(total, dtype=np.float32)[:, None, None]
    dpos = torch.from_numpy(poses).cuda()
    hulls, topo = poly
    dpoly = (torch.from_numpy(hulls.view(np.int32)).cuda(),
             {k: torch.from_numpy(x.view(np.int32) if x.dtype == np.uint32 else x).cuda() for k, x in topo.items()})
    dt_, dp_, dpool = (torch.from_numpy(t.view(np.int32)).cuda(), torch.from_numpy(prm).cuda(), torch.from_numpy(pool).cuda())
    mesh = pg.TriMesh(ctx, v, i, flags=pg.TRIMESH_FIX_INTERNAL_EDGES if fix else 0)
    K = 64
    tc = pg.TriMeshContacts(ctx, mesh, n, K)
    pred = 0.02
    for f in range(warmup):
        tc.update((dt_, dp_, dpos[f], dpool, dpoly), pred)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
    l0 = ctx.kernel_launches
    for k, (a, b) in enumerate(ev):
        flush.zero_()
        a.record(stream)
        tc.update((dt_, dp_, dpos[warmup + k], dpool, dpoly), pred)
        b.record(stream)
    torch.cuda.synchronize()
    launches = (ctx.kernel_launches - l0) // max(frames, 1)
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    counts, tris, recs = tc.read()
    active = int(counts.sum())
    with_points = int(sum((recs[s, :counts[s]]["n_points"] > 0).sum() for s in range(n)))
    # oracle frame loop on a sample of shapes (the same frames), timed for the CPU baseline
    sample = min(n, sample)
    sel = np.arange(sample)
    ref = O.TriMeshContacts(v, i, sample, fix_internal_edges=fix)
    mesh_pose = np.array([0, 0, 0, 1, 0, 0, 0], np.float32)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    for f in range(total):
        ref.update(mesh_pose, ShapeSet.from_arrays(t[sel], prm[sel], poses[f][sel], pool, poly), pred, threads)
    cpu_s = (time.perf_counter() - t0) / total
    same = all(int(counts[s]) == len(ref.inter[s]) and np.array_equal(tris[s, :counts[s]], ref.inter[s]) for s in range(sample))
    if same:
        from parry_gb300 import manifold as M
        g = np.concatenate([recs[s, :counts[s]] for s in range(sample)]).copy()
        w = np.concatenate([ref.records[s].view(M.MANIFOLD_DTYPE).reshape(-1) for s in range(sample)]).copy()
        g["status"] = 0
        w["status"] = 0
        gw, ww = M.as_words(g), M.as_words(w)
        live = np.arange(M.MAX_POINTS)[None, :] < w["n_points"].astype(np.int64)[:, None]
        same = bool(np.array_equal(g["n_points"], w["n_points"]) and np.array_equal(gw[:, :8], ww[:, :8]) and
                    np.array_equal(gw[:, 8:].reshape(len(g), M.MAX_POINTS, 10)[live], ww[:, 8:].reshape(len(w), M.MAX_POINTS, 10)[live]))
    tc.close()
    mesh.close()
    return {"workload": f"{n} ball/cuboid/capsule/hull(16-64) shapes drifting onto the 65,536-triangle terrain, prediction {pred}, "
                        f"at most {K} triangles per shape" + (", FIX_INTERNAL_EDGES (pseudo-normal constraints)" if fix else ""),
            "metric": "frames/s", "value": round(1e3 / ms, 2), "unit": "frames/s", "ms_per_frame": round(ms, 4), "frames": frames,
            "shape_triangle_manifolds": active, "with_points": with_points,
            "manifold_updates_per_s": round(active / (ms / 1e3), 1), "gpu_launches": int(launches),
            "matches_oracle_on_sample": bool(same),
            "cpu_baseline": {"value": round(sample / n / cpu_s, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": f"the first {sample} shapes (one frame scaled to all {n}); C++ manifolds, numpy workspace"}}


def contacts_section(ctx, stream, steps: int, warmup: int, n_pairs: int, flush, epa_blocks: int = 0) -> dict:
    """Batched query::contact on uneven convex-hull pairs (8-256 vertices, log-uniform), the
    GJK/EPA workload: device-resident pairs/s, end-to-end pairs/s through host buffers, kernel
    split, FP32 roofline from the oracle's support-scan count, and the oracle CPU baseline."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O

    s, pairs = W.hull_pairs(n_pairs)
    t, prm, pos, pool = s.arrays()
    dev = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (t.view(np.int32), prm, pos, pool))
    dpairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    contacts_section.device_inputs = (dev, dpairs)
    has = torch.empty(n_pairs, dtype=torch.uint8, device="cuda")
    res = torch.empty((n_pairs, 13), dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    if epa_blocks:
        cfg = dict(ctx.config, epa_blocks_per_sm=epa_blocks, contact_warp_cost=4096, contact_epa_inline=2)
        ctx_c = pg.Context(**cfg)
        ctx_c.set_stream(stream.cuda_stream)
        tune = {"fixed": {k: cfg[k] for k in ("epa_blocks_per_sm", "contact_warp_cost", "contact_epa_inline")}}
        ctx = ctx_c
    else:
        # tuned on the whole pair set: the best EPA residency depends on how many pairs reach EPA at
        # once, so a smaller sample picks for a different load
        chosen = pg.autotune_contacts(ctx, dev, dpairs, 0.0, reps=1)
        tune = {"chosen": {k: chosen[k] for k in ("epa_blocks_per_sm", "contact_warp_cost", "contact_epa_inline")},
                "sample_pairs": n_pairs, "seconds": round(time.perf_counter() - t0, 3)}
    for _ in range(max(1, warmup)):
        pg.contacts(ctx, dev, dpairs, 0.0, out=(has, res))
    torch.cuda.synchronize()
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_timing()
    st_ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    en_ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    l0 = ctx.kernel_launches
    for k in range(steps):
        flush.zero_()
        st_ev[k].record(stream)
        pg.contacts(ctx, dev, dpairs, 0.0, out=(has, res))
        en_ev[k].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(st_ev, en_ev)) / steps
    g_ms, g_n = ctx.kernel_time("contacts_gjk")
    e_ms, e_n = ctx.kernel_time("contacts_epa")
    b_ms, b_n = ctx.kernel_time("contacts_bin")
    ctx.enable_kernel_timing(False)
    launches = ctx.kernel_launches - l0
    _, _, gst = pg.contacts(ctx, dev, dpairs, 0.0, out=(has, res), want_stats=True)
    # end to end from pinned host buffers
    host = tuple(torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (t.view(np.int32), prm, pos, pool))
    hpairs = torch.from_numpy(pairs.view(np.int32)).pin_memory()
    hhas = torch.empty(n_pairs, dtype=torch.uint8, pin_memory=True)
    hres = torch.empty((n_pairs, 13), dtype=torch.float32, pin_memory=True)
    pg.contacts(ctx, host, hpairs, 0.0, out=(hhas, hres))
    e2e = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pg.contacts(ctx, host, hpairs, 0.0, out=(hhas, hres))
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = statistics.mean(e2e)
    h2d = sum(a.numel() * a.element_size() for a in host) + hpairs.numel() * 4
    d2h = n_pairs * (13 * 4 + 1)
    # oracle on a bounded sample: CPU baseline and the support-scan count of the flop model
    sample = min(n_pairs, 131072)
    threads = os.cpu_count() or 1
    O.contacts(s, pairs[:2048], 0.0, threads=threads)
    t0 = time.perf_counter()
    oh, oo, ost = O.contacts(s, pairs[:sample], 0.0, threads=threads)
    cpu_s = time.perf_counter() - t0
    same = bool(np.array_equal(oh, has[:sample].cpu().numpy()))
    flops_per_pair = 5.0 * ost["support_vertices"] / sample
    kernel_ms = g_ms / max(g_n, 1) + e_ms / max(e_n, 1)
    sm_mhz = 2070.0
    try:
        sm_mhz = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["sm_max_mhz"])
    except Exception:
        pass
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    fp32_nominal = sms * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_peak = measured_fp32_peak()
    achieved = flops_per_pair * n_pairs / (kernel_ms / 1e3) / 1e12
    # algorithmic HBM bytes per pair: both hulls' vertices once, the pair, two poses and params, the
    # output; against the DRAM bytes an ncu capture of the same kernels measured per pair
    hull_bytes = 12.0 * float(np.sum(prm.view(np.uint32)[:, 1][pairs.reshape(-1)].astype(np.float64))) / n_pairs
    alg_bytes = hull_bytes + 8 + 2 * (28 + 16 + 4) + 53
    hbm_peak, hbm_kind = measured_peak_hbm()
    prof = profiled_traffic("contacts_gjk_epa_hull_pairs", "dram_bytes_per_pair")
    return {
        "workload": "convex hull pairs, 8-256 vertices log-uniform on ellipsoids, random relative pose, prediction 0",
        "pairs": n_pairs, "metric": "contact pairs/s", "value": round(n_pairs / (ms / 1e3), 1), "unit": "pairs/s",
        "ms_per_step": round(ms, 4), "kernel_ms": {"bin": round(b_ms / max(b_n, 1), 4), "gjk": round(g_ms / max(g_n, 1), 4),
                                          "epa": round(e_ms / max(e_n, 1), 4)},
        "gpu_launches": launches,
        "autotune": tune,
        "e2e": {"value": round(n_pairs / (e2e_ms / 1e3), 1), "unit": "pairs/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 3)},
        "mean_iterations": {"gjk": round(gst["gjk_iters"] / n_pairs, 4), "epa": round(gst["epa_iters"] / n_pairs, 4),
                            "epa_calls": gst["epa_calls"]},
        "contact_fraction": round(float(has.float().mean().item()), 4),
        "roofline": {"bound": "fp32", "achieved": round(achieved, 4), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                     "frac": round(achieved / fp32_peak, 6), "peak_source": "measured: cuBLAS SGEMM 8192^3, TF32 off, in this process",
                     "nominal_peak": round(fp32_nominal, 1), "nominal_source": "SMs x 128 lanes x 2 (FMA) x max SM clock",
                     "flops_per_pair": round(flops_per_pair, 1),
                     "flops_model": "5 flops per vertex dot x vertices scanned by the f32 oracle's support calls on a sample"},
        "roofline_hbm": {"bound": "hbm", "achieved": round(alg_bytes * n_pairs / (kernel_ms / 1e3) / 1e9, 1), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(alg_bytes * n_pairs / (kernel_ms / 1e3) / 1e9 / hbm_peak, 4),
                         "peak_source": hbm_kind, "algorithmic_bytes_per_pair": round(alg_bytes, 1),
                         "dram_bytes_per_pair_profiled": prof,
                         "bytes_model": "12 B per hull vertex of both shapes once + pair, poses, params, output"},
        "cpu_baseline": {"value": round(sample / cpu_s, 1), "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"first {sample} pairs; C++ restatement of parry3d f32 query::contact"},
        "matches_oracle_on_sample": same,
        "error_vs_f64_oracle": contacts_f64_error(s, pairs, has.cpu().numpy(), res.cpu().numpy()),
        "mixed_shapes": mixed_contacts(ctx, stream, steps, n_pairs, flush),
    }


def manifolds_section(ctx, stream, steps: int, warmup: int, n_pairs: int, flush) -> dict:
    """Persistent contact manifolds on ball/cuboid/capsule pairs drifting frame to frame: each step
    updates every pair's record in place at the next frame's poses (device-resident), plus a cold
    update from empty records, the end-to-end call through host records, a bit-exact check against
    the oracle on a sample, and the oracle CPU baseline."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    from parry_gb300 import manifold as M
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O

    t, prm, pos0, pool, poly, pairs = W.primitive_pairs(n_pairs)
    frames = warmup + steps + 1
    dt_ = torch.from_numpy(t.view(np.int32)).cuda()
    dp_ = torch.from_numpy(prm).cuda()
    dpool = torch.from_numpy(pool).cuda()
    hulls, topo = poly
    dpoly = (torch.from_numpy(hulls.view(np.int32)).cuda(),
             {k: torch.from_numpy(v.view(np.int32) if v.dtype == np.uint32 else v).cuda() for k, v in topo.items()})
    dpairs = torch.from_numpy(pairs.view(np.int32)).cuda()
    host_poses = [W.drifted_poses(pos0, f) for f in range(frames)]
    dposes = [torch.from_numpy(p).cuda() for p in host_poses]
    rec = torch.zeros((n_pairs, M.RECORD_WORDS), dtype=torch.int32, device="cuda")
    pred = 0.02
    # cold: empty records, every generator from scratch
    cold_ms = []
    for _ in range(3):
        rec.zero_()
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        pg.contact_manifolds(ctx, (dt_, dp_, dposes[0], dpool, dpoly), dpairs, pred, rec)
        b.record(stream)
        torch.cuda.synchronize()
        cold_ms.append(a.elapsed_time(b))
    for f in range(1, warmup + 1):
        pg.contact_manifolds(ctx, (dt_, dp_, dposes[f], dpool, dpoly), dpairs, pred, rec)
    torch.cuda.synchronize()
    before_last = None
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_timing()
    l0 = ctx.kernel_launches
    st_ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    en_ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        f = warmup + 1 + k
        if k == steps - 1:
            torch.cuda.synchronize()
            before_last = rec[: min(n_pairs, 65536)].cpu().numpy().view(np.uint32).copy()
        flush.zero_()
        st_ev[k].record(stream)
        pg.contact_manifolds(ctx, (dt_, dp_, dposes[f], dpool, dpoly), dpairs, pred, rec)
        en_ev[k].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(st_ev, en_ev)) / steps
    m_ms, m_n = ctx.kernel_time("manifolds")
    ctx.enable_kernel_timing(False)
    launches = ctx.kernel_launches - l0
    last_f = warmup + steps
    after = rec.cpu().numpy().view(np.uint32).copy()
    recs_after = M.as_records(after)
    # bit-exact check on a sample: the oracle applies the last frame to the same starting records
    sample = len(before_last)
    shapes_last = pg.ShapeSet.from_arrays(t, prm, host_poses[last_f], pool, poly)
    chk = before_last.copy()
    O.contact_manifolds(shapes_last, pairs[:sample], pred, chk)
    g, w = recs_after[:sample], M.as_records(chk)
    n = w["n_points"].astype(np.int64)
    valid = np.arange(M.MAX_POINTS)[None, :] < n[:, None]
    gp = after[:sample, 8:].reshape(sample, M.MAX_POINTS, 10)
    wp = chk[:, 8:].reshape(sample, M.MAX_POINTS, 10)
    same = bool(np.array_equal(g["n_points"], w["n_points"]) and np.array_equal(after[:sample, :8], chk[:, :8])
                and np.array_equal(gp[valid], wp[valid]))
    # end to end: pinned host records and shape arrays, both copies inside the timed region
    host_rec = torch.from_numpy(after.view(np.int32)).pin_memory()
    ht = torch.from_numpy(t.view(np.int32)).pin_memory()
    hp = torch.from_numpy(prm).pin_memory()
    hq = [torch.from_numpy(p).pin_memory() for p in host_poses]
    hpool = torch.from_numpy(pool).pin_memory()
    hpoly = (torch.from_numpy(hulls.view(np.int32)).pin_memory(),
             {k: torch.from_numpy(v.view(np.int32) if v.dtype == np.uint32 else v).pin_memory() for k, v in topo.items()})
    hpairs = torch.from_numpy(pairs.view(np.int32)).pin_memory()
    pg.contact_manifolds(ctx, (ht, hp, hq[0], hpool, hpoly), hpairs, pred, host_rec)
    e2e = []
    for k in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pg.contact_manifolds(ctx, (ht, hp, hq[(k + 1) % frames], hpool, hpoly), hpairs, pred, host_rec)
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = statistics.mean(e2e)
    h2d = (t.nbytes + prm.nbytes + host_poses[0].nbytes + pool.nbytes + hulls.nbytes + sum(v.nbytes for v in topo.values())
           + pairs.nbytes + after.nbytes)
    d2h = after.nbytes
    # oracle CPU baseline on a bounded sample (one frame update from the same records)
    threads = os.cpu_count() or 1
    csample = min(n_pairs, 262144)
    base = after[:csample].copy()
    t0 = time.perf_counter()
    O.contact_manifolds(pg.ShapeSet.from_arrays(t, prm, host_poses[0], pool, poly), pairs[:csample], pred, base, threads=threads)
    cpu_s = time.perf_counter() - t0
    npts = recs_after["n_points"].astype(np.float64)
    mean_pts = float(npts.mean())
    # algorithmic bytes per pair: pair 8 B, two shapes (type 4 + params 16 + pose 28), record
    # header and live points read and written (32 B + 40 B per point each way)
    bytes_per_pair = 8 + 2 * 48 + 2 * (32 + 40 * mean_pts)
    kernel_ms = m_ms / max(m_n, 1)
    achieved = bytes_per_pair * n_pairs / (kernel_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    kinds = np.bincount((t[pairs[:, 0]] * 4 + t[pairs[:, 1]]).astype(np.int64), minlength=16)
    return {
        "workload": "ball/cuboid/capsule/convex-hull(16-64 points) pairs (uniform kinds), random relative pose at distance "
                    "U[0.5, 3], drifting frame to frame (v U[-0.3, 0.3]^3, w U[-0.5, 0.5]^3, dt 1/60), prediction 0.02",
        "pairs": n_pairs, "metric": "manifold pair updates/s", "value": round(n_pairs / (ms / 1e3), 1), "unit": "pairs/s",
        "ms_per_step": round(ms, 4), "cold_ms": round(min(cold_ms), 4),
        "cold_value": round(n_pairs / (min(cold_ms) / 1e3), 1),
        "kernel_ms": round(kernel_ms, 4),
        "gpu_launches": launches,
        "mean_points": round(mean_pts, 3), "pairs_with_points": round(float((npts > 0).mean()), 4),
        "pair_kinds": [int(x) for x in kinds],
        "e2e": {"value": round(n_pairs / (e2e_ms / 1e3), 1), "unit": "pairs/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 3)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "peak_source": peak_kind, "bytes_per_pair": round(bytes_per_pair, 1),
                     "bytes_model": "pair 8 + 2 x (type 4 + params 16 + pose 28) + record header and live points read and "
                                    "written (2 x (32 + 40 x mean points))"},
        "cpu_baseline": {"value": round(csample / cpu_s, 1), "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"one frame update of the first {csample} pairs; C++ restatement of parry3d f32"},
        "matches_oracle_on_sample": same, "oracle_sample": sample,
    }


def scene_section(ctx, stream, frames: int, warmup: int, flush, n_shapes: int = 262144, n_rays: int = 4194304) -> dict:
    """The per-frame pipeline on 262,144 moving shapes (ball / cuboid / capsule / hull, 25 % each) in
    an 800-wide cube with 4,194,304 rays per frame: integrate, AABBs, refit, pairs, manifolds carried
    per pair, rays; `frames` frames replayed from a CUDA graph, a stage split from one eager frame, the
    end-to-end frame with its outputs read back to the host, and the oracle frame on the host cores."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W
    from parry_gb300 import manifold as M
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O

    # the shapes' density is kept when the scene is scaled down (cube side 800 at 262,144 shapes)
    extent = 400.0 * (n_shapes / 262144.0) ** (1.0 / 3.0)
    t, prm, pos, pool, poly, vel, rays = W.frame_scene(n_shapes, n_rays, extent)
    shapes = pg.ShapeSet.from_arrays(t, prm, pos, pool, poly)
    pred, dt, max_toi = 0.1, 1.0 / 60.0, 100.0
    sc = pg.Scene(ctx, shapes, vel, pred, max(1 << 16, 4 * n_shapes))
    sc.set_rays(torch.from_numpy(rays).cuda(), max_toi)
    sc.step(dt, 2 * max(1, (warmup + 1) // 2), use_graph=True)
    torch.cuda.synchronize()
    l0 = ctx.kernel_launches
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.zero_()
    a.record(stream)
    sc.step(dt, frames, use_graph=True)
    b.record(stream)
    torch.cuda.synchronize()
    graph_ms = a.elapsed_time(b) / frames
    launches = ctx.kernel_launches - l0
    frame_no, npairs = sc.info()
    plain_stats = sc.stats()
    # stage split: one eager frame with per-stage events
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_timing()
    sc.step(dt, 1, use_graph=False)
    stages = {}
    for name in ("integrate", "aabbs", "refit", "pairs", "carry", "manifolds", "rays"):
        ms, n = ctx.kernel_time("scene_" + name)
        stages[name] = round(ms / max(n, 1), 4)
    ctx.enable_kernel_timing(False)
    st = sc.read()
    npts = st["manifolds"]["n_points"]
    hits = int((st["ray_part"] != pg.NO_HIT).sum())
    # end to end: each frame's outputs (poses, pairs, manifold records, ray hits) read back into pinned
    # host buffers allocated once
    rows = max(65536, 2 * int(npairs))
    pin = {"poses": torch.empty((n_shapes, 7), dtype=torch.float32, pin_memory=True),
           "pairs": torch.empty((rows, 2), dtype=torch.int32, pin_memory=True),
           "manifolds": torch.empty((rows, M.RECORD_WORDS), dtype=torch.int32, pin_memory=True),
           "ray_part": torch.empty(len(rays), dtype=torch.int32, pin_memory=True),
           "ray_toi": torch.empty(len(rays), dtype=torch.float32, pin_memory=True),
           "ray_normal": torch.empty((len(rays), 3), dtype=torch.float32, pin_memory=True)}
    e2e = []
    for _ in range(5):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc.step(dt, 1, use_graph=False)
        out = sc.read(out=pin)
        e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = statistics.mean(e2e[1:])
    d2h = sum(v.numel() * v.element_size() for v in out.values())
    # the same with each frame's copies overlapped with the next frame (Scene.read(wait=False)): K
    # frames from the first step to the last frame's copies done
    sc.step(dt, 1, use_graph=False)
    sc.read(out=pin, wait=False)
    sc.read_wait()
    k_async = 8
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(k_async):
        sc.step(dt, 1, use_graph=False)
        out_a = sc.read(out=pin, wait=False)
    sc.read_wait()
    async_ms = (time.perf_counter() - t0) * 1e3 / k_async
    d2h_async = sum(v.numel() * v.element_size() for v in out_a.values())
    sc.close()
    learned = scene_learned(ctx, stream, shapes, vel, rays, pred, dt, max_toi, max(1 << 16, 4 * n_shapes), frames, warmup, flush,
                            st, graph_ms, plain_stats, stages["manifolds"])
    # the oracle frame on the host cores: the full shape set, a 262,144-ray sample scaled to 4,194,304
    threads = os.cpu_count() or 1
    sample = min(262144, len(rays))
    t0 = time.perf_counter()
    want = O.scene_frames(shapes, vel, pred, dt, 1, threads=threads)
    t_frame = time.perf_counter() - t0
    moved = shapes.with_poses(O.integrate(pos, vel, dt))
    comp = O.Compound(moved)
    t0 = time.perf_counter()
    w_part, w_toi, w_nrm = comp.cast_rays_and_get_normal(rays[:sample], max_toi, solid=True, threads=threads)
    t_rays = (time.perf_counter() - t0) * (len(rays) / sample)
    cpu_frame_ms = (t_frame + t_rays) * 1e3
    # parity of a fresh first frame with the oracle frame timed above: poses, the whole pair set, every
    # manifold record, and the rays of the timed sample
    sc = pg.Scene(ctx, shapes, vel, pred, max(1 << 16, 4 * n_shapes))
    sc.set_rays(torch.from_numpy(rays).cuda(), max_toi)
    sc.step(dt, 1, use_graph=False)
    got = sc.read()
    sc.close()
    order = np.lexsort((got["pairs"][:, 1], got["pairs"][:, 0]))
    gw = M.as_words(got["manifolds"])[order]
    ww = want["manifolds"]
    live = np.arange(M.MAX_POINTS)[None, :] < ww[:, 0].astype(np.int64)[:, None] if len(ww) else None
    same = {
        "poses": bool(np.array_equal(got["poses"], want["poses"])),
        "pairs": bool(np.array_equal(got["pairs"][order], want["pairs"])),
        "manifolds": bool(len(gw) == len(ww) and np.array_equal(gw[:, :8], ww[:, :8]) and np.array_equal(
            gw[:, 8:].reshape(len(gw), M.MAX_POINTS, 10)[live], ww[:, 8:].reshape(len(ww), M.MAX_POINTS, 10)[live])),
        "rays": bool(np.array_equal(got["ray_part"][:sample], w_part) and np.array_equal(got["ray_toi"][:sample], w_toi)
                     and np.array_equal(got["ray_normal"][:sample], w_nrm)),
    }
    return {
        "workload": f"{n_shapes:,} shapes (ball/cuboid/capsule/hull 16-64 points, 25 % each, sizes log-uniform [0.25, 4]) in "
                    f"[-{extent:.0f}, {extent:.0f})^3, v U[-5, 5]^3, w U[-1, 1]^3, dt 1/60, prediction 0.1, {n_rays:,} rays "
                    "(max_toi 100) per frame",
        "metric": "frames/s", "value": round(1e3 / graph_ms, 2), "unit": "frames/s", "ms_per_frame": round(graph_ms, 4),
        "frames": frames, "graph": True, "gpu_launches": launches, "pairs_per_frame": int(npairs),
        "pairs_with_points": int((npts > 0).sum()), "ray_hits": hits,
        "rays_per_s_in_pipeline": round(len(rays) * 1e3 / graph_ms, 1),
        "stage_ms_eager_frame": stages,
        "learned_seeding": learned,
        "e2e": {"value": round(1e3 / async_ms, 2), "unit": "frames/s", "ms_per_step": round(async_ms, 3), "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(d2h_async),
                "note": "each frame (eager, not replayed) with its poses, pairs, manifold records and ray hits read into pinned host "
                        "buffers allocated once, the copies of one frame overlapped with the next (Scene.read(wait=False)); 8 frames "
                        "from the first step to the last frame's copies done",
                "sync_read": {"value": round(1e3 / e2e_ms, 2), "unit": "frames/s", "ms_per_step": round(e2e_ms, 3),
                              "d2h_bytes_per_step": int(d2h),
                              "note": "each frame stepped, then read with Scene.read (waits for the copies); mean of 4 frames after one"}},
        "cpu_baseline": {"value": round(1e3 / cpu_frame_ms, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"one oracle frame on all shapes (binned BVH rebuilt) plus rays timed on {sample} and scaled "
                                   f"to {len(rays)}; C++ restatement of parry3d f32"},
        "matches_oracle": all(same.values()),
        "matches_oracle_detail": same | {"checked": f"first frame: all {len(ww)} pairs and manifold records, the first "
                                                    f"{sample} rays, bit-exact"},
    }


def scene_learned(ctx, stream, shapes, vel, rays, pred, dt, max_toi, cap, frames, warmup, flush, state, plain_ms, plain_stats,
                  plain_manifolds_ms) -> dict:
    """The frame pipeline with the network seeding the polyhedral pairs that hold no cached normal
    (new pairs): the network is trained on the final GJK directions of the polyhedral pairs of a
    plain frame (`state`), then a fresh scene runs the same frames with seeding on (the features and
    the tcgen05 inference inside each frame's graph) and is compared with the plain run at the same
    frame: frame time, the last frame's GJK iterations and seeded pairs, the eager manifold stage."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300.shapes import BALL, CUBOID, CAPSULE

    t = shapes.arrays()[0]
    pairs = state["pairs"]
    ta, tb = t[pairs[:, 0]], t[pairs[:, 1]]
    poly = (ta != BALL) & (tb != BALL) & ~((ta == tb) & ((ta == CUBOID) | (ta == CAPSULE)))
    p_tr = np.ascontiguousarray(pairs[poly])
    now = shapes.with_poses(state["poses"])
    labels = np.zeros((len(p_tr), 3), np.float32)
    pg.contacts(ctx, now, p_tr, pred, final_dirs=labels)
    labels /= np.maximum(np.linalg.norm(labels, axis=1, keepdims=True), 1e-12)
    mlp = pg.WarmStartMLP(ctx, seed=7)
    f_tr = torch.from_numpy(np.ascontiguousarray(mlp.features(now, p_tr))).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mlp.train(f_tr, torch.from_numpy(labels).cuda(), epochs=4, batch=8192, lr=2e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del f_tr
    sc = pg.Scene(ctx, shapes, vel, pred, cap)
    sc.set_rays(torch.from_numpy(rays).cuda(), max_toi)
    sc.set_mlp(mlp)
    sc.step(dt, 2 * max(1, (warmup + 1) // 2), use_graph=True)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.zero_()
    a.record(stream)
    sc.step(dt, frames, use_graph=True)
    b.record(stream)
    torch.cuda.synchronize()
    learned_ms = a.elapsed_time(b) / frames
    st = sc.stats()
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_timing()
    sc.step(dt, 1, use_graph=False)
    ms, n = ctx.kernel_time("scene_manifolds")
    ctx.enable_kernel_timing(False)
    sc.close()
    return {
        "ms_per_frame": round(learned_ms, 4), "plain_ms_per_frame": round(plain_ms, 4),
        "frame_time_ratio_plain_over_learned": round(plain_ms / learned_ms, 4),
        "last_frame": {"seeded_pairs": st["seeded_pairs"], "gjk_iters": {"plain": plain_stats["gjk_iters"], "learned": st["gjk_iters"]},
                       "epa_iters": {"plain": plain_stats["epa_iters"], "learned": st["epa_iters"]}},
        "manifolds_stage_ms_eager": {"plain": plain_manifolds_ms, "learned": round(ms / max(n, 1), 4)},
        "train": {"pairs": int(len(p_tr)), "epochs": 4, "seconds": round(train_s, 2),
                  "labels": "final GJK directions of the plain frame's polyhedral pairs"},
    }


def learned_section(ctx, stream, dev_shapes, dev_pairs, n_eval: int, n_train: int, steps: int, flush) -> dict:
    """Learned warm start: train the MLP on the plain GJK/EPA's final directions of `n_train`
    held-out-seed hull pairs, then compare plain and learned init directions on the evaluation
    pairs (the contacts section's pairs): mean iterations, pairs/s (MLP inference included in the
    learned timing), and agreement of the answers."""
    import numpy as np
    import torch
    import parry_gb300 as pg
    from parry_gb300 import workloads as W

    s_tr, p_tr = W.hull_pairs(n_train, seed=0x51AB1E)
    t, prm, pos, pool = s_tr.arrays()
    dtr = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (t.view(np.int32), prm, pos, pool))
    dptr = torch.from_numpy(p_tr.view(np.int32)).cuda()
    labels = torch.empty((n_train, 3), dtype=torch.float32, device="cuda")
    pg.contacts(ctx, dtr, dptr, 0.0, final_dirs=labels)
    labels = labels / labels.norm(dim=1, keepdim=True).clamp_min(1e-12)
    mlp = pg.WarmStartMLP(ctx, seed=7)
    f_tr = mlp.features(dtr, dptr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = mlp.train(f_tr, labels, epochs=4, batch=8192, lr=2e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del dtr, dptr, f_tr, labels
    has = torch.empty(n_eval, dtype=torch.uint8, device="cuda")
    res = torch.empty((n_eval, 13), dtype=torch.float32, device="cuda")
    has_l = torch.empty_like(has)
    res_l = torch.empty_like(res)

    def plain():
        pg.contacts(ctx, dev_shapes, dev_pairs, 0.0, out=(has, res))

    def learned():
        f = mlp.features(dev_shapes, dev_pairs)
        d = mlp.predict(f)
        pg.contacts(ctx, dev_shapes, dev_pairs, 0.0, init_dirs=d, out=(has_l, res_l))

    out = {}
    for name, fn in (("plain", plain), ("learned", learned)):
        fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        out[name] = sum(a.elapsed_time(b) for a, b in ev) / steps
    # stage split of the learned step: features, fused tcgen05 inference
    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_timing()
    for _ in range(steps):
        f = mlp.features(dev_shapes, dev_pairs)
        d = mlp.predict(f)
    torch.cuda.synchronize()
    inf_ms, inf_n = ctx.kernel_time("mlp_predict")
    ctx.enable_kernel_timing(False)
    ev_f = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    ev_f[0].record(stream)
    for _ in range(steps):
        f = mlp.features(dev_shapes, dev_pairs)
    ev_f[1].record(stream)
    torch.cuda.synchronize()
    feat_ms = ev_f[0].elapsed_time(ev_f[1]) / steps
    inf_ms = inf_ms / max(inf_n, 1)
    mlp_flops = 2 * (48 * 128 + 3 * 128 * 128 + 128 * 3)
    peak_tc, peak_kind = measured_peak_bf16()
    tflops = mlp_flops * n_eval / (inf_ms / 1e3) / 1e12
    _, _, st_p = pg.contacts(ctx, dev_shapes, dev_pairs, 0.0, out=(has, res), want_stats=True)
    _, _, st_l = pg.contacts(ctx, dev_shapes, dev_pairs, 0.0, init_dirs=d, out=(has_l, res_l), want_stats=True)
    # the ceiling of any predictor: the exact direction the plain run ends with, as init_dir
    best = torch.empty((n_eval, 3), dtype=torch.float32, device="cuda")
    pg.contacts(ctx, dev_shapes, dev_pairs, 0.0, final_dirs=best)
    best = best / best.norm(dim=1, keepdim=True).clamp_min(1e-30)
    _, _, st_b = pg.contacts(ctx, dev_shapes, dev_pairs, 0.0, init_dirs=best, out=(has_l, res_l), want_stats=True)
    _, _, st_l = pg.contacts(ctx, dev_shapes, dev_pairs, 0.0, init_dirs=d, out=(has_l, res_l), want_stats=True)
    hp, hl = has.cpu().numpy(), has_l.cpu().numpy()
    both = (hp == 1) & (hl == 1)
    dd = np.abs(res.cpu().numpy()[both, 12] - res_l.cpu().numpy()[both, 12])
    ip = (st_p["gjk_iters"]) / n_eval
    il = (st_l["gjk_iters"]) / n_eval
    return {
        "train_pairs": n_train, "eval_pairs": n_eval, "train_seconds": round(train_s, 3),
        "loss_per_epoch": [round(float(x), 5) for x in losses],
        "mean_gjk_iterations": {"plain": round(ip, 4), "learned": round(il, 4), "ratio": round(ip / il, 4),
                                "exact_final_direction": round(st_b["gjk_iters"] / n_eval, 4),
                                "ceiling_ratio": round(st_p["gjk_iters"] / st_b["gjk_iters"], 4)},
        "mean_gjk_plus_epa_iterations": {
            "plain": round((st_p["gjk_iters"] + st_p["epa_iters"]) / n_eval, 4),
            "learned": round((st_l["gjk_iters"] + st_l["epa_iters"]) / n_eval, 4),
            "exact_final_direction": round((st_b["gjk_iters"] + st_b["epa_iters"]) / n_eval, 4),
            "ratio": round((st_p["gjk_iters"] + st_p["epa_iters"]) / (st_l["gjk_iters"] + st_l["epa_iters"]), 4)},
        "mlp_stage_ms": {"features": round(feat_ms, 4), "inference": round(inf_ms, 4)},
        "mlp_inference_roofline": {"bound": "tensor", "kernel": "k_mlp_infer_tc (tcgen05.mma, TMEM)", "achieved": round(tflops, 2),
                                   "peak": peak_tc, "unit": "TFLOP/s", "frac": round(tflops / peak_tc, 4), "peak_source": peak_kind,
                                   "flops_per_pair": mlp_flops},
        "pairs_per_s": {"plain": round(n_eval / (out["plain"] / 1e3), 1), "learned": round(n_eval / (out["learned"] / 1e3), 1),
                        "ratio": round(out["plain"] / out["learned"], 4)},
        "ms_per_step": {"plain": round(out["plain"], 4), "learned_incl_mlp": round(out["learned"], 4)},
        "answers": {"has_contact_agreement": round(float((hp == hl).mean()), 6),
                    "depth_abs_diff_p99": float(np.quantile(dd, 0.99)) if dd.size else 0.0,
                    "depth_abs_diff_max": float(dd.max()) if dd.size else 0.0},
        "mlp_flops_per_pair": mlp_flops,
    }


def summarize(line: dict) -> dict:
    """One short entry per section (throughput, unit, parity flag, main ratios), placed last in the
    JSON line so that a reader of the output's tail sees every section's headline numbers."""
    def pick(sec, *keys):
        if not isinstance(sec, dict):
            return None
        out = {}
        for k in keys:
            v = sec
            for part in k.split("."):
                v = v.get(part) if isinstance(v, dict) else None
            if v is not None:
                out[k.replace(".", "_")] = v
        return out

    return {
        "rays": {"value": line["value"], "unit": line["unit"], "e2e": line["e2e"]["value"],
                 "roofline_frac": line["roofline"]["frac"], "cpu": line["cpu_baseline"]["value"]},
        "contacts": pick(line.get("contacts"), "value", "unit", "kernel_ms", "matches_oracle_on_sample", "e2e.value",
                         "cpu_baseline.value", "dram_bytes_per_pair", "mixed_shapes.value"),
        "learned": pick(line.get("learned_warm_start"), "mean_gjk_iterations.ratio", "mean_gjk_iterations.ceiling_ratio",
                        "mean_gjk_plus_epa_iterations.ratio", "pairs_per_s.ratio", "mlp_inference_roofline.achieved",
                        "answers.has_contact_agreement"),
        "manifolds": pick(line.get("manifolds"), "value", "unit", "matches_oracle_on_sample", "e2e.value"),
        "frame_pipeline": pick(line.get("frame_pipeline"), "value", "unit", "matches_oracle", "e2e.value", "cpu_baseline.value",
                               "learned_seeding.frame_time_ratio_plain_over_learned", "learned_seeding.last_frame.seeded_pairs"),
        "broadphase": pick(line.get("broadphase"), "value", "unit", "matches_oracle"),
        "shape_cast": pick(line.get("shape_cast"), "value", "unit", "matches_oracle_on_sample"),
        "trimesh_contacts": pick(line.get("trimesh_contacts"), "value", "unit", "matches_oracle_on_sample"),
        "hull_build": pick(line.get("hull_build"), "value", "unit", "matches_host_builder_on_sample"),
        "host_link": line.get("host_link"),
    }


def run_reference(args) -> int:
    world, rank, local = dist_info()
    if rank != 0:
        return 0
    from parry_gb300 import workloads as W
    from oracle import build as ob
    ob.build()
    from oracle import oracle as O
    v, i = W.terrain_mesh()
    rays = W.terrain_rays(args.n_rays)
    threads = os.cpu_count() or 1
    m = O.TriMesh(v, i, "f32")
    for _ in range(args.warmup):
        m.cast_rays_and_get_normal(rays, MAX_TOI, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m.cast_rays_and_get_normal(rays, MAX_TOI, threads=threads)
    dt = time.perf_counter() - t0
    ms = dt / args.steps * 1e3
    value = args.n_rays / (ms / 1e3) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(1, args.n_rays),
            "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"the full workload ({args.n_rays} rays) per step; C++ restatement of parry3d "
                                       f"0.25 f32 (binned BVH, find_best), std::thread over {threads} threads"},
            "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "parry3d itself is Rust and cannot be built here (no cargo/rustc); the oracle port stands in"}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args) -> int:
    import numpy as np
    import torch

    world, rank, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from parry_gb300 import _build
    _build.build()
    import parry_gb300 as pg
    from parry_gb300 import workloads as W

    n = args.n_rays
    v, i = W.terrain_mesh()
    # one batch of world x n rays; this rank casts its contiguous range (parry_gb300.sharding), the
    # mesh and BVH replicated on every rank
    from parry_gb300 import sharding
    r0, r1 = sharding.ray_ranges(n * world, world)[rank]
    rays_h = W.terrain_rays(n * world)[r0:r1] if world > 1 else W.terrain_rays(n)
    fixed = args.ray_sort is not None
    ctx = pg.Context(device=local, sort_rays=fixed and args.ray_sort >= 0, ray_sort_key=max(args.ray_sort or 0, 0))
    # One explicit stream shared by the library and the timing events (torch's default stream
    # handle is 0, which the library would map to its own stream).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    mesh = pg.TriMesh(ctx, v, i)
    rays_d = torch.from_numpy(rays_h).cuda()
    feat = torch.empty(n, dtype=torch.int32, device="cuda")
    toi = torch.empty(n, dtype=torch.float32, device="cuda")
    nrm = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # launch configuration: tuned on the first 262,144 rays unless fixed on the command line
    tune = None
    if not fixed:
        t0 = time.perf_counter()
        chosen = mesh.autotune(rays_d[: min(n, 262144)], MAX_TOI, reps=3)
        tune = {"chosen": {k: chosen[k] for k in ("sort_rays", "ray_sort_key", "ray_traversal", "ray_block", "ray_refill")},
                "sample_rays": min(n, 262144), "seconds": round(time.perf_counter() - t0, 3)}

    def step():
        mesh.cast_rays_and_get_normal(rays_d, MAX_TOI, out=(feat, toi, nrm))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    ctx.enable_kernel_timing(True)
    ctx.reset_kernel_timing()
    launches0 = ctx.kernel_launches
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        step()
        ends[k].record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    launches = ctx.kernel_launches - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(step_ms) / len(step_ms)
    k_ms, k_n = ctx.kernel_time("trimesh_rays")
    s_ms, s_n = ctx.kernel_time("ray_sort")
    ctx.enable_kernel_timing(False)
    ms = reduce_max(ms, world)
    value = world * n / (ms / 1e3) / 1e6

    # e2e: the same public call with pinned host buffers (H2D rays, D2H results inside the region)
    rays_p = torch.from_numpy(rays_h).pin_memory()
    feat_p = torch.empty(n, dtype=torch.int32, pin_memory=True)
    toi_p = torch.empty(n, dtype=torch.float32, pin_memory=True)
    nrm_p = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    for _ in range(2):
        mesh.cast_rays_and_get_normal(rays_p, MAX_TOI, out=(feat_p, toi_p, nrm_p))
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mesh.cast_rays_and_get_normal(rays_p, MAX_TOI, out=(feat_p, toi_p, nrm_p))
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = statistics.mean(e2e_ms)
    e2e = reduce_max(e2e, world)
    e2e_value = world * n / (e2e / 1e3) / 1e6
    same = bool(np.array_equal(feat_p.numpy(), feat.cpu().numpy()))
    # the same call staged through device copies (ray_host_access = 2; the default above reads the
    # pinned rays and writes the results in place over the coherent host link), same tuned
    # configuration
    cfg_ip = dict(ctx.config)
    cfg_ip["ray_host_access"] = 2
    ctx_ip = pg.Context(**cfg_ip)
    ctx_ip.set_stream(stream.cuda_stream)
    mesh_ip = pg.TriMesh(ctx_ip, v, i)
    for _ in range(2):
        mesh_ip.cast_rays_and_get_normal(rays_p, MAX_TOI, out=(feat_p, toi_p, nrm_p))
    ip_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mesh_ip.cast_rays_and_get_normal(rays_p, MAX_TOI, out=(feat_p, toi_p, nrm_p))
        ip_ms.append((time.perf_counter() - t0) * 1e3)
    ip = statistics.mean(ip_ms)
    ip = reduce_max(ip, world)
    same_ip = bool(np.array_equal(feat_p.numpy(), feat.cpu().numpy()) and np.array_equal(toi_p.numpy(), toi.cpu().numpy()))
    e2e_staged = {"value": round(world * n / (ip / 1e3) / 1e6, 3), "unit": "Mrays/s", "ms_per_step": round(ip, 4),
                  "h2d_bytes_per_step": int(rays_p.numel() * 4), "d2h_bytes_per_step": int(n * 20), "matches_device_run": same_ip,
                  "how": "staged: chunked cudaMemcpyAsync uploads / downloads over two streams around the traversal "
                         "(ray_host_access=2)"}
    mesh_ip.close()
    ctx_ip.close()
    link_before = host_link_rates(stream)
    contacts = None
    learned = None
    manifolds = None
    scene = None
    if args.manifold_pairs > 0:
        manifolds = manifolds_section(ctx, stream, args.steps, args.warmup, args.manifold_pairs, flush)
    if args.scene_frames > 0:
        scene = scene_section(ctx, stream, args.scene_frames, args.warmup, flush, args.scene_shapes, args.scene_rays)
    trimesh_contacts = None
    if args.terrain_shapes > 0:
        trimesh_contacts = trimesh_contacts_section(ctx, stream, args.steps, args.warmup, args.terrain_shapes, flush)
        trimesh_contacts["fix_internal_edges"] = trimesh_contacts_section(ctx, stream, args.steps, args.warmup, args.terrain_shapes,
                                                                          flush, fix=True, sample=1024)
    hull_build = None
    if args.hull_clouds > 0:
        hull_build = hull_build_section(ctx, args.steps, args.hull_clouds)
    shape_cast = None
    if args.cast_pairs > 0:
        shape_cast = shape_cast_section(ctx, stream, args.steps, args.cast_pairs, flush)
    broadphase = None
    if args.broadphase_shapes > 0:
        broadphase = broadphase_section(ctx, stream, args.steps, args.warmup, args.broadphase_shapes, flush)
    if args.contact_pairs > 0:
        contacts = contacts_section(ctx, stream, args.steps, args.warmup, args.contact_pairs, flush, args.contact_epa_blocks)
        if args.train_pairs > 0:
            dev, dpairs = contacts_section.device_inputs
            learned = learned_section(ctx, stream, dev, dpairs, args.contact_pairs, args.train_pairs, args.steps, flush)
        contacts_section.device_inputs = None

    if rank == 0:
        cpu_value, stats, threads = cpu_oracle_rays(v, i, rays_h, reps=3)
        wide = stats["wide_visits"] / n
        leaves = stats["leaf_tests"] / n
        bytes_per_ray = 24 + 20 + 64 * wide + 36 * leaves
        k_avg = k_ms / max(k_n, 1)
        achieved = bytes_per_ray * n / (k_avg / 1e3) / 1e9
        peak, peak_kind = measured_peak_hbm()
        traffic = profiled_traffic("trimesh_rays_terrain")
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(world, n),
            "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s", "h2d_bytes_per_step": n * 24,
                    "d2h_bytes_per_step": n * 20, "ms_per_step": round(e2e, 4), "matches_device_path": same,
                    "how": "ray_host_access default: on a coherent host link (Grace NVLink-C2C) the traversal reads the "
                           "pinned rays and writes the pinned results in place",
                    "staged": e2e_staged},
            "roofline": {"bound": "hbm", "kernel": "k_trimesh_rays", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": peak_kind,
                         "bytes_per_ray": round(bytes_per_ray, 1),
                         "bytes_model": "24 B ray + 20 B hit + 64 B x wide-node visits + 36 B x triangle tests, visit "
                                        "counts of the f32 oracle's parry binned BVH on the same rays",
                         "oracle_wide_visits_per_ray": round(wide, 3), "oracle_tri_tests_per_ray": round(leaves, 3),
                         "kernel_ms": round(k_avg, 4), "sort_ms": round(s_ms / max(s_n, 1), 4)},
            "cpu_baseline": {"value": round(cpu_value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"the full workload ({n} rays), median of 3; C++ restatement of parry3d f32"},
            "autotune": tune if tune else {"fixed": ctx.config},
            "error_vs_f64_oracle": rays_f64_error(v, i, rays_h, feat.cpu().numpy(), toi.cpu().numpy(), nrm.cpu().numpy()),
            "gpu_launches": launches,
            "clocks": clocks,
            "contacts": contacts,
            "learned_warm_start": learned,
            "manifolds": manifolds,
            "frame_pipeline": scene,
            "broadphase": broadphase,
            "shape_cast": shape_cast,
            "trimesh_contacts": trimesh_contacts,
            "hull_build": hull_build,
            "host_link": {"before_sections": link_before, "after_sections": host_link_rates(stream)},
        }
        line["summary"] = summarize(line)
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-rays", type=int, default=N_RAYS)
    ap.add_argument("--cast-pairs", type=int, default=1 << 20, help="pairs of the shape-casting section (0 skips it)")
    ap.add_argument("--hull-clouds", type=int, default=1 << 20, help="clouds of the GPU hull-construction section (0 skips it)")
    ap.add_argument("--terrain-shapes", type=int, default=65536, help="shapes of the TriMesh contact-manifold section (0 skips it)")
    ap.add_argument("--broadphase-shapes", type=int, default=131072,
                    help="balls and cuboids of the broadphase + contact section (0 skips it)")
    ap.add_argument("--contact-pairs", type=int, default=1 << 20,
                    help="hull pairs of the GJK/EPA section (0 skips it)")
    ap.add_argument("--manifold-pairs", type=int, default=1 << 20,
                    help="ball/cuboid/capsule pairs of the contact-manifold section (0 skips it)")
    ap.add_argument("--scene-frames", type=int, default=100,
                    help="frames of the per-frame pipeline section (0 skips it)")
    ap.add_argument("--ray-sort", type=int, default=None, choices=[-1, 0, 1, 2],
                    help="fixed ray ordering before TriMesh traversal (-1 none, else the ray_sort_key mode); "
                         "default: chosen by the autotuner")
    ap.add_argument("--scene-shapes", type=int, default=262144, help="shapes of the per-frame pipeline section")
    ap.add_argument("--scene-rays", type=int, default=4194304, help="rays per frame of the per-frame pipeline section")
    ap.add_argument("--contact-epa-blocks", type=int, default=0,
                    help="contacts section: fixed EPA residency (one thread per pair, queued EPA) instead of the autotuner (0)")
    ap.add_argument("--train-pairs", type=int, default=1 << 21,
                    help="training pairs of the learned warm-start section (0 skips it)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
