"""Benchmark of the GB300 edge-collapse simplifier.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload NAME]

Default workload: meshopt_simplifyWithAttributes on the 2,097,152-triangle displaced
octahedron sphere (normals w=0.5, equirectangular UV w=1.0 with the seam split, 10% target,
target_error 5e-3). A step is one complete simplification of that mesh.

* value: input Mtris/s with the mesh resident in HBM (meshoptgpu_simplifyDevice), device
  time from CUDA events on the launching stream; L2 is flushed between steps (outside the
  events) by writing a 512 MiB buffer.
* e2e: the same metric through the drop-in C ABI (meshopt_simplifyWithAttributes) with
  pinned host buffers: host->device copies of the step's inputs, the simplification and the
  device->host copy of the result are inside the timed region.
* roofline: the dominant kernel's algorithmic bytes per launch over its CUDA-event time.
* cpu_baseline: the CPU oracle (plain-C restatement of the reference) on the same mesh,
  single thread (the reference simplifier is single-threaded), on this host.
* --impl reference: the reference's CPU implementation on this host (oracle/_ref when it was
  compiled here, else the oracle port), same metric and workload.

Multi-GPU: a single mesh does not shard without changing the result (one global greedy
order), so N>1 runs N independent replicas and reports the aggregate ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from meshoptimizer_gb300 import workloads as W  # noqa: E402

# Algorithmic bytes of the dominant kernel, kPerform (one cooperative launch per pass): the
# compulsory traffic of a pass, every array it must touch read (and written where it changes)
# once, from the per-pass counters the library reports (T triangles of the pass, V vertices of
# the buffer; a mesh of T triangles uses about T / 2 of them):
#   candidate records  42 B per evaluated candidate (pick records 16 + 16, sorted position 4,
#                      error bits 4, kind 1, decision 1): every candidate up to the stop cut
#                      is decided
#   per-vertex reset   36 B per vertex (collapse_remap 4, both parities of both marks 32)
#   positions          8 B per triangle (16 B per used vertex, read by the ring walks)
#   adjacency          24 B per triangle (three 8-byte corner records, read by the ring walks)
#   apply              144 B per committed collapse (position quadrics: source read, target read
#                      and written), plus 144 + 48 a with a attributes (attribute quadric and a
#                      gradients: source read, target read and written)
#   loop remap         16 B per vertex (loop and loopback read and written)
#   compaction         12 B per input triangle + 12 B per kept triangle
def kperform_bytes(p, vertices, next_triangles, attributes=0):
    apply = 144 + (144 + 48 * attributes if attributes else 0)
    T = p["triangles"]
    return (42 * p["evaluated"] + 36 * vertices + 8 * T + 24 * T + apply * p["done"] + 16 * vertices + 12 * T + 12 * next_triangles)


KPERFORM_BYTES_DEFINITION = ("kperform_bytes(): 42 B per evaluated candidate, 52 B per vertex (reset of remap and marks, loops), "
                             "44 B per triangle (positions, adjacency, indices in), 12 B per kept triangle, "
                             "144 B per commit + (144 + 48 a) B with a attributes")


# Per-pass byte model of the whole pass (attribute path included), for the per-phase GB/s of
# the stress line: adjacency 12 B per input triangle (indices) + 24 B per triangle (corner records
# written) + 8 B per vertex (counts and offsets); pick 12 B per triangle + 12 B per candidate
# written; rank 12 B per candidate read + 37 B per candidate written + the rows of the used
# vertices (T / 2 of them: position 16, position quadric 48, remap 4, kind 1, adjacency offsets 8,
# and 48 + 20 a with attributes); sort 8 B per candidate read twice + 13 B written; perform as
# kperform_bytes.
def pass_phase_bytes(p, vertices, next_triangles, attributes=0):
    T, Cn = p["triangles"], p["candidates"]
    rows = 77 + (48 + 20 * attributes if attributes else 0)
    return {"adjacency": 36 * T + 8 * vertices, "pick": 12 * T + 12 * Cn, "rank": 49 * Cn + rows * (T // 2),
            "sort": 29 * Cn, "perform": kperform_bytes(p, vertices, next_triangles, attributes)}


WORKLOADS = {
    "groups_4096": None,  # cluster groups: handled by bench_groups()
    "serving": None,      # request loop: handled by bench_serving()
    "cluster_lod_level": None,  # one cluster-LOD level: handled by bench_clod_level()
    "sphere_attr_2m": lambda: W.config_sphere_attr(9),
    "sphere_attr_524k": lambda: W.config_sphere_attr(8),
    "heightfield_256": W.config_heightfield_256,
    "heightfield_20k": lambda: dict(name="heightfield_101", indices=W.heightfield(101, seed=9)[0], positions=W.heightfield(101, seed=9)[1],
                                    target=W.target_count(3 * 2 * 100 * 100, 0.3), error=1e-2, options=0),
    "fractal_3163": lambda: W.config_fractal_3163(3163),
    "fractal_1024": lambda: W.config_fractal_3163(1024),
}


def load_groups(count=4096, seed=3):
    """4096 connected patches of a displaced icosphere, 200-512 triangles each, LockBorder, 50%, 2e-2."""
    meshes = []
    for idx, pos in W.sphere_patches(count, seed=seed):
        meshes.append(dict(indices=idx, positions=pos, target=W.target_count(len(idx), 0.5), error=2e-2, options=1))
    return meshes


def cpu_groups(meshes, threads):
    """Oracle port over independent groups on `threads` host threads (static work split)."""
    import concurrent.futures as cf

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    if not oracle.available("port"):
        oracle.build(with_reference=False)
    oracle.load("port")

    def work(chunk):
        return [oracle.simplify("port", m["indices"], m["positions"], m["target"], m["error"], m["options"]) for m in chunk]

    chunks = [meshes[i::threads] for i in range(threads)]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        parts = list(ex.map(work, chunks))
    dt = time.perf_counter() - t0
    out = [None] * len(meshes)
    for i, part in enumerate(parts):
        for j, r in enumerate(part):
            out[i + j * threads] = r
    return dt, out


def bench_groups(args, mg, torch, seed_offset=0):
    """Cluster groups: batched (one persistent launch) vs plain (one drop-in call per group).
    Each rank simplifies its own 4096 groups (seed + rank): replicas, weak scaling."""
    meshes = load_groups(seed=3 + seed_offset)
    tris = sum(len(m["indices"]) // 3 for m in meshes)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    d_in, descs = [], []
    for m in meshes:
        di = torch.from_numpy(m["indices"].view(np.int32)).to(dev)
        dp = torch.from_numpy(m["positions"]).to(dev)
        do = torch.empty(max(len(m["indices"]), 1), dtype=torch.int32, device=dev)
        d_in.append((di, dp, do))
        descs.append(dict(d_indices=di.data_ptr(), index_count=len(m["indices"]), d_positions=dp.data_ptr(), vertex_count=len(m["positions"]),
                          target=m["target"], error=m["error"], options=m["options"], d_destination=do.data_ptr()))
    raw_descs = descs
    descs = mg.BatchDescriptors(descs)   # built once: a step is the C-ABI batch call itself
    for _ in range(max(args.warmup, 1)):
        mg.simplify_batch_device(descs, stream=stream.cuda_stream)   # the first call autotunes the block size
    launches0 = mg.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    with ClockSampler(0) as clocks:
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            counts, errs = mg.simplify_batch_device(descs, stream=stream.cuda_stream)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    launches = mg.launch_count() - launches0
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    value = tris * args.steps / (total_ms / 1e3) / 1e6
    out_tris = int(sum(int(c) for c in counts)) // 3
    batched_out = [d_in[i][2][:int(counts[i])].cpu().numpy().view(np.uint32) for i in range(len(meshes))]

    # e2e: host arrays through meshoptgpu_simplifyBatchHost (inputs packed into pinned memory and
    # copied up, results copied back and scattered into the callers' buffers: all inside the call)
    hb = mg.HostBatch(meshes)
    for _ in range(max(args.warmup, 1)):
        hb.run()
    tt = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hb.run()
        tt += time.perf_counter() - t0
    host_res = hb.results()
    h2d = sum(m["indices"].nbytes + m["positions"].nbytes for m in meshes)
    d2h = sum(len(r[0]) * 4 for r in host_res)

    plain_gpu, exact = None, True
    if not getattr(args, "no_plain", False):
        plain_gpu, exact, plain = _groups_plain(args, mg, torch, meshes, raw_descs, stream, batched_out, host_res)
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        dt, ref = cpu_groups(meshes, threads)
        exact = exact and all(np.array_equal(a, r[0]) for a, r in zip(batched_out, ref))
        cpu = {"value": round(tris / dt / 1e6, 4), "unit": "Mtris/s", "cores": threads, "kind": "port",
               "sample": f"all {len(meshes)} groups once, independent groups split statically over {threads} threads"}
    line = _groups_line(args, mg, meshes, tris, out_tris, total_ms, tt, h2d, d2h, plain_gpu, cpu, exact, clocks, launches)
    line["error_vs_fp64_oracle"] = None
    if not args.no_cpu_baseline:
        line["error_vs_fp64_oracle"] = fp64_statement(meshes, [(len(o) // 3, float(e)) for o, e in zip(batched_out, errs)])
    return line


def _groups_plain(args, mg, torch, meshes, raw_descs, stream, batched_out, host_res):
    """plain: one drop-in call per group (host pointers), and one device-resident call per group"""
    for m in meshes[:64]:
        mg.simplify(m["indices"], m["positions"], m["target"], m["error"], m["options"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain = [mg.simplify(m["indices"], m["positions"], m["target"], m["error"], m["options"]) for m in meshes]
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    for m, dsc in zip(meshes, raw_descs):
        mg.simplify_device(dsc["d_destination"], dsc["d_indices"], dsc["index_count"], dsc["d_positions"], dsc["vertex_count"], 12,
                           m["target"], m["error"], m["options"], stream=stream.cuda_stream)
    torch.cuda.synchronize()
    t_plain_dev = time.perf_counter() - t0

    exact = all(np.array_equal(a, b[0]) for a, b in zip(batched_out, plain)) and all(np.array_equal(a[0], b[0]) for a, b in zip(host_res, plain))
    tris = sum(len(m["indices"]) // 3 for m in meshes)
    plain_gpu = {"dropin_host_mtris_s": round(tris / t_plain / 1e6, 4), "dropin_host_ms": round(1e3 * t_plain, 1),
                 "device_resident_mtris_s": round(tris / t_plain_dev / 1e6, 4), "device_resident_ms": round(1e3 * t_plain_dev, 1),
                 "calls": len(meshes)}
    return plain_gpu, exact, plain


def _groups_line(args, mg, meshes, tris, out_tris, total_ms, tt, h2d, d2h, plain_gpu, cpu, exact, clocks, launches):
    value = tris * args.steps / (total_ms / 1e3) / 1e6
    line = {
        "metric": "input Mtris/s simplified (bit-exact)", "value": round(value, 4), "unit": "Mtris/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "cluster_groups_4096", "groups": len(meshes), "input_tris": tris, "output_tris": out_tris,
                   "tris_per_group": "200-512", "options": "LockBorder", "target": "50%", "target_error": 2e-2,
                   "batch_threads_per_cta": mg.batch_threads(), "batch_smem_kib": mg.tuning(max(len(m["indices"]) for m in meshes))["batch_smem_kib"],
                   "l2": "flushed between steps (512 MiB write, outside the timed events)"},
        "e2e": {"value": round(tris * args.steps / tt / 1e6, 4), "unit": "Mtris/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": round(1e3 * tt / args.steps, 3)},
        "plain_gpu": plain_gpu,
        "cpu_baseline": cpu, "bit_exact_vs_plain_and_oracle": bool(exact), "clocks": clocks.summary(), "gpu_launches": int(launches),
    }
    return line


def bench_clod_level(args, mg, torch, levels=9, group_tris=1024):
    """One cluster-LOD level over the 2,097,152-triangle attribute sphere: 2048 groups of 1024
    triangles over one shared vertex buffer, boundary locks on the device, every group simplified
    to half with Sparse | ErrorAbsolute | Permissive (meshoptgpu_simplifyGroups, one call)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    groups, pos, attr, w, _ = W.cluster_groups(levels, group_tris)
    tris = sum(len(g) // 3 for g in groups)
    idx = np.concatenate(groups).astype(np.uint32)
    off = np.zeros(len(groups) + 1, np.uint64)
    off[1:] = np.cumsum([len(g) for g in groups])
    targets = np.array([(len(g) // 6) * 3 for g in groups], np.uint64)
    options = mg.SimplifySparse | mg.SimplifyErrorAbsolute | mg.SimplifyPermissive
    error = float(np.finfo(np.float32).max)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    di = torch.from_numpy(idx.view(np.int32)).to(dev)
    dp = torch.from_numpy(pos).to(dev)
    da = torch.from_numpy(attr).to(dev)
    do = torch.empty_like(di)
    dremap = torch.empty(len(pos), dtype=torch.int32, device=dev)
    mg.generate_position_remap_device(dremap.data_ptr(), dp.data_ptr(), len(pos), 12, stream=stream.cuda_stream)
    remap = dremap.cpu().numpy().view(np.uint32)
    locks0 = np.where(np.any(attr != attr[remap], axis=1), 2, 0).astype(np.uint8)   # protected seams, as the builder sets up
    dl = torch.from_numpy(locks0).to(dev)

    def level():
        return mg.simplify_groups_device(do.data_ptr(), di.data_ptr(), off, dp.data_ptr(), len(pos), 12, dremap.data_ptr(), dl.data_ptr(), targets,
                                         error, options, d_attributes=da.data_ptr(), attributes_stride=attr.shape[1] * 4, weights=w,
                                         stream=stream.cuda_stream)

    for _ in range(max(args.warmup, 1)):
        level()
    launches0 = mg.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    with ClockSampler(0) as clocks:
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            counts, errs = level()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    launches = mg.launch_count() - launches0
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    out = do.cpu().numpy().view(np.uint32)
    locks = dl.cpu().numpy()

    # e2e: the level's inputs from pinned host memory and its outputs back inside the timed region
    h_idx = torch.from_numpy(idx.view(np.int32)).pin_memory()
    h_pos = torch.from_numpy(pos).pin_memory()
    h_attr = torch.from_numpy(attr).pin_memory()
    h_out = torch.empty(len(idx), dtype=torch.int32).pin_memory()
    tt = 0.0
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        di.copy_(h_idx, non_blocking=True)
        dp.copy_(h_pos, non_blocking=True)
        da.copy_(h_attr, non_blocking=True)
        level()
        h_out.copy_(do, non_blocking=True)
        torch.cuda.synchronize()
        if i >= args.warmup:
            tt += time.perf_counter() - t0

    # ---- re-clusterization of the simplified groups (clusterlod's clusterize with its default
    # configuration for 128-triangle clusters: meshopt_buildMeshletsFlex, 128 vertices, 42..128
    # triangles, cone weight 0, split factor 2, then meshopt_optimizeMeshletLevel(1) on every
    # meshlet), the level's second step
    cl_params = (128, 42, 128, 0.0, 2.0)
    sgroups = [out[int(off[g]):int(off[g]) + int(counts[g])].copy() for g in range(len(groups))]
    sidx = np.concatenate(sgroups).astype(np.uint32)
    soff = np.zeros(len(groups) + 1, np.uint64)
    soff[1:] = np.cumsum([len(sg) for sg in sgroups])
    rows = mg.meshlet_rows(soff, cl_params[0], cl_params[1])
    dsi = torch.from_numpy(sidx.view(np.int32)).to(dev)
    dm = torch.empty(max(int(rows[-1]), 1) * 4, dtype=torch.int32, device=dev)
    dmv = torch.empty(max(len(sidx), 1), dtype=torch.int32, device=dev)
    dmt = torch.empty(max(len(sidx), 1), dtype=torch.uint8, device=dev)

    def clusterize():
        return mg.build_meshlets_flex_groups_device(dm.data_ptr(), dmv.data_ptr(), dmt.data_ptr(), rows, dsi.data_ptr(), soff, dp.data_ptr(),
                                                    len(pos), 12, *cl_params, optimize_level=1, stream=stream.cuda_stream)

    for _ in range(max(args.warmup, 1)):
        clusterize()
    cev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.zero_()
        cev[i][0].record(stream)
        mcounts = clusterize()
        cev[i][1].record(stream)
    torch.cuda.synchronize()
    cl_ms = sum(a.elapsed_time(b) for a, b in cev) / args.steps
    stris = len(sidx) // 3
    gm = dm.cpu().numpy().view(np.uint32).reshape(-1, 4)
    gv = dmv.cpu().numpy().view(np.uint32)
    gt = dmt.cpu().numpy()

    cpu, exact, cl_cpu, cl_exact, fp64 = None, None, None, None, None
    if not args.no_cpu_baseline:
        import concurrent.futures as cf

        import clod
        import meshlets as ML
        import oracle

        if not oracle.available("port"):
            oracle.build(with_reference=False)
        oracle.load("port")
        ref_locks = clod.lock_boundary(locks0, groups, remap)
        threads = os.cpu_count() or 1

        def work(gs):
            return [oracle.simplify("port", groups[g], pos, int(targets[g]), error, options, attributes=attr, weights=w, lock=ref_locks) for g in gs]

        chunks = [list(range(i, len(groups), threads)) for i in range(threads)]
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            parts = list(ex.map(work, chunks))
        dt = time.perf_counter() - t0
        exact = bool(np.array_equal(locks, ref_locks))
        for ch, part in zip(chunks, parts):
            for g, (o, e) in zip(ch, part):
                exact = exact and int(counts[g]) == len(o) and np.array_equal(out[int(off[g]):int(off[g]) + len(o)], o) and float(errs[g]) == e
        cpu = {"value": round(tris / dt / 1e6, 4), "unit": "Mtris/s", "cores": threads, "kind": "port",
               "sample": f"the whole level once: lockBoundary restatement, then all {len(groups)} groups split statically over {threads} threads"}
        fp64 = fp64_statement([dict(indices=groups[g], positions=pos, target=int(targets[g]), error=error, options=options, attributes=attr,
                                    weights=w, lock=ref_locks) for g in range(len(groups))],
                              [(int(counts[g]) // 3, float(errs[g])) for g in range(len(groups))])

        def cl_work(gs):
            res = []
            for g in gs:
                m, v, t = ML.build_meshlets_flex(sgroups[g], pos, *cl_params, kind="port")
                v, t = ML.optimize_meshlets(m, v, t, 1, kind="port")
                res.append((m, v, t))
            return res

        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            cl_parts = list(ex.map(cl_work, chunks))
        cdt = time.perf_counter() - t0
        cl_exact = True
        for ch, part in zip(chunks, cl_parts):
            for g, (m, v, t) in zip(ch, part):
                n = int(mcounts[g])
                ok = n == len(m) and np.array_equal(gm[int(rows[g]):int(rows[g]) + n], m)
                ok = ok and np.array_equal(gv[int(soff[g]):int(soff[g]) + len(v)], v) and np.array_equal(gt[int(soff[g]):int(soff[g]) + len(t)], t)
                cl_exact = cl_exact and ok
        cl_cpu = {"value": round(stris / cdt / 1e6, 4), "unit": "Mtris/s", "cores": threads, "kind": "port",
                  "sample": f"all {len(groups)} simplified groups once, split statically over {threads} threads"}
    h2d = idx.nbytes + pos.nbytes + attr.nbytes
    return {
        "metric": "input Mtris/s simplified (bit-exact)", "value": round(tris * args.steps / (total_ms / 1e3) / 1e6, 4), "unit": "Mtris/s",
        "ms_per_step": round(total_ms / args.steps, 3),
        "config": {"workload": f"cluster_lod_level_{tris}", "groups": len(groups), "tris_per_group": group_tris, "input_tris": tris,
                   "output_tris": int(counts.sum()) // 3, "attributes": attr.shape[1], "options": "Sparse|ErrorAbsolute|Permissive",
                   "target": "50% per group", "locks": "boundary (device) + protected seams",
                   "batch_threads_per_cta": mg.batch_threads(), "l2": "flushed between steps (512 MiB write, outside the timed events)"},
        "e2e": {"value": round(tris * args.steps / tt / 1e6, 4), "unit": "Mtris/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(idx.nbytes), "ms_per_step": round(1e3 * tt / args.steps, 3)},
        "cpu_baseline": cpu, "bit_exact_vs_oracle": exact, "error_vs_fp64_oracle": fp64, "clocks": clocks.summary(), "gpu_launches": int(launches),
        "clusterize": {"metric": "simplified Mtris/s clusterized (bit-exact)", "value": round(stris / (cl_ms / 1e3) / 1e6, 4), "unit": "Mtris/s",
                       "ms_per_step": round(cl_ms, 3), "meshlets": int(mcounts.sum()),
                       "config": {"function": "meshopt_buildMeshletsFlex per group, then meshopt_optimizeMeshletLevel(1) per meshlet (meshoptgpu_buildMeshletsFlexGroups)", "input_tris": stris,
                                  "max_vertices": cl_params[0], "min_triangles": cl_params[1], "max_triangles": cl_params[2],
                                  "cone_weight": cl_params[3], "split_factor": cl_params[4], "one_warp_per_group": True},
                       "cpu_baseline": cl_cpu, "bit_exact_vs_oracle": cl_exact},
        "level_ms": round(total_ms / args.steps + cl_ms, 3),
    }


def bench_serving(args, mg, torch):
    """Open-loop Poisson arrivals of simplify requests against the continuous-batching server and
    against the plain path (one request at a time); p50/p99 latency and Mtris/s per rate.

    Requests: seeded heightfield meshes whose triangle counts are lognormal (median 20k, sigma 1,
    clipped to [1k, 1M]), kept resident on the device as a pool of distinct meshes; each request
    picks a pool mesh, a target ratio uniform in [0.1, 0.5] and target_error 1e-2."""
    import random

    pool_size = 96
    sizes = W.lognormal_sizes(pool_size, seed=4, median=20000.0, sigma=1.0)
    dev = torch.device("cuda", 0)
    pool, pool_host = [], []
    for i, t in enumerate(sizes):
        n = int(round((t / 2) ** 0.5)) + 1
        idx, pos = W.heightfield(n, seed=1000 + i, amp=0.05)
        pool_host.append((idx, pos))
        pool.append((torch.from_numpy(idx.view(np.int32)).to(dev), torch.from_numpy(pos).to(dev), len(idx), len(pos)))
    n_req = args.requests
    rng = random.Random(7)
    reqs = []
    for r in range(n_req):
        m = rng.randrange(pool_size)
        ratio = rng.uniform(0.1, 0.5)
        reqs.append((m, W.target_count(pool[m][2], ratio)))
    out_off = np.cumsum([0] + [pool[m][2] for m, _ in reqs])
    out = torch.empty(int(out_off[-1]) + 1, dtype=torch.int32, device=dev)
    total_tris = sum(pool[m][2] // 3 for m, _ in reqs)

    def run(rate, plain):
        gaps = np.random.default_rng(int(rate) * 7 + (1 if plain else 0)).exponential(1.0 / rate, size=n_req)
        arrivals = np.cumsum(gaps)
        with mg.Server(memory_budget=40 << 30, plain=plain, large_workers=args.serve_workers, perform_blocks=args.serve_blocks,
                       large_index_count=args.serve_large, batch_workers=args.serve_batch_workers) as srv:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            tickets = []
            for i, (m, target) in enumerate(reqs):
                now = time.perf_counter() - t0
                if arrivals[i] > now:
                    time.sleep(arrivals[i] - now)
                di, dp, ni, nv = pool[m]
                tickets.append(srv.submit(di.data_ptr(), ni, dp.data_ptr(), nv, target, 1e-2, 0, out.data_ptr() + 4 * int(out_off[i])))
            res = [srv.wait(t) for t in tickets]
            t_end = time.perf_counter() - t0
            stats = srv.stats()
        lat = np.array([r[3] for r in res])
        ok = all(r[0] == mg.STATUS_OK for r in res)
        return {"rate_per_s": rate, "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                "mean_ms": round(float(lat.mean()), 3), "mtris_s": round(total_tris / t_end / 1e6, 3), "wall_s": round(t_end, 3),
                "all_ok": ok, "batches": stats["batches"], "single_mesh_runs": stats["singles"],
                "peak_reserved_gb": round(stats["peak_reserved"] / 2 ** 30, 3), "peak_in_flight": stats["peak_inflight"]}, res

    rates = [float(x) for x in args.rates.split(",")]
    served, plain = [], []
    served_res = None
    for rate in rates:
        line, res = run(rate, False)
        served.append(line)
        served_res = served_res or res
    plain_res = None
    for rate in rates[: args.plain_rates]:
        line, res = run(rate, True)
        plain.append(line)
        plain_res = plain_res or res
    # the served results equal the plain (single-mesh path, alone) results request by request
    same = plain_res is not None and all(a[1] == b[1] and a[2] == b[2] for a, b in zip(served_res, plain_res))
    # per rate that both arms ran: served delivers more input Mtris/s, and its p99 is lower
    beats = [{"rate_per_s": a["rate_per_s"], "mtris_s": a["mtris_s"] > b["mtris_s"], "p99": a["p99_ms"] < b["p99_ms"]}
             for a, b in zip(served, plain)]
    fp64 = None
    if not getattr(args, "no_cpu_baseline", False):
        # a sample of the served results (the first requests of the first rate) against the FP64 oracle
        k = min(400, n_req)
        cases = []
        for i in range(k):
            m, target = reqs[i]
            cases.append(dict(indices=pool_host[m][0], positions=pool_host[m][1], target=target, error=1e-2, options=0))
        fp64 = fp64_statement(cases, [(served_res[i][1] // 3, served_res[i][2]) for i in range(k)],
                              sample=f"the first {k} requests of the {rates[0]:g} req/s run")
    line = {
        "metric": "input Mtris/s simplified (bit-exact); p50/p99 request latency", "value": served[0]["mtris_s"], "unit": "Mtris/s", "n_gpus": 1,
        "steps": n_req, "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serving_poisson", "requests_per_rate": n_req, "pool_meshes": pool_size, "tris": "lognormal median 20k sigma 1 [1k,1M]",
                   "ratio": "U[0.1,0.5]", "target_error": 1e-2, "memory_budget_gb": 40, "request_input_tris": total_tris,
                   "single_mesh_workers": args.serve_workers, "pass_kernel_grid_cap": args.serve_blocks or 64,
                   "batch_kernel_max_index_count": args.serve_large or 30000,
                   "plain": "one request at a time on the single-mesh GPU path, in arrival order"},
        "served": served, "plain": plain, "served_equals_plain": bool(same), "served_beats_plain": beats, "error_vs_fp64_oracle": fp64,
    }
    return line


def load_workload(name):
    c = WORKLOADS[name]()
    c["tris"] = len(c["indices"]) // 3
    return c


class ClockSampler:
    """nvidia-smi clock/throttle samples every 25 ms while running; entering waits (up to 3 s)
    for the first sample, so that the sampling runs before the timed region starts, and the
    summary keeps the samples stamped between entering and leaving (all of them if none is)."""

    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.device_index = device_index
        self.proc = None
        self.lines = []
        self.t_enter = self.t_exit = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "25",
                                          "-i", str(self.device_index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.time()
            while not self.lines and self.proc.poll() is None and time.time() - t0 < 3.0:
                time.sleep(0.005)
        except (OSError, FileNotFoundError):
            self.proc = None
        self.t_enter = time.time()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self.t_exit = time.time()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = [[x.strip() for x in l.split(",")] for l in self.lines]
        rows = [f for f in rows if len(f) >= 10]

        def stamp(f):
            try:
                return time.mktime(time.strptime(f[0].split(".")[0], "%Y/%m/%d %H:%M:%S")) + float("0." + f[0].split(".")[1])
            except (ValueError, IndexError):
                return None

        inside = [f for f in rows if self.t_enter and self.t_exit and stamp(f) is not None and self.t_enter - 0.05 <= stamp(f) <= self.t_exit + 0.05]
        for f in inside or rows:
            try:
                sm.append(float(f[2]))
                mx.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def kernel_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` on `workload` from a committed ncu summary
    (profiles/traffic.json: dram__bytes_read.sum + dram__bytes_write.sum averaged over the
    captured launches, cold cache and, where captured, with the cache as the run left it), or
    None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.isfile(path):
        return None
    with open(path) as f:
        entries = json.load(f)
    for e in entries:
        if e.get("kernel") == kernel and e.get("workload") == workload:
            out = {"dram_bytes_per_launch": int(e["dram_bytes_per_launch"]), "source": e["source"]}
            if "dram_bytes_per_launch_in_run" in e:
                out["dram_bytes_per_launch_in_run"] = int(e["dram_bytes_per_launch_in_run"])
            return out
    return None


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(c, min_seconds=8.0, max_runs=4):
    """Oracle port (single thread) on the same mesh; returns (Mtris/s, runs, seconds, output, error)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    if not oracle.available("port"):
        oracle.build(with_reference=False)
    runs, t0 = 0, time.perf_counter()
    out = err = None
    while runs < max_runs and (runs == 0 or time.perf_counter() - t0 < min_seconds):
        out, err = oracle.simplify("port", c["indices"], c["positions"], c["target"], c["error"], c["options"],
                                   attributes=c.get("attributes"), weights=c.get("weights"))
        runs += 1
    dt = time.perf_counter() - t0
    return c["tris"] * runs / dt / 1e6, runs, dt, out, err


def run_reference(args):
    """--impl reference: the reference's own CPU implementation of the path on this host."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    kind = "ref" if oracle.available("ref") else "port"
    if kind == "port" and not oracle.available("port"):
        oracle.build(with_reference=False)
    c = load_workload(args.workload)
    call = lambda: oracle.simplify(kind, c["indices"], c["positions"], c["target"], c["error"], c["options"],  # noqa: E731
                                   attributes=c.get("attributes"), weights=c.get("weights"))
    for _ in range(min(args.warmup, 1)):
        call()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = c["tris"] * args.steps / total / 1e6
    line = {
        "impl": "reference", "metric": "input Mtris/s simplified (bit-exact)", "value": round(value, 4), "unit": "Mtris/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": c["name"], "input_tris": c["tris"], "target_index_count": c["target"], "target_error": c["error"],
                   "options": c["options"]},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mtris/s", "cores": 1,
                         "kind": "reference" if kind == "ref" else "port",
                         "sample": f"{args.steps} full simplifications of {c['name']} (single thread: the simplifier has no threading)"},
        "e2e": {"value": round(value, 4), "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def fp64_statement(cases, results, threads=None, sample=None):
    """The FP32 results' error stated against the FP64 oracle (the same driver in double).

    cases: dicts with indices, positions, target, error, options (and attributes, weights, lock);
    results: the GPU's (output triangles, result error) for each case, in order."""
    import concurrent.futures as cf

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    if not oracle.available("port"):
        oracle.build(with_reference=False)
    oracle.load("port")

    def one(c):
        out64, e64, _ = oracle.simplify("port", c["indices"], c["positions"], c["target"], c["error"], c["options"],
                                        attributes=c.get("attributes"), weights=c.get("weights"), lock=c.get("lock"), fp64=True)
        return len(out64) // 3, e64

    with cf.ThreadPoolExecutor(threads or os.cpu_count() or 1) as ex:
        ref = list(ex.map(one, cases))
    rel, same, t32, t64 = [], 0, 0, 0
    for (tris32, e32), (tris64, e64) in zip(results, ref):
        d = abs(float(e32) - e64)
        rel.append(d / e64 if e64 > 0 else (0.0 if d == 0 else float("inf")))
        same += int(tris32 == tris64)
        t32 += int(tris32)
        t64 += tris64
    out = {"results": len(cases), "max_relative_difference": float(max(rel)) if rel else 0.0,
           "median_relative_difference": float(statistics.median(rel)) if rel else 0.0,
           "output_tris_equal": same, "fp32_output_tris": t32, "fp64_output_tris": t64}
    if sample:
        out["sample"] = sample
    return out


def bench_single(args, mg, torch, c, dist=None, world=1, rank=0, local=0, roofline=True, e2e_leg=True, cpu_leg=True, per_pass=False):
    """One complete simplification of one mesh per step: device-resident value, roofline of the
    pass kernel, drop-in e2e, CPU baseline, bit-exactness and the FP64 statement."""
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    idx = torch.from_numpy(c["indices"].view(np.int32)).to(dev)
    pos = torch.from_numpy(c["positions"]).to(dev)
    has_attr = c.get("attributes") is not None
    attr = torch.from_numpy(c["attributes"]).to(dev) if has_attr else None
    out = torch.empty_like(idx)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    V = pos.shape[0]
    ac = attr.shape[1] if has_attr else 0
    ac_used = int(np.count_nonzero(np.asarray(c["weights"]) > 0)) if has_attr else 0

    def step():
        return mg.simplify_device(out.data_ptr(), idx.data_ptr(), idx.numel(), pos.data_ptr(), V, 12, c["target"], c["error"], c["options"],
                                  d_attributes=attr.data_ptr() if has_attr else 0, attributes_stride=4 * ac,
                                  weights=c.get("weights"), stream=stream.cuda_stream)

    for _ in range(max(args.warmup, 0)):
        n_out, err = step()
    tuned = mg.tuning(idx.numel(), ac_used)  # the first warm-up call tuned this size class's launch shape

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = mg.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            n_out, err = step()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = mg.launch_count() - launches0
    total_ms = sum(a.elapsed_time(b) for a, b in ev)

    # per-launch CUDA-event timing of the roofline kernel: the same steps replayed with the
    # host-driven pass loop (events cannot be recorded inside the device-resident loop's graph)
    k_launches = k_ms = host_loop_ms = 0
    if roofline:
        mg.set_device_loop(False)
        step()
        mg.set_kernel_profile(args.kernel)
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for i in range(args.steps):
            flush.zero_()
            kev[i][0].record(stream)
            step()
            kev[i][1].record(stream)
        torch.cuda.synchronize()
        k_launches, k_ms = mg.kernel_profile()
        mg.set_kernel_profile(None)
        mg.set_device_loop(True)
        host_loop_ms = sum(a.elapsed_time(b) for a, b in kev)
    from meshoptimizer_gb300 import replicas

    rate, secs, _ = replicas.aggregate(total_ms / 1e3, float(c["tris"] * args.steps), dist=dist, device=dev)
    total_ms = secs * 1e3
    value = rate / 1e6
    gpu_out = out[:n_out].cpu().numpy().view(np.uint32)

    # per-pass and per-phase view of one more run (not timed for the value)
    mg.set_timing(True)
    step()
    phases = mg.last_phase_times()
    passes = mg.last_pass_stats()
    pass_phases = mg.last_pass_phase_times()
    trace = mg.last_round_trace()
    mg.set_timing(False)

    # end to end through the drop-in C ABI with pinned host buffers
    e2e = None
    if e2e_leg:
        h_idx = torch.from_numpy(c["indices"].view(np.int32)).pin_memory()
        h_pos = torch.from_numpy(c["positions"]).pin_memory()
        h_attr = torch.from_numpy(c["attributes"]).pin_memory() if has_attr else None
        h_out = torch.empty(len(c["indices"]), dtype=torch.int32).pin_memory()
        n_idx, n_pos = h_idx.numpy().view(np.uint32), h_pos.numpy()
        n_attr = h_attr.numpy() if has_attr else None
        n_outb = h_out.numpy().view(np.uint32)

        def e2e_step():
            if has_attr:
                return mg.simplify_raw(n_outb, n_idx, len(n_idx), n_pos, V, 12, c["target"], c["error"], c["options"], attributes=n_attr,
                                       attributes_stride=4 * ac, weights=c["weights"], attribute_count=ac)
            return mg.simplify_raw(n_outb, n_idx, len(n_idx), n_pos, V, 12, c["target"], c["error"], c["options"])

        for _ in range(max(args.warmup, 0)):
            e2e_step()
        tt = 0.0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            n_e2e, _ = e2e_step()
            tt += time.perf_counter() - t0
        if dist:
            t = torch.tensor([tt], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            tt = float(t.item())
        assert np.array_equal(n_outb[:n_e2e], gpu_out), "drop-in and device-resident results differ"
        h2d = c["indices"].nbytes + c["positions"].nbytes + (c["attributes"].nbytes if has_attr else 0)
        d2h = n_e2e * 4
        e2e = {"value": round(world * c["tris"] * args.steps / tt / 1e6, 4), "unit": "Mtris/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": round(1e3 * tt / args.steps, 3), "host_memory": "pinned"}

        # the same calls from ordinary (pageable) numpy arrays, as most drop-in callers hold their meshes
        p_idx, p_pos = np.array(c["indices"], copy=True), np.array(c["positions"], copy=True)
        p_attr = np.array(c["attributes"], copy=True) if has_attr else None
        p_out = np.zeros(len(c["indices"]), np.uint32)

        def pageable_step():
            if has_attr:
                return mg.simplify_raw(p_out, p_idx, len(p_idx), p_pos, V, 12, c["target"], c["error"], c["options"], attributes=p_attr,
                                       attributes_stride=4 * ac, weights=c["weights"], attribute_count=ac)
            return mg.simplify_raw(p_out, p_idx, len(p_idx), p_pos, V, 12, c["target"], c["error"], c["options"])

        pageable_step()
        tp = 0.0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            n_pg, _ = pageable_step()
            tp += time.perf_counter() - t0
        assert np.array_equal(p_out[:n_pg], gpu_out), "pageable drop-in and device-resident results differ"
        e2e["pageable"] = {"value": round(world * c["tris"] * args.steps / tp / 1e6, 4), "unit": "Mtris/s",
                           "ms_per_step": round(1e3 * tp / args.steps, 3)}

    if rank != 0:
        return None

    # roofline of the selected kernel: algorithmic bytes over its measured launch time
    peak, peak_kind = measured_peak()
    roof = None
    nxt = [p["triangles"] for p in passes[1:]] + [int(n_out) // 3]
    if k_launches:
        avg_ms = k_ms / k_launches
        bytes_run = sum(kperform_bytes(p, V, t, ac_used) for p, t in zip(passes, nxt))
        bytes_per_launch = bytes_run / max(len(passes), 1)
        achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else 0
        roof = {"bound": "hbm", "kernel": args.kernel, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": None,
                "avg_launch_us": round(1e3 * avg_ms, 2), "launches": k_launches,
                "algorithmic_bytes_per_launch": int(bytes_per_launch), "unit_definition": KPERFORM_BYTES_DEFINITION,
                "share_of_step": round(k_ms / host_loop_ms, 4) if host_loop_ms else None,
                "kernel_timing": "CUDA events around every launch on its stream, over the same steps replayed with the host-driven "
                                 "pass loop (the timed steps run the device-resident loop, whose graph cannot hold events)"}
        tr = kernel_traffic(args.kernel, c["name"])
        if tr:
            roof["traffic"] = tr["dram_bytes_per_launch"]
            if "dram_bytes_per_launch_in_run" in tr:
                roof["traffic_in_run"] = tr["dram_bytes_per_launch_in_run"]
            roof["traffic_source"] = tr["source"]

    cpu = bit_exact = fp64 = None
    if cpu_leg:
        mt, runs, secs_cpu, ref_out, ref_err = cpu_baseline(c)
        bit_exact = bool(np.array_equal(ref_out, gpu_out)) and abs(ref_err - err) <= 1e-6 * max(abs(ref_err), 1e-30)
        fp64 = fp64_statement([c], [(int(n_out) // 3, err)], threads=1)
        fp64["fp32_result_error"] = err
        cpu = {"value": round(mt, 4), "unit": "Mtris/s", "cores": 1, "kind": "port",
               "sample": f"{runs} full simplification(s) of {c['name']} in {secs_cpu:.1f} s, single thread (the simplifier has no threading)"}

    line = {
        "metric": "input Mtris/s simplified (bit-exact)", "value": round(value, 4), "unit": "Mtris/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": c["name"], "input_tris": c["tris"], "output_tris": int(n_out) // 3, "target_index_count": c["target"],
                   "target_error": c["error"], "options": c["options"], "attributes": ac, "result_error": err,
                   "l2": "flushed between steps (512 MiB write, outside the timed events)", "parallelism": f"replicas{world}",
                   "autotuned": {"perform_blocks_per_sm": tuned["perform_blocks_per_sm"], "sort_items_per_thread": tuned["sort_items"]}},
        "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "bit_exact_vs_oracle": bit_exact, "error_vs_fp64_oracle": fp64,
        "clocks": clocks.summary(), "gpu_launches": int(launches),
        "phases_ms": {k: round(v, 3) for k, v in phases.items()},
        "passes": [{k: p[k] for k in ("triangles", "candidates", "evaluated", "done", "rounds", "active", "windows")} for p in passes],
        "round_trace_us": [[n, round(t, 1)] for n, t in trace[:64]],
    }
    if per_pass:
        # per pass: CUDA-event time of each phase (host-driven loop, timing on) and the phase's
        # algorithmic bytes over it
        rows = []
        for p, t, ph in zip(passes, nxt, pass_phases):
            b = pass_phase_bytes(p, V, t, ac_used)
            rows.append({"triangles": p["triangles"], "candidates": p["candidates"], "rounds": p["rounds"],
                         "ms": {k: round(v, 3) for k, v in ph.items()},
                         "gb_s": {k: round(b[k] / (ph[k] / 1e3) / 1e9, 1) if ph[k] > 0 else None for k in b},
                         "algorithmic_mb": {k: round(b[k] / 1e6, 2) for k in b}})
        line["per_pass"] = rows
        line["per_pass_definition"] = ("ms: CUDA events around each phase of each pass (host-driven pass loop); gb_s: the phase's "
                                       "algorithmic bytes (pass_phase_bytes in bench.py) over that time, against the measured "
                                       f"{peak} GB/s copy bandwidth")
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sphere_attr_2m", choices=sorted(WORKLOADS))
    ap.add_argument("--kernel", default="kPerform", help="kernel whose CUDA-event time gives the roofline line")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the groups, serving, cluster-LOD and heightfield summaries of the default line")
    ap.add_argument("--no-plain", action="store_true", help="groups: skip the separate one-call-per-group comparison leg")
    ap.add_argument("--requests", type=int, default=10000, help="serving: requests per arrival rate")
    ap.add_argument("--rates", default="500,1000,2000,4000", help="serving: Poisson arrival rates (requests/s)")
    ap.add_argument("--plain-rates", type=int, default=4, help="serving: how many of the rates also run the plain path")
    ap.add_argument("--serve-workers", type=int, default=16, help="serving: concurrent single-mesh workers")
    ap.add_argument("--serve-blocks", type=int, default=0, help="serving: pass-kernel grid cap per request (0: server default)")
    ap.add_argument("--serve-large", type=int, default=0, help="serving: index count above which requests skip the batch kernel (0: default)")
    ap.add_argument("--serve-batch-workers", type=int, default=0, help="serving: concurrent batch launches (0: default)")
    args = ap.parse_args()

    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    import meshoptimizer_gb300 as mg
    from meshoptimizer_gb300 import build as mgbuild

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    mgbuild.build()
    mg.load()
    if args.workload == "groups_4096":
        print(json.dumps(bench_groups(args, mg, torch, seed_offset=rank)))
        return
    if args.workload == "serving":
        print(json.dumps(bench_serving(args, mg, torch)))
        return
    if args.workload == "cluster_lod_level":
        print(json.dumps(bench_clod_level(args, mg, torch)))
        return
    c = load_workload(args.workload)
    line = bench_single(args, mg, torch, c, dist=dist, world=world, rank=rank, local=local, e2e_leg=not args.no_e2e,
                        cpu_leg=not args.no_cpu_baseline, per_pass=args.workload.startswith("fractal"))
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    if not args.no_extras and world == 1:
        g = bench_groups(argparse.Namespace(steps=3, warmup=3, no_cpu_baseline=args.no_cpu_baseline), mg, torch)
        line["batched_groups"] = {k: g[k] for k in ("value", "unit", "ms_per_step", "e2e", "plain_gpu", "cpu_baseline",
                                                   "bit_exact_vs_plain_and_oracle", "error_vs_fp64_oracle")}
        line["batched_groups"]["config"] = g["config"]
        sv = bench_serving(argparse.Namespace(requests=args.requests, rates=args.rates, plain_rates=args.plain_rates,
                                              serve_workers=args.serve_workers, serve_blocks=args.serve_blocks, serve_large=args.serve_large,
                                              serve_batch_workers=args.serve_batch_workers, no_cpu_baseline=args.no_cpu_baseline), mg, torch)
        line["serving"] = {k: sv[k] for k in ("served", "plain", "served_equals_plain", "served_beats_plain", "error_vs_fp64_oracle", "config")}
        cl = bench_clod_level(argparse.Namespace(steps=3, warmup=3, no_cpu_baseline=args.no_cpu_baseline), mg, torch)
        line["cluster_lod_level"] = {k: cl[k] for k in ("value", "unit", "ms_per_step", "config", "e2e", "cpu_baseline", "bit_exact_vs_oracle",
                                                        "error_vs_fp64_oracle", "clusterize", "level_ms")}
        hf = bench_single(argparse.Namespace(steps=10, warmup=3, kernel=args.kernel), mg, torch, load_workload("heightfield_256"),
                          local=local, e2e_leg=True, cpu_leg=not args.no_cpu_baseline)
        line["heightfield_256"] = {k: hf[k] for k in ("value", "unit", "ms_per_step", "config", "e2e", "roofline", "cpu_baseline",
                                                      "bit_exact_vs_oracle", "error_vs_fp64_oracle", "phases_ms", "passes")}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
