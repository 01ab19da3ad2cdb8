#!/usr/bin/env python3
"""Benchmark of the two voxel hot paths on GB300.

Headline step (value): one 1920x1080 frame of the 1024^3 sparse terrain scene
(8^3 bricks under a 128^3 pointer grid, ~15% solid, uint16 materials),
primary rays plus one shadow ray per hit towards normalize(0.3, 0.5, 0.8),
FP32, one plain per-view launch; metric Mrays/s = (primary + shadow rays) / s.
roofline.l2 gives the same algorithmic bytes against the L2 read bandwidth
measured in the run (the raymarch's fetches hit in L2).
Also reported on the same line:
  mesh        batched meshing of 4096 standalone 32^3 uint16 chunks (Gvox/s,
              persistent kernel vs one launch per chunk, directly and replayed
              as a CUDA graph, HBM roofline, CPU oracle on the host cores
              with a bit-exact check); mesh.uint8: the same chunks as uint8
              and the 256^3 uint8 grid of the small plain case;
  served      the served raymarch stream: p50/p99 latency and Mrays/s at the
              offered load, capacity (requests submitted at once) and the
              plain form (one launch per request, waited for);
  served_edit the served edit+remesh+render stream: p50/p99, capacity and
              plain form in requests/s; gvox_meshed_s_wall = voxels of the
              dirty chunks per second of the run, gvox_meshed_s_busy = the
              same per second of request processing (edit, remesh and render
              together, not the mesher alone);
  downstream  device scene build, quad -> vertex expansion and the erosion
              pyramid, with their rooflines;
  cpu_baseline the CPU oracle on the same frame (all host cores, and one).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 runs independent replicas, one per rank and GPU (the path has no
exchange step): value = rays of all ranks / the slowest rank's time.  Under
torchrun WORLD_SIZE must equal N; run directly, the script starts the N
replica processes itself (gloo on 127.0.0.1 for the barrier and the max).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s + meshed Gvox/s; served p50/p99 vs per-call launch, bit-exact on 1 GB300"
FRAME_W, FRAME_H = 1920, 1080
CAM_ORIGIN = (-300.0, -200.0, 800.0)
CAM_TARGET = (512.0, 512.0, 512.0)
L2_FLUSH_BYTES = 512 << 20
MESH_CHUNKS = 4096


def ncu_traffic(kernel):
    """DRAM bytes (read + write) of one launch of `kernel` from the committed
    ncu capture summary, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_dram_bytes.json")) as f:
            d = json.load(f)[kernel]
        return int(d["dram_bytes_read"]) + int(d["dram_bytes_write"])
    except Exception:
        return None


def ncu_field(kernel, key):
    """A figure of one kernel from the committed ncu capture summary, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_dram_bytes.json")) as f:
            return json.load(f)[kernel][key]
    except Exception:
        return None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def spawn_replicas(n: int) -> int:
    """Runs this command as n replica processes (RANK = LOCAL_RANK = 0..n-1,
    rendezvous on 127.0.0.1) when it was not launched by torchrun; rank 0
    prints the line.  Returns the worst exit code."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + sys.argv[1:], env=env))
    rcs = [p.wait() for p in procs]
    return max(rcs, key=abs)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # replicas only: gloo for the barrier and the max
        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def count_rays(hits) -> int:
    # every pixel casts a primary ray; a shadow ray was traced iff it took steps
    return int(hits.shape[0] + np.count_nonzero(hits["shadow_steps"]))


# ------------------------------------------------------------------ our arm

def bench_raymarch(ctx, meso, steps, warmup, dist, clocks):
    t = meso.terrain_preset("scene1024")
    scene = ctx.scene_from_terrain(t)
    cam = meso.camera(CAM_ORIGIN, CAM_TARGET, FRAME_W, FRAME_H)
    flush = ctx.alloc(L2_FLUSH_BYTES)
    out = ctx.alloc(FRAME_W * FRAME_H * 24)
    for _ in range(warmup):
        ctx.raymarch(scene, cam, out=out, download=False)
    ctx.sync()
    hits = out.download(meso.HIT_DTYPE, FRAME_W * FRAME_H)
    rays = count_rays(hits)
    evs = [(ctx.event(), ctx.event()) for _ in range(steps)]
    launches0 = ctx.kernel_launches
    barrier(dist)
    ctx.sync()
    with clocks:
        for a, b in evs:
            flush.zero()  # L2 flush outside the event pair
            ctx.record(a)
            ctx.raymarch(scene, cam, out=out, download=False)
            ctx.record(b)
        ctx.sync()
    launches = ctx.kernel_launches - launches0
    barrier(dist)
    times = [ctx.elapsed_ms(a, b) for a, b in evs]
    ms = sum(times) / len(times)
    # end to end through the host-buffer entry point: camera in, hits back to pinned memory
    pinned = ctx.pinned(FRAME_W * FRAME_H * 24)
    for _ in range(2):
        ctx.raymarch_host(scene, cam, out_ptr=pinned.ptr)
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.raymarch_host(scene, cam, out_ptr=pinned.ptr)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / steps
    e2e_hits = pinned.view(meso.HIT_DTYPE, FRAME_W * FRAME_H)
    assert np.array_equal(e2e_hits.view(np.uint8), hits.view(np.uint8)), "host entry point disagrees"
    fetches, bricks, nhits, traversals = ctx.raymarch_stats(scene, cam, out=out)
    algo_bytes = 4 * fetches + 64 * bricks + 2 * nhits + 24 * FRAME_W * FRAME_H
    info = scene.info()
    solid = scene.count_solid()
    return {
        "scene": scene, "cam": cam, "hits": hits, "rays": rays, "ms": ms, "times": times,
        "launches": launches, "e2e_ms": e2e_ms, "algo_bytes": algo_bytes,
        "counts": {"pointer_fetches": fetches, "bricks_entered": bricks, "hits": nhits, "traversals": traversals},
        "bricks": int(info.n_bricks), "scene_bytes": int(info.device_bytes),
        "occupancy": solid / float(t.nx * t.ny * t.nz),
    }


def bench_mesh(ctx, meso, steps, warmup):
    data, _ = ctx.generate_chunks_u16(MESH_CHUNKS, seed0=1)
    cap = MESH_CHUNKS * 8192
    qbuf = ctx.alloc(cap * 8)
    cnt = ctx.alloc(8)
    flush = ctx.alloc(L2_FLUSH_BYTES)
    src = meso.MeshSource()
    src.kind = meso.SRC_CHUNKS_U16
    src.d_data = data.ptr
    out = meso.MeshOutput(qbuf.ptr, cap, cnt.ptr, None)
    L = meso._lib
    import ctypes

    def run(per_launch=False):
        fn = L.meso_mesh_chunks_per_launch if per_launch else L.meso_mesh_chunks
        meso._check(fn(ctx.handle, ctypes.byref(src), None, MESH_CHUNKS, ctypes.byref(out), None))

    for _ in range(warmup):
        run()
    ctx.sync()
    total = ctypes.c_uint64()
    meso._check(L.meso_mesh_check(ctx.handle, ctypes.byref(out), None, ctypes.byref(total)))
    quads = int(total.value)
    evs = [(ctx.event(), ctx.event()) for _ in range(steps)]
    for a, b in evs:
        flush.zero()
        ctx.record(a)
        run()
        ctx.record(b)
    ctx.sync()
    times = [ctx.elapsed_ms(a, b) for a, b in evs]
    ms = sum(times) / len(times)
    # plain form: one launch per chunk
    run(per_launch=True)
    ctx.sync()
    a, b = ctx.event(), ctx.event()
    flush.zero()
    ctx.record(a)
    run(per_launch=True)
    ctx.record(b)
    ctx.sync()
    ms_plain = ctx.elapsed_ms(a, b)
    meso._check(L.meso_mesh_check(ctx.handle, ctypes.byref(out), None, ctypes.byref(total)))
    assert int(total.value) == quads
    # the plain form captured once into a CUDA graph (4096 kernel nodes) and replayed
    st = ctx.stream()

    def plain_on_stream():
        meso._check(L.meso_mesh_chunks_per_launch(ctx.handle, ctypes.byref(src), None, MESH_CHUNKS,
                                                  ctypes.byref(out), st))

    g = ctx.capture(plain_on_stream, st)
    g.launch(st)
    ctx.sync(st)
    ga, gb = ctx.event(), ctx.event()
    flush.zero(st)
    ctx.record(ga, st)
    g.launch(st)
    ctx.record(gb, st)
    ctx.sync(st)
    ms_graph = ctx.elapsed_ms(ga, gb)
    meso._check(L.meso_mesh_check(ctx.handle, ctypes.byref(out), st, ctypes.byref(total)))
    assert int(total.value) == quads
    g.destroy()
    vox = MESH_CHUNKS * 32768
    algo = MESH_CHUNKS * 65536 + 8 * quads
    # end to end through the host entry point: the chunks in page-locked host
    # memory, the quads written back into page-locked host memory, every step
    h_in = ctx.pinned(MESH_CHUNKS * 65536)
    meso._check(L.meso_memcpy_d2h(ctx.handle, h_in.ptr, data.ptr, MESH_CHUNKS * 65536, None))
    ctx.sync()
    h_out = ctx.pinned(cap * 8)

    def host_call():
        meso._check(L.meso_mesh_host(ctx.handle, meso.SRC_CHUNKS_U16, h_in.ptr, MESH_CHUNKS, 0, 0, None,
                                     MESH_CHUNKS, h_out.ptr, cap, ctypes.byref(total)))

    for _ in range(2):
        host_call()
    t0 = time.perf_counter()
    for _ in range(steps):
        host_call()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / steps
    assert int(total.value) == quads
    dev_q = np.sort(qbuf.download(np.uint64, quads))
    e2e_exact = bool(np.array_equal(np.sort(h_out.view(np.uint64, quads)), dev_q))
    h_in.free()
    h_out.free()
    return {"ms": ms, "ms_plain": ms_plain, "quads": quads, "gvox_s": vox / (ms * 1e6),
            "gvox_s_plain": vox / (ms_plain * 1e6), "gvox_s_graph": vox / (ms_graph * 1e6),
            "algo_bytes": algo, "data": data, "qbuf": qbuf, "e2e_ms": e2e_ms, "e2e_exact": e2e_exact}


def bench_mesh_u8(ctx, meso, m, steps):
    """The 8-bit sources: the same 4096 chunks with materials folded into
    1..255, and the small dense case, a 256^3 uint8 grid meshed as 512 chunks with
    their neighbours' faces, batched and one launch per chunk."""
    import ctypes
    L = meso._lib
    h = m["data"].download(np.uint16)
    data = ctx.to_device(np.where(h > 0, 1 + (h.astype(np.uint32) % 255), 0).astype(np.uint8))
    del h
    cnt = ctx.alloc(8)
    flush = ctx.alloc(L2_FLUSH_BYTES)
    total = ctypes.c_uint64()

    def timed(src, coords, n, per_launch=False, reps=steps):
        out = meso.MeshOutput(m["qbuf"].ptr, MESH_CHUNKS * 8192, cnt.ptr, None)
        fn = L.meso_mesh_chunks_per_launch if per_launch else L.meso_mesh_chunks
        cp = coords.ptr if coords is not None else None
        for _ in range(3):
            meso._check(fn(ctx.handle, ctypes.byref(src), cp, n, ctypes.byref(out), None))
        evs = [(ctx.event(), ctx.event()) for _ in range(reps)]
        for a, b in evs:
            flush.zero()
            ctx.record(a)
            meso._check(fn(ctx.handle, ctypes.byref(src), cp, n, ctypes.byref(out), None))
            ctx.record(b)
        ctx.sync()
        meso._check(L.meso_mesh_check(ctx.handle, ctypes.byref(out), None, ctypes.byref(total)))
        return sum(ctx.elapsed_ms(a, b) for a, b in evs) / reps, int(total.value)

    src = meso.MeshSource()
    src.kind = meso.SRC_CHUNKS_U8
    src.d_data = data.ptr
    ms, quads = timed(src, None, MESH_CHUNKS)
    hbm = peaks()[0]
    algo = MESH_CHUNKS * 32768 + 8 * quads
    ach = algo / (ms * 1e6)
    res = {"workload": f"the {MESH_CHUNKS} chunks as uint8 (materials folded into 1..255)",
           "gvox_s": round(MESH_CHUNKS * 32768 / (ms * 1e6), 2), "ms": round(ms, 4), "quads": quads,
           "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                        "frac": round(ach / hbm, 4), "algorithmic_bytes_per_launch": algo,
                        "kernel": "mesh_kernel<CHUNKS_U8>"}}
    del data
    g = ctx.generate_dense_u8(256, 256, 256, seed=1)
    coords = ctx.to_device(np.array([(x, y, z) for z in range(8) for y in range(8) for x in range(8)], np.int32))
    gs = meso.MeshSource()
    gs.kind = meso.SRC_GRID_U8
    gs.d_data = g.ptr
    gs.nx = gs.ny = gs.nz = 256
    ms_b, q_b = timed(gs, coords, 512)
    ms_p, q_p = timed(gs, coords, 512, per_launch=True, reps=max(1, min(steps, 3)))
    assert q_b == q_p
    res["dense_256"] = {"workload": "256^3 uint8 value-noise grid (3 octaves, seed 1), 512 chunks with neighbour faces",
                        "gvox_s": round(512 * 32768 / (ms_b * 1e6), 2), "ms": round(ms_b, 4), "quads": q_b,
                        "per_chunk_launch_gvox_s": round(512 * 32768 / (ms_p * 1e6), 3),
                        "batched_over_per_launch": round(ms_p / ms_b, 2)}
    res["dense_256"]["ray"] = bench_ray_dense256(ctx, meso, g, steps, flush)
    return res


CFG1_ORIGIN, CFG1_TARGET, CFG1_W, CFG1_H = (-160.0, -96.0, 384.0), (128.0, 128.0, 128.0), 640, 360


def bench_ray_dense256(ctx, meso, grid, steps, flush):
    """The small plain case's raymarch: the 256^3 uint8 grid as a brick map
    (built on the device from the generated grid), one 640x360 pinhole camera
    (60 degree vertical FOV) outside the grid aimed at its centre, primary
    rays to the first hit; one launch per step, L2 flushed between steps.
    The oracle DDA traces the same frame on all host cores beside it."""
    import oracle
    scene = ctx.scene_from_grid(meso.SRC_GRID_U8, grid, (256, 256, 256))
    cam = meso.camera(CFG1_ORIGIN, CFG1_TARGET, CFG1_W, CFG1_H)
    out = ctx.alloc(CFG1_W * CFG1_H * 24)
    for _ in range(3):
        ctx.raymarch(scene, cam, shadow=False, out=out, download=False)
    evs = [(ctx.event(), ctx.event()) for _ in range(steps)]
    for a, b in evs:
        flush.zero()
        ctx.record(a)
        ctx.raymarch(scene, cam, shadow=False, out=out, download=False)
        ctx.record(b)
    ctx.sync()
    ms = sum(ctx.elapsed_ms(a, b) for a, b in evs) / steps
    hits = out.download(meso.HIT_DTYPE, CFG1_W * CFG1_H)
    solid = scene.count_solid()
    host = oracle.gen_dense_u8(256, 256, 256, 1)
    bm = oracle.HostBrickMap.from_dense(host.astype(np.uint16))
    threads = oracle.hardware_threads()
    ocam = oracle.camera(CFG1_ORIGIN, CFG1_TARGET, CFG1_W, CFG1_H)
    reps, t0 = 0, time.perf_counter()
    while True:
        ref = oracle.raymarch(bm, ocam, shadow=False, nthreads=threads)
        reps += 1
        if time.perf_counter() - t0 > 2.0 or reps >= 20:
            break
    cpu_s = (time.perf_counter() - t0) / reps
    scene.destroy()
    rays = CFG1_W * CFG1_H
    return {"workload": "256^3 uint8 grid as a brick map, 640x360 pinhole camera (60 deg vertical FOV) from "
                        f"{CFG1_ORIGIN} aimed at {CFG1_TARGET}, primary rays to the first hit, one launch",
            "mrays_s": round(rays / (ms * 1e3), 1), "ms": round(ms, 4), "rays": rays,
            "hits": int(np.isfinite(hits["t"]).sum()), "occupancy": round(solid / 256 ** 3, 4),
            "parity_bit_exact": bool(np.array_equal(hits.view(np.uint8), ref.view(np.uint8))),
            "cpu_baseline": {"value": round(rays / cpu_s / 1e6, 2), "unit": "Mrays/s", "cores": threads,
                             "kind": "port", "sample": f"the full 640x360 frame, {reps} runs of {cpu_s * 1e3:.1f} ms"}}


def bench_mesh_brickmap(ctx, meso, scene, steps):
    """Brick-map meshing: every 32^3 chunk of the 1024^3 terrain (32,768
    chunks, neighbours' faces seen across chunk borders) in one persistent
    launch; air chunks are passed over by the scene's cell map, the occupied
    bricks of the others staged by the whole CTA.  Algorithmic bytes: 4 B
    per pointer fetched (64 per
    chunk), 1 KiB of materials + 64 B of occupancy per occupied brick, the
    one-voxel halo (6 x 32 x 32 occupancy bits per chunk) and 8 B per quad."""
    import ctypes
    L = meso._lib
    n = 32 ** 3
    idx = np.arange(n)
    coords = ctx.to_device(np.stack([idx % 32, (idx // 32) % 32, idx // 1024], 1).astype(np.int32))
    cap = 96 << 20
    qbuf, cnt = ctx.alloc(cap * 8), ctx.alloc(8)
    flush = ctx.alloc(L2_FLUSH_BYTES)
    src = meso.MeshSource()
    src.kind = meso.SRC_BRICKMAP
    src.scene = scene.handle
    out = meso.MeshOutput(qbuf.ptr, cap, cnt.ptr, None)

    def run():
        meso._check(L.meso_mesh_chunks(ctx.handle, ctypes.byref(src), coords.ptr, n, ctypes.byref(out), None))

    for _ in range(3):
        run()
    evs = [(ctx.event(), ctx.event()) for _ in range(steps)]
    for a, b in evs:
        flush.zero()
        ctx.record(a)
        run()
        ctx.record(b)
    ctx.sync()
    ms = sum(ctx.elapsed_ms(a, b) for a, b in evs) / steps
    total = ctypes.c_uint64()
    meso._check(L.meso_mesh_check(ctx.handle, ctypes.byref(out), None, ctypes.byref(total)))
    quads = int(total.value)
    bricks = int(scene.info().n_bricks)
    algo = n * 64 * 4 + bricks * (1024 + 64) + n * 6 * 32 * 32 // 8 + 8 * quads
    hbm = peaks()[0]
    ach = algo / (ms * 1e6)
    for b_ in (qbuf, cnt, flush, coords):
        b_.free()
    return {"workload": "all 32768 chunks of the 1024^3 terrain brick map (8^3 bricks, uint16), one persistent launch",
            "gvox_s": round(n * 32768 / (ms * 1e6), 2), "ms": round(ms, 4), "quads": quads, "bricks": bricks,
            "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(ach / hbm, 4), "algorithmic_bytes_per_launch": algo,
                         "traffic": ncu_traffic("mesh_kernel<BRICKMAP>"), "kernel": "mesh_kernel<BRICKMAP>"}}


def cpu_mesh_baseline(m, n_single=512):
    """Oracle mesher on the host cores: all threads over the whole batched
    workload (checked bit for bit against the GPU's quads), one thread over
    the first n_single chunks."""
    import ctypes
    import oracle
    data = np.ascontiguousarray(m["data"].download(np.uint16).reshape(MESH_CHUNKS, 32, 32, 32))
    gq = np.sort(m["qbuf"].download(np.uint64, count=m["quads"]))
    src = oracle._source(oracle.SRC_CHUNKS_U16, data)
    coords = np.zeros((MESH_CHUNKS, 3), np.int32)
    coords[:, 0] = np.arange(MESH_CHUNKS)
    out = np.zeros(len(gq) + 1, np.uint64)
    threads = oracle.hardware_threads()
    t0 = time.perf_counter()
    total = int(oracle.lib().mo_mesh_chunks_mt(ctypes.byref(src), oracle._ptr(coords), MESH_CHUNKS, threads,
                                                 oracle._ptr(out), out.size))
    dt = time.perf_counter() - t0
    parity = total == len(gq) and bool(np.array_equal(out[:total], gq))
    t0 = time.perf_counter()
    oracle.lib().mo_mesh_chunks_mt(ctypes.byref(src), oracle._ptr(coords), n_single, 1, oracle._ptr(out), out.size)
    dt1 = time.perf_counter() - t0
    return {"value": round(MESH_CHUNKS * 32768 / dt / 1e9, 4), "unit": "Gvox/s", "cores": threads, "kind": "port",
            "sample": f"all {MESH_CHUNKS} chunks, {dt:.2f} s",
            "single_thread": {"value": round(n_single * 32768 / dt1 / 1e9, 5), "unit": "Gvox/s", "cores": 1,
                              "sample": f"the first {n_single} chunks, {dt1:.2f} s"},
            "parity_bit_exact": parity}


def bench_downstream(ctx, meso, m, steps):
    """The steps either side of the hot paths: device scene build, quad ->
    vertex expansion and the erosion pyramid on the batched-meshing data."""
    import ctypes
    L = meso._lib
    hbm = peaks()[0]
    res = {}
    # device scene build of the 1024^3 terrain (pointer grid + pools written)
    t0 = time.perf_counter()
    sc = ctx.scene_from_terrain(meso.terrain_preset("scene1024"))
    build_s = time.perf_counter() - t0
    info = sc.info()
    written = info.n_bricks * (64 + 1024) + (1024 // 8) ** 3 * 4
    res["scene_build"] = {"workload": "1024^3 terrain (6-octave fBm heightfield, caves), device generator + scan",
                          "ms": round(build_s * 1e3, 2), "bricks": int(info.n_bricks),
                          "gb_s_written": round(written / build_s / 1e9, 1)}
    sc.destroy()
    # quad -> vertex expansion of the batched mesh output (8 B in, 64 B out per quad)
    nq = m["quads"]
    origins = ctx.to_device(np.stack([np.arange(MESH_CHUNKS), np.zeros(MESH_CHUNKS), np.zeros(MESH_CHUNKS)], 1)
                            .astype(np.int32))
    verts = ctx.alloc(nq * 64)
    flush = ctx.alloc(L2_FLUSH_BYTES)

    def timed(fn):
        fn()
        ctx.sync()
        tot = 0.0
        for _ in range(steps):
            flush.zero()
            a, b = ctx.event(), ctx.event()
            ctx.record(a)
            fn()
            ctx.record(b)
            ctx.sync()
            tot += ctx.elapsed_ms(a, b)
        return tot / steps

    ms = timed(lambda: meso._check(L.meso_quads_to_vertices(ctx.handle, m["qbuf"].ptr, nq, origins.ptr,
                                                            MESH_CHUNKS, verts.ptr, None)))
    ach = nq * 72 / (ms * 1e6)
    res["quads_to_vertices"] = {"quads": nq, "ms": round(ms, 4), "roofline": {
        "bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s", "frac": round(ach / hbm, 4),
        "algorithmic_bytes_per_launch": nq * 72}}
    verts.free()
    # erosion pyramid (4 mips) of the 4096 standalone chunks: 64 KiB in, 4 x 4 KiB out per chunk
    out = ctx.alloc(MESH_CHUNKS * 4 * 4096)
    src = meso.MeshSource()
    src.kind = meso.SRC_CHUNKS_U16
    src.d_data = m["data"].ptr
    ms = timed(lambda: meso._check(L.meso_erode_mips(ctx.handle, ctypes.byref(src), None, MESH_CHUNKS, 4, out.ptr,
                                                     None)))
    algo = MESH_CHUNKS * (65536 + 4 * 4096)
    ach = algo / (ms * 1e6)
    res["erode_mips"] = {"workload": f"{MESH_CHUNKS} chunks of 32^3 uint16, 4 mips", "ms": round(ms, 4),
                         "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                                      "frac": round(ach / hbm, 4), "algorithmic_bytes_per_launch": algo}}
    out.free()
    flush.free()
    return res


def poisson_arrivals(rate, seconds, seed):
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            return out
        out.append(t)


def outside_pose(rng, n, target):
    """Camera origin outside the n^3 grid (distance 1.1 n from the centre, upper hemisphere)."""
    v = rng.normal(size=3)
    v[2] = abs(v[2]) + 0.2
    v /= np.linalg.norm(v)
    return tuple(float(c) for c in (np.full(3, n / 2.0) + v * 1.1 * n)), tuple(float(c) for c in target)


def replay(server, items, submit):
    """Submits items[k] = (arrival_s, ...) at their arrival times; returns completions."""
    comps = []
    t0 = server.now()
    i = 0
    while i < len(items):
        now = server.now() - t0
        while i < len(items) and items[i][0] <= now:
            submit(items[i])
            i += 1
        comps += server.poll()
        if i < len(items):
            dt = items[i][0] - (server.now() - t0)
            if dt > 2e-4:
                time.sleep(min(dt, 1e-3))
    server.drain(600.0)
    comps += server.poll()
    return comps


def summarize(comps):
    ok = [c for c in comps if c.status == 0]
    lat = np.array([c.done_s - c.submit_s for c in ok]) * 1e3
    span = (max(c.done_s for c in ok) - min(c.submit_s for c in comps)) if ok else 1.0
    rays = sum(c.n_rays for c in ok)
    return {
        "requests": len(comps), "completed": len(ok), "rejected": sum(c.status == 3 for c in comps),
        "p50_ms": round(float(np.percentile(lat, 50)), 3) if len(lat) else None,
        "p99_ms": round(float(np.percentile(lat, 99)), 3) if len(lat) else None,
        "mrays_s": round(rays / span / 1e6, 1), "span_s": round(span, 3),
    }


def bench_serve_render(ctx, meso, seconds, rate=2000.0):
    """Served raymarching: 4 resident scenes (512^3, 1024^3, 1024^3, 2048^3),
    Poisson arrivals, image size uniform over {256^2, 512^2, 1920x1080,
    3840x2160}, primary rays only, 120 GB HBM budget."""
    names = ("serve512", "serve1024", "serve1024b", "serve2048")
    scenes = [ctx.scene_from_terrain(meso.terrain_preset(n)) for n in names]
    dims = [meso.terrain_preset(n).nx for n in names]
    sizes = [(256, 256), (512, 512), (1920, 1080), (3840, 2160)]
    rng = np.random.default_rng(7)
    items = []
    for t in poisson_arrivals(rate, seconds, 7):
        s = int(rng.integers(0, 4))
        n = dims[s]
        tgt = (rng.uniform(0.25, 0.75) * n, rng.uniform(0.25, 0.75) * n, rng.uniform(0.02, 0.2) * n)
        o, tg = outside_pose(rng, n, tgt)
        w, h = sizes[int(rng.integers(0, 4))]
        items.append((t, s, meso.camera(o, tg, w, h)))
    srv = meso.Server(ctx, scenes, max_inflight_batches=4, max_batch_rays=16 << 20, max_queue=512,
                      hbm_budget_bytes=120 << 30)
    comps = replay(srv, items, lambda it: srv.submit(it[1], it[2], shadow=False))
    srv.close()
    res = summarize(comps)
    res["offered_mrays_s"] = round(sum(it[2].width * it[2].height for it in items) / seconds / 1e6, 1)
    # capacity: the first K requests submitted at once (no arrival pacing)
    k = min(2000, len(items))
    srv = meso.Server(ctx, scenes, max_inflight_batches=4, max_batch_rays=16 << 20, hbm_budget_bytes=120 << 30)
    t0 = time.perf_counter()
    for it in items[:k]:
        srv.submit(it[1], it[2], shadow=False)
    srv.drain(600.0)
    burst_s = time.perf_counter() - t0
    burst = srv.poll(1 << 16)
    srv.close()
    px = sum(it[2].width * it[2].height for it in items[:k])
    res["capacity_mrays_s"] = round(px / burst_s / 1e6, 1)
    # plain form: the same K requests, one launch per request, each waited for
    out = ctx.alloc(3840 * 2160 * 24)
    ctx.sync()
    t0 = time.perf_counter()
    for it in items[:k]:
        ctx.raymarch(scenes[it[1]], it[2], shadow=False, out=out, download=False)
        ctx.sync()
    res["plain_per_view_mrays_s"] = round(px / (time.perf_counter() - t0) / 1e6, 1)
    res["capacity_over_plain"] = round(res["capacity_mrays_s"] / max(res["plain_per_view_mrays_s"], 1e-9), 2)
    res["capacity_requests"] = k
    assert all(c.status == 0 for c in burst)
    res["workload"] = (f"4 resident scenes {dims}, Poisson {rate:.0f} req/s for {seconds:.0f} s (seed 7), "
                       "sizes {256^2, 512^2, 1920x1080, 3840x2160}, primary rays, HBM budget 120 GB")
    # per image-size class: the class's requests among the first K, submitted
    # at once (capacity) and one launch each, waited for (plain)
    per_size, plain_s, cap_sz = {}, {}, {}
    for w, h in sizes:
        its = [it for it in items[:k] if (it[2].width, it[2].height) == (w, h)]
        if not its:
            continue
        spx = len(its) * w * h
        srv = meso.Server(ctx, scenes, max_inflight_batches=4, max_batch_rays=16 << 20, hbm_budget_bytes=120 << 30)
        t0 = time.perf_counter()
        for it in its:
            srv.submit(it[1], it[2], shadow=False)
        srv.drain(600.0)
        cap_s = time.perf_counter() - t0
        srv.poll(1 << 16)
        srv.close()
        ctx.sync()
        t0 = time.perf_counter()
        for it in its:
            ctx.raymarch(scenes[it[1]], it[2], shadow=False, out=out, download=False)
            ctx.sync()
        plain_s[(w, h)] = time.perf_counter() - t0
        cap_sz[(w, h)] = cap_s
        per_size[f"{w}x{h}"] = {"requests": len(its), "capacity_mrays_s": round(spx / cap_s / 1e6, 1),
                                "plain_per_view_mrays_s": round(spx / plain_s[(w, h)] / 1e6, 1),
                                "capacity_over_plain": round(plain_s[(w, h)] / cap_s, 2)}
    res["per_size"] = per_size
    # the bound for this mix: even if batching made the two small classes cost
    # nothing, the 1080p and 4K requests (whose single launches already fill
    # the GPU) need at least their own batched time, so
    # capacity/plain <= (plain time of all classes) / (batched time of the large classes)
    big = sum(v for (w, h), v in cap_sz.items() if w * h >= 1920 * 1080)
    res["mix_bound_capacity_over_plain"] = round(sum(plain_s.values()) / max(big, 1e-9), 2)
    out.free()
    # delivered: the same arrivals for half the time, each request's hits
    # copied into page-locked host memory before its completion is reported
    # (one destination buffer per size class, shared by the requests of that
    # class: their contents are not read here)
    dst = {wh: ctx.pinned(wh[0] * wh[1] * 24) for wh in sizes}
    half = [it for it in items if it[0] <= seconds / 2]
    srv = meso.Server(ctx, scenes, max_inflight_batches=4, max_batch_rays=16 << 20, max_queue=512,
                      hbm_budget_bytes=120 << 30)
    comps = replay(srv, half, lambda it: srv.submit(it[1], it[2], shadow=False,
                                                    dst=dst[(it[2].width, it[2].height)]))
    srv.close()
    d = summarize(comps)
    d["workload"] = f"the first {seconds / 2:.0f} s of the same arrivals, hits delivered into page-locked host memory"
    d["delivered_gb_s"] = round(sum(c.n_rays for c in comps if c.status == 0) * 24 / d["span_s"] / 1e9, 1)
    # the link's own rate for such copies: one 4K frame of hits (199 MB)
    # copied device -> page-locked host memory, and four such copies at once
    # on the server's four slot streams
    big = dst[(3840, 2160)]
    src_hits = ctx.alloc(big.nbytes)
    L = meso._lib
    streams = [ctx.stream() for _ in range(4)]
    for k in range(2):
        meso._check(L.meso_memcpy_d2h(ctx.handle, big.ptr, src_hits.ptr, big.nbytes, None))
    ctx.sync()
    t0 = time.perf_counter()
    for k in range(5):
        meso._check(L.meso_memcpy_d2h(ctx.handle, big.ptr, src_hits.ptr, big.nbytes, None))
    ctx.sync()
    one = big.nbytes * 5 / (time.perf_counter() - t0) / 1e9
    t0 = time.perf_counter()
    for k in range(5):
        for st in streams:
            meso._check(L.meso_memcpy_d2h(ctx.handle, big.ptr, src_hits.ptr, big.nbytes, st))
    for st in streams:
        ctx.sync(st)
    four = big.nbytes * 20 / (time.perf_counter() - t0) / 1e9
    d["link_d2h_gb_s"] = {"one_stream": round(one, 1), "four_streams": round(four, 1)}
    src_hits.free()
    res["delivered"] = d
    for b_ in dst.values():
        b_.free()
    for s in scenes:
        s.destroy()
    return res


def bench_serve_edit(ctx, meso, seconds, rate=200.0):
    """Served edit + remesh + render on the 4096^3 scene (~2% solid): 1-32
    spheres per request (radius 2-32, add/remove 50/50, material 1..65535),
    remesh of the dirty 32^3 chunks, then a 1920x1080 render (primary)."""
    t = meso.terrain_preset("edit4096")
    scene = ctx.scene_from_terrain(t, spare_bricks=4 << 20)
    occupancy = scene.count_solid() / float(t.nx * t.ny * t.nz)
    n = t.nx
    rng = np.random.default_rng(9)
    items = []
    for ta in poisson_arrivals(rate, seconds, 9):
        edits = []
        for _ in range(int(rng.integers(1, 33))):
            c = [int(rng.integers(0, n)), int(rng.integers(0, n)), int(rng.integers(0, 192))]
            m = 0 if rng.random() < 0.5 else int(rng.integers(1, 65536))
            import ctypes
            edits.append(meso.SphereEdit((ctypes.c_int32 * 3)(*c), int(rng.integers(2, 33)), m, 0))
        o, tg = outside_pose(rng, n, (edits[0].center[0], edits[0].center[1], edits[0].center[2]))
        items.append((ta, edits, meso.camera(o, tg, 1920, 1080)))
    # the server keeps the scene's mesh store current and delivers each render
    # into page-locked host memory before reporting it complete
    dst = ctx.pinned(1920 * 1080 * 24)
    srv = meso.Server(ctx, [scene], max_inflight_batches=4, max_batch_rays=4 << 20, max_queue=512,
                      max_edit_quads=64 << 20, keep_meshes=1)
    comps = replay(srv, items, lambda it: srv.submit(0, it[2], shadow=False, edits=it[1], dst=dst))
    si = srv.store(0).info()
    store_info = {"live_quads": int(si.live_quads), "arena_quads": int(si.arena_quads),
                  "arena_used": int(si.arena_used), "compactions": int(si.compactions)}
    srv.close()
    res = summarize(comps)
    res["mesh_store"] = store_info
    ok = [c for c in comps if c.status == 0]
    chunks = sum(c.n_dirty_chunks for c in ok)
    busy = sum(c.done_s - c.start_s for c in ok)
    res["dirty_chunks"] = chunks
    res["quads"] = int(sum(c.n_quads for c in ok))
    res["gvox_meshed_s_wall"] = round(chunks * 32768 / res["span_s"] / 1e9, 3)
    res["gvox_meshed_s_busy"] = round(chunks * 32768 / max(busy, 1e-9) / 1e9, 3)
    res["workload"] = (f"4096^3 terrain (512^3 pointer grid), Poisson {rate:.0f} req/s for {seconds:.0f} s (seed 9), "
                       "1-32 sphere edits + remesh of dirty chunks into the scene's resident mesh store + "
                       "1920x1080 primary render delivered into page-locked host memory")
    res["voxel_occupancy"] = round(occupancy, 5)
    # capacity (requests submitted at once) and the plain form (edit, one mesh
    # launch per dirty chunk, one render launch, waited for) on fresh copies
    k = min(200, len(items))
    scene.destroy()
    scene = ctx.scene_from_terrain(t, spare_bricks=4 << 20)
    srv = meso.Server(ctx, [scene], max_inflight_batches=4, max_batch_rays=4 << 20, max_edit_quads=64 << 20,
                      keep_meshes=1)
    t0 = time.perf_counter()
    for it in items[:k]:
        srv.submit(0, it[2], shadow=False, edits=it[1], dst=dst)
    srv.drain(600.0)
    cap_s = time.perf_counter() - t0
    comps = srv.poll(1 << 16)
    srv.close()
    cap_chunks = sum(c.n_dirty_chunks for c in comps)
    scene.destroy()
    scene = ctx.scene_from_terrain(t, spare_bricks=4 << 20)
    qbuf, cnt = ctx.alloc((64 << 20) * 8), ctx.alloc(8)
    hits = ctx.alloc(1920 * 1080 * 24)
    cx = n // 32
    src = meso.MeshSource()
    src.kind = meso.SRC_BRICKMAP
    src.scene = scene.handle
    mo = meso.MeshOutput(qbuf.ptr, 64 << 20, cnt.ptr, None)
    import ctypes
    L = meso._lib
    plain_chunks = 0
    ctx.sync()
    t0 = time.perf_counter()
    for it in items[:k]:
        dirty = scene.edit(it[1])
        if len(dirty):
            coords = np.stack([dirty % cx, (dirty // cx) % cx, dirty // (cx * cx)], 1).astype(np.int32)
            cb = ctx.to_device(coords)
            meso._check(L.meso_mesh_chunks_per_launch(ctx.handle, ctypes.byref(src), cb.ptr, len(dirty),
                                                      ctypes.byref(mo), None))
            plain_chunks += len(dirty)
        ctx.raymarch(scene, it[2], shadow=False, out=hits, download=False)
        meso._check(L.meso_memcpy_d2h(ctx.handle, dst.ptr, hits.ptr, 1920 * 1080 * 24, None))
        ctx.sync()
    plain_s = time.perf_counter() - t0
    res["capacity_requests"] = k
    res["capacity_req_s"] = round(k / cap_s, 1)
    res["capacity_gvox_meshed_s"] = round(cap_chunks * 32768 / cap_s / 1e9, 3)
    res["plain_req_s"] = round(k / plain_s, 1)
    res["plain_gvox_meshed_s"] = round(plain_chunks * 32768 / plain_s / 1e9, 3)
    res["capacity_over_plain"] = round(res["capacity_req_s"] / max(res["plain_req_s"], 1e-9), 2)
    scene.destroy()
    return res


def cpu_baseline_port(meso, ctx, r):
    """Oracle DDA on the host cores over the whole frame, scene copied from the device."""
    import oracle
    ptr, occ, mat = r["scene"].download()
    bm = oracle.HostBrickMap.from_arrays((1024, 1024, 1024), ptr, occ, mat)
    ocam = oracle.camera(CAM_ORIGIN, CAM_TARGET, FRAME_W, FRAME_H)
    threads = oracle.hardware_threads()
    t0 = time.perf_counter()
    h = oracle.raymarch(bm, ocam, nthreads=threads)
    dt = time.perf_counter() - t0
    parity = bool(np.array_equal(h.view(np.uint8), r["hits"].view(np.uint8)))
    rows, row0 = FRAME_H // 8, (FRAME_H - FRAME_H // 8) // 2
    t0 = time.perf_counter()
    h1 = oracle.raymarch_rows(bm, ocam, row0, rows, nthreads=1)
    dt1 = time.perf_counter() - t0
    return {"value": count_rays(h) / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"the full {FRAME_W}x{FRAME_H} frame (primary + shadow), {dt:.2f} s",
            "single_thread": {"value": round(count_rays(h1) / dt1 / 1e6, 3), "unit": "Mrays/s", "cores": 1,
                              "sample": f"rows {row0}-{row0 + rows - 1} of the frame, {dt1:.2f} s"},
            "parity_full_frame_bit_exact": parity}


def run_ours(args, world, rank, local, dist):
    import mesoengine_gb300 as meso
    ctx = meso.Context(local)
    clocks = Clocks(local)
    r = bench_raymarch(ctx, meso, args.steps, args.warmup, dist, clocks)
    clk = clocks.summary()
    ms_max = reduce_max(dist, r["ms"])
    rays_all = reduce_sum(dist, float(r["rays"]))
    value = rays_all / (ms_max * 1e3)  # Mrays/s
    hbm, which = peaks()
    achieved = r["algo_bytes"] / (r["ms"] * 1e6)  # GB/s
    l2 = ctx.measure_l2_read(32 << 20, 50)  # the fetches hit in L2: its read bandwidth beside HBM's
    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "Mrays/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_max, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded terrain: 6-octave fBm heightfield + 3-D value-noise caves)",
        "config": {
            "workload": "1024^3 sparse brick scene, 1920x1080 primary + 1 shadow ray per hit, plain per-view launch",
            "scene": "8^3 bricks, 128^3 uint32 pointer grid, uint16 materials, "
                     f"{r['bricks']} bricks, {r['scene_bytes'] / 2**20:.0f} MiB resident",
            "camera": {"origin": CAM_ORIGIN, "target": CAM_TARGET, "fov_y_deg": 60},
            "rays_per_frame": r["rays"],
            "voxel_occupancy": round(r["occupancy"], 4),
            "tuning": {k: v for k, v in ctx.config().items() if k not in ("device", "hbm_budget_bytes")},
            "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MiB memset outside the timed events)",
            "parallelism": f"replicas x{world}",
        },
        "clocks": clk,
        "e2e": {"value": round(r["rays"] / (r["e2e_ms"] * 1e3), 2), "unit": "Mrays/s",
                "h2d_bytes_per_step": 72, "d2h_bytes_per_step": FRAME_W * FRAME_H * 24,
                "api": "meso_raymarch_host (camera from host memory; the kernel writes the hits into a page-locked host buffer over the CPU-GPU link)"},
        "gpu_launches": int(r["launches"]),
        "roofline": {
            "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "traffic": ncu_traffic("raymarch_kernel"), "peak_source": which,
            "kernel": "raymarch_kernel",
            # what limits it (ncu): instruction issue, not DRAM -- its fetches hit in L1/L2
            "limiter": "issue",
            "issue_active_pct": ncu_field("raymarch_kernel", "smsp__issue_active_pct"),
            "active_lanes_per_instruction": ncu_field("raymarch_kernel", "active_lanes_per_instruction"),
            "l2_frac": round(achieved / l2, 4),
            "l2": {"peak": round(l2, 1), "unit": "GB/s", "frac": round(achieved / l2, 4),
                   "how": "meso_measure_l2_read: a 32 MiB buffer read 50 times with 16-byte L1-bypassing loads"},
            "algorithmic_bytes_per_launch": int(r["algo_bytes"]),
            "counts": r["counts"],
        },
    }
    if rank == 0 and not args.skip_mesh:
        m = bench_mesh(ctx, meso, args.steps, args.warmup)
        ach = m["algo_bytes"] / (m["ms"] * 1e6)
        line["mesh"] = {
            "workload": f"{MESH_CHUNKS} standalone 32^3 uint16 chunks, occupancy log-uniform 0.1%-90%, 1-64 materials",
            "gvox_s": round(m["gvox_s"], 2), "ms": round(m["ms"], 4), "quads": m["quads"],
            "per_chunk_launch_gvox_s": round(m["gvox_s_plain"], 3),
            "per_chunk_launch_graph_replay_gvox_s": round(m["gvox_s_graph"], 3),
            "batched_over_per_launch": round(m["ms_plain"] / m["ms"], 2),
            "e2e": {"value": round(MESH_CHUNKS * 32768 / (m["e2e_ms"] * 1e6), 2), "unit": "Gvox/s",
                    "ms": round(m["e2e_ms"], 4), "h2d_bytes_per_step": MESH_CHUNKS * 65536,
                    "d2h_bytes_per_step": 8 * m["quads"] + 8, "same_quads_as_device_path": m["e2e_exact"],
                    "api": "meso_mesh_host (chunks in page-locked host memory, uploaded in slices of 1024 while "
                           "the previous slice is meshed; quads written by the kernel into page-locked host memory)"},
            "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(ach / hbm, 4), "algorithmic_bytes_per_launch": m["algo_bytes"],
                         "traffic": ncu_traffic("mesh_kernel<CHUNKS_U16>"), "kernel": "mesh_kernel<CHUNKS_U16>"},
        }
        if not args.skip_cpu:
            line["mesh"]["cpu_baseline"] = cpu_mesh_baseline(m)
        line["mesh"]["uint8"] = bench_mesh_u8(ctx, meso, m, args.steps)
        line["mesh"]["brickmap"] = bench_mesh_brickmap(ctx, meso, r["scene"], args.steps)
        line["downstream"] = bench_downstream(ctx, meso, m, args.steps)
    if rank == 0 and not args.skip_serve:
        line["served"] = bench_serve_render(ctx, meso, args.serve_seconds)
        line["served_edit"] = bench_serve_edit(ctx, meso, args.serve_seconds)
    if rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline_port(meso, ctx, r)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


# ------------------------------------------------------------ reference arm

def run_reference(args, world, rank, local, dist):
    """The reference has no raymarcher (it rasterises imposter cubes through
    Vulkan, which cannot run here); its stand-in is the CPU oracle DDA on all
    host cores, on the same scene and camera.  Each step traces a bounded
    sample of 270 rows of the frame."""
    if rank != 0:
        return
    import oracle
    import mesoengine_gb300 as meso_presets  # parameters only (terrain preset), no device use
    t = meso_presets.terrain_preset("scene1024")
    ot = oracle.terrain(t.nx, t.ny, t.nz, t.seed, t.height_period, t.height_octaves, t.height_base, t.height_amp,
                        t.cave_period, t.cave_threshold)
    threads = oracle.hardware_threads()
    bm = oracle.HostBrickMap.from_terrain(ot, nthreads=threads)
    cam = oracle.camera(CAM_ORIGIN, CAM_TARGET, FRAME_W, FRAME_H)
    rows = 270
    for k in range(args.warmup):
        oracle.raymarch_rows(bm, cam, (k * rows) % FRAME_H, rows, nthreads=threads)
    total_rays, total_s = 0, 0.0
    for k in range(args.steps):
        r0 = (k * rows) % FRAME_H
        t0 = time.perf_counter()
        h = oracle.raymarch_rows(bm, cam, r0, rows, nthreads=threads)
        total_s += time.perf_counter() - t0
        total_rays += count_rays(h)
    value = total_rays / total_s / 1e6
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1000 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (same seeded 1024^3 terrain and camera)",
        "config": {"workload": "1024^3 sparse brick scene, 1920x1080 primary + 1 shadow ray per hit",
                   "sample_rows_per_step": rows},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{rows} rows of the 1920x1080 frame per step"},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile_case(case: str):
    """One kernel of interest after a few warm-up launches, for ncu captures:
    'ray' = the 1080p frame of the 1024^3 scene (3 warm-up launches + 1),
    'mesh' = the 4096-chunk batched mesh (3 warm-up launches + 1),
    'meshbrick' = all 32768 chunks of the 1024^3 brick map (3 warm-up launches + 1)."""
    import mesoengine_gb300 as meso
    ctx = meso.Context(0)
    if case == "ray":
        scene = ctx.scene_from_terrain(meso.terrain_preset("scene1024"))
        cam = meso.camera(CAM_ORIGIN, CAM_TARGET, FRAME_W, FRAME_H)
        out = ctx.alloc(FRAME_W * FRAME_H * 24)
        for _ in range(4):
            ctx.raymarch(scene, cam, out=out, download=False)
    elif case == "meshbrick":
        scene = ctx.scene_from_terrain(meso.terrain_preset("scene1024"))
        idx = np.arange(32 ** 3)
        coords = np.stack([idx % 32, (idx // 32) % 32, idx // 1024], 1).astype(np.int32)
        for _ in range(4):
            ctx.mesh(meso.SRC_BRICKMAP, coords=coords, scene=scene, capacity=96 << 20)
    else:
        data, _ = ctx.generate_chunks_u16(MESH_CHUNKS, seed0=1)
        for _ in range(4):
            ctx.mesh(meso.SRC_CHUNKS_U16, data, n=MESH_CHUNKS, capacity=MESH_CHUNKS * 8192)
    ctx.sync()
    print(f"profile case {case} done, {ctx.kernel_launches} launches")
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile", choices=["ray", "mesh", "meshbrick"], default=None,
                    help="run one small single-kernel case for an ncu capture and exit")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-mesh", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.profile:
        run_profile_case(args.profile)
        return
    args.warmup = max(3, args.warmup)
    if args.gpus < 1:
        ap.error("--gpus must be at least 1")
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_replicas(args.gpus))
    if int(os.environ.get("WORLD_SIZE", "1")) != args.gpus:
        ap.error(f"--gpus {args.gpus} but WORLD_SIZE={os.environ.get('WORLD_SIZE')}: one process per GPU")
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, local, dist)
    else:
        run_ours(args, world, rank, local, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
