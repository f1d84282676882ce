#!/usr/bin/env python3
"""Benchmark of the DoonEngine lighting + draw path on GB300.

Workload ("large"): a 64x32x64-chunk map (512x256x512 voxels, ~15% of chunks non-empty; seeded
heightfield + 2000 boxes and spheres), a fixed camera, 1920x1080 primary rays, lighting with
1 diffuse path per voxel per frame and K=32 fixed direct / specular rays per voxel.  One step is one
frame in the reference's order: DN_draw -> DN_sync_gpu -> DN_update_lighting (main.c:503-505).
Data are synthetic and seeded (the reference publishes no scenes or numbers).

Metric: aggregate rays/s = every traversal segment (primary, shadow, specular, diffuse) counted once by
device counters, over the summed CUDA-event time of the timed steps (inputs resident in HBM, L2 flushed
between steps outside the timed events).  ``e2e``: the same frames through the C API drawing into pinned
host memory, each step ending with the image, hit indices and faces on the host (wall clock).

--impl reference: the reference path runs only as GLSL (no graphics stack here), so the reference arm
times the CPU restatement of its algorithm (oracle/) on the host cores, on a bounded sample per step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAKS_FALLBACK = {"hbm_gbs": 6800.0}
METRIC = "aggregate rays/s"
L2_FLUSH_BYTES = 256 << 20


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    except Exception:
        return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        finally:
            os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce_max(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def workload_desc(cfg, vol=None, nonempty=None, name="large"):
    sx, sy, sz = cfg["map"]
    d = {"workload": "%s: %dx%dx%d chunks (%dx%dx%d voxels), heightfield + %d boxes/spheres, %dx%d draw, "
                     "K=%d direct/specular rays, 1 diffuse path per voxel per frame"
                     % (name, sx, sy, sz, sx * 8, sy * 8, sz * 8, cfg["shapes"], cfg["res"][0], cfg["res"][1], cfg["K"]),
         "map_chunks": [sx, sy, sz], "resolution": list(cfg["res"]), "K": cfg["K"], "diffuse_spp": 1,
         "seed": cfg["seed"], "frame": "draw -> sync -> lighting",
         "l2": "flushed between timed steps (256 MiB write, outside the timed events)"}
    if nonempty is not None:
        d["nonempty_chunk_frac"] = round(nonempty, 4)
    return d


# ------------------------------------------------------------------ our arm

def run_ours(args):
    rank, world, local, pg = dist_setup()
    import doonengine_gb300 as dn
    from doonengine_gb300 import configs
    lib = dn.load()
    if lib.dn_cuda_init(local) != 0:
        raise RuntimeError("dn_cuda_init(%d): %s" % (local, lib.dn_cuda_last_error().decode()))
    dn.init()
    vol, cfg = configs.build_volume(args.config, seed=configs.CONFIGS[args.config]["seed"] + 1000 * rank)
    vol.s.mapId = rank
    if args.residency == "lru":
        vol.set_residency("lru")
    nonempty = vol.nonempty_chunks() / vol.num_tiles
    W, H = cfg["res"]
    img = dn.Image(W, H, on_device=True)
    view, proj = vol.view_proj(H / W)
    stream = vol.stream()
    frame = [0]

    def step(image):
        t = 1.0 + 0.25 * frame[0]
        vol.draw(image, view, proj)
        vol.sync(dn.DN_READ_WRITE, 1)
        vol.update_lighting(1, 1000, t)
        frame[0] += 1

    for _ in range(args.warmup):
        step(img)
    assert vol.finish(), lib.dn_cuda_last_error().decode()

    K = args.steps
    evs = []
    for _ in range(3 * K):
        e = __import__("ctypes").c_void_p()
        lib.dn_cuda_event_create(e)
        evs.append(e)
    vol.reset_stats()
    launches0 = lib.dn_cuda_launch_count()
    clocks = ClockSampler(local)
    barrier(pg)
    lib.dn_cuda_device_sync()
    clocks.start()
    t0 = time.perf_counter()
    for k in range(K):
        lib.dn_cuda_flush_l2(stream, L2_FLUSH_BYTES)
        lib.dn_cuda_event_record(evs[3 * k], stream)
        t = 1.0 + 0.25 * frame[0]
        vol.draw(img, view, proj)
        vol.sync(dn.DN_READ_WRITE, 1)
        lib.dn_cuda_event_record(evs[3 * k + 1], stream)
        vol.update_lighting(1, 1000, t)
        lib.dn_cuda_event_record(evs[3 * k + 2], stream)
        frame[0] += 1
    lib.dn_cuda_device_sync()
    barrier(pg)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = lib.dn_cuda_launch_count() - launches0 - K   # minus the L2-flush kernels
    ms = __import__("ctypes").c_float()
    dev_ms, light_ms = 0.0, 0.0
    for k in range(K):
        lib.dn_cuda_event_elapsed_ms(evs[3 * k], evs[3 * k + 2], ms)
        dev_ms += ms.value
        lib.dn_cuda_event_elapsed_ms(evs[3 * k + 1], evs[3 * k + 2], ms)
        light_ms += ms.value
    st_all = vol.stats_kind(0)
    st_light = vol.stats_kind(2)
    assert vol.finish(), lib.dn_cuda_last_error().decode()

    rays_total = allreduce_sum(pg, st_all["rays"])
    lit_total = allreduce_sum(pg, st_all["litVoxels"])
    prim_total = allreduce_sum(pg, st_all["primaryRays"])
    dev_ms_max = allreduce_max(pg, dev_ms)
    value = rays_total / (dev_ms_max / 1e3)

    # roofline of the dominant kernel (lighting: k_light + k_commit), algorithmic bytes from exact counters:
    # 4 B per chunk cell visited, 64 B per chunk mask entered, 28 B per voxel hit, 40 B per lit voxel
    peaks, peak_kind = load_peaks()
    peak = float(peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"]))
    bytes_light = (4 * st_light["outerSteps"] + 64 * st_light["chunksEntered"] + 28 * st_light["hits"]
                   + 40 * st_light["litVoxels"])
    per_launch_bytes = bytes_light / K
    per_launch_s = (light_ms / K) / 1e3
    achieved = per_launch_bytes / per_launch_s / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "k_light_traffic.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            # captured DRAM bytes per lit voxel of the profiled launch, scaled to this run's launches
            traffic = tj["dram_bytes_per_lit_voxel"] * st_light["litVoxels"] / K
        except Exception:
            traffic = None

    result = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": dev_ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded heightfield + boxes/spheres; the reference publishes no scenes)",
        "config": dict(workload_desc(cfg, vol, nonempty, args.config), parallelism="replicas: one map per GPU, no collective",
                       frames_timed="frames %d..%d of the accumulation (frame 0 starts with no chunk loaded; chunks "
                                    "load one sync after a ray requests them, so the lighting work grows over the "
                                    "first frames)" % (args.warmup, args.warmup + K - 1),
                       **({"residency": "DN_RESIDENCY_LRU (the reference's voxel-buffer nodes; each sync reads the "
                                        "rays' flags back and walks the tiles on the host)"}
                          if args.residency == "lru" else {})),
        "lit_voxels_per_s": lit_total / (dev_ms_max / 1e3),
        "primary_rays_per_s": prim_total / (dev_ms_max / 1e3),
        "rays_per_step": rays_total / K,
        "wall_s": wall,
        "gpu_launches": int(allreduce_sum(pg, launches)),
        "roofline": {"bound": "hbm", "kernel": "k_light_packet+k_commit (DN_update_lighting)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic, "algorithmic_bytes_per_launch": per_launch_bytes,
                     "traffic_source": "scaled, not measured in this run: DRAM bytes per lit voxel of one ncu capture "
                                       "(profiles/k_light_traffic.json) x this run's lit voxels per launch",
                     "launch_ms": per_launch_s * 1e3},
        "clocks": clk,
        "light_counters_per_step": {k: v / K for k, v in st_light.items()},
    }

    # e2e: the same frames through the C API into pinned host memory, host-side wall clock per step
    if not args.no_e2e:
        himg = dn.Image(W, H, on_device=False)
        vol.reset_stats()
        barrier(pg)
        lib.dn_cuda_device_sync()
        t0 = time.perf_counter()
        for k in range(K):
            step(himg)
            assert vol.finish()
        e2e_s = time.perf_counter() - t0
        e2e_s = allreduce_max(pg, e2e_s)
        st_e = vol.stats_kind(0)
        e_rays = allreduce_sum(pg, st_e["rays"])
        result["e2e"] = {"value": e_rays / e2e_s, "unit": "rays/s",
                         "h2d_bytes_per_step": 2 * 256 * 32 + 1024,
                         "d2h_bytes_per_step": W * H * (16 + 4 + 1) + 8,
                         "path": "DN_draw(host DNimage) + DN_sync_gpu + DN_update_lighting + DN_finish"}
        himg.close()

    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline_sample(vol, view, proj, W, H, args.cpu_seconds)
    result["rays_by_kind_per_step"] = {"primary": prim_total / K, "lighting": (rays_total - prim_total) / K}
    vol.close()
    img.close()

    # the headline metric's other two parts on the same box: batched vs plain on the batched workload,
    # and serving latency / throughput on the serving workload (one GPU; replicas skip them)
    if world == 1 and not args.no_batched:
        t1 = time.perf_counter()
        result["batched_vs_plain"] = batched_vs_plain(args, lib, rank, pg, local, args.batched_warmup,
                                                      args.batched_frames)
        log("batched vs plain: %.1f s" % (time.perf_counter() - t1))
    if world == 1 and not args.no_serving:
        t1 = time.perf_counter()
        rates = [float(x) for x in args.serving_rates.split(",")]
        sv = serving_sweep(args, lib, rank, world, 256, rates, args.serving_seconds, args.budget_gb)
        result["serving"] = serving_summary(sv)
        log("serving: %.1f s" % (time.perf_counter() - t1))
        if args.pressure_budget_gb > 0:
            t1 = time.perf_counter()
            rates = [float(x) for x in args.pressure_rates.split(",")]
            sv = serving_sweep(args, lib, rank, world, 256, rates, args.pressure_seconds, args.pressure_budget_gb)
            result["serving_under_eviction"] = serving_summary(sv)
            log("serving under eviction: %.1f s" % (time.perf_counter() - t1))
    if rank == 0:
        print(json.dumps(result), flush=True)


def serving_summary(sv):
    """The serving line's figures that the headline carries: per offered rate p50 / p99 latency, achieved
    request rate and rays/s, and the highest achieved rate whose p99 stays within 33 ms."""
    rows = [{k: r.get(k) for k in ("offered_rps", "achieved_rps", "p50_ms", "p99_ms", "rays_per_s", "completed",
                                   "drained", "evictions", "restores", "evicted_gb", "restored_gb", "server_admit_s",
                                   "server_evict_s", "server_restore_s", "server_issue_s", "device_s",
                                   "host_pinned_gb", "host_pinned_grown_gb")}
            for r in sv["sweep"]]
    return {"workload": sv["config"]["workload"], "device_budget_gb": sv["config"]["device_budget_gb"],
            "offered_rps": [r["offered_rps"] for r in rows], "p50_ms": [r["p50_ms"] for r in rows],
            "p99_ms": [r["p99_ms"] for r in rows], "max_rps_p99_le_33ms": sv["max_rps_with_p99_le_33ms"],
            "rays_per_s": sv["value"], "evictions": sv["evictions"], "restores": sv["restores"],
            "resident_bytes": sv["resident_bytes"], "host_pinned_gb": sv["host_pinned_gb"], "sweep": rows,
            "build_s": sv["build_s"]}


def cpu_baseline_sample(vol, view, proj, W, H, seconds):
    """The oracle on the host cores, on this run's own map state: a pixel sample of the draw and a request
    sample of the lighting, timed with all threads.  Test infrastructure, measured, not shipped."""
    from oracle import oracle as O
    import doonengine_gb300 as dn
    from doonengine_gb300 import _lib
    lib = dn.load()
    ncores = os.cpu_count() or 1
    st, vis, _, ns = vol.export_tiles()
    reqs = vol.export_requests()
    idx, dif, spe = vol.export_lighting()
    om = O.OracleMap(vol.map_size)
    om.import_state(vol.s, st, vis, vol.s.frameNum)
    # the device's sample counts and lighting too: with zero counts every voxel would trace its first-sample
    # rays (one shadow ray instead of K), a lighter mix than the GPU's
    om.import_lighting(idx, dif, spe)
    om.import_samples(ns)
    om.set_requests(reqs)
    params = om.light_params(vol.s, 1, 1000, float(vol.s.lastTime))
    iv, icv, ip = _lib.DNmat4(), _lib.DNmat4(), _lib.DNmat4()
    lib.DN_draw_matrices(view, proj, iv, icv, ip)
    rng = np.random.default_rng(0)
    order = rng.permutation(len(reqs)).astype(np.uint32)
    pix = rng.choice(W * H, size=min(W * H, 1 << 16), replace=False).astype(np.uint32)
    om.reset_counters()
    t0 = time.perf_counter()
    om.draw(vol.s, iv, icv, ip, W, H, pixels=pix, nthreads=ncores)
    # the frame's request groups in a seeded order, passed over again (the same work: nothing is
    # committed) until the time budget is spent
    n, done, at, budget = 64, 0, 0, seconds
    while len(order) and time.perf_counter() - t0 < budget:
        chunk = order[at:at + n]
        om.light_requests(vol.s, params, chunk, nthreads=ncores)
        done += len(chunk)
        at = (at + len(chunk)) % len(order)
        n = min(n * 2, 1 << 14)
    el = time.perf_counter() - t0
    c = om.counters()
    om.close()
    return {"value": c["rays"] / el, "unit": "rays/s", "cores": ncores, "kind": "port",
            "sample": "%d pixels of the %dx%d draw + %d lighting request groups (%.2f passes over the last timed "
                      "frame's %d) (%d rays, %.1f s)" % (len(pix), W, H, done, done / max(1, len(order)), len(order),
                                                        c["rays"], el)}


# ------------------------------------------------------------ batched workload

def batched_vs_plain(args, lib, rank, pg, local, frames_warm, frames_timed, autotune=True):
    """The batched workload (64 maps of uneven size and resolution) in both forms on identical map state:
    two identical sets of maps built from the same seeds; every frame number runs the plain per-scene form
    on set A (each map's DN_draw, DN_sync_gpu, DN_update_lighting, DN_finish, one map at a time, as one GL
    context issues them) and the batched form on set B (DN_batch_run over all maps + DN_batch_finish).  Both
    sets therefore trace exactly the same rays in every frame (their counters are compared).  The first
    ``frames_warm`` frames cover the streaming ramp (chunks load one sync after a ray requests them); the
    next ``frames_timed`` are timed, each form by wall clock from issue to its results on the host, with
    the L2 flushed before each form's frame; the batched frames are also timed on the device."""
    import ctypes
    import doonengine_gb300 as dn
    from doonengine_gb300 import configs
    specs = configs.batched_specs(args.maps, seed=7 + 1000 * rank)
    sets = {"plain": [], "batched": []}
    t0 = time.perf_counter()
    tiles = nonempty = pixels = 0
    for form in ("plain", "batched"):
        for i, sp in enumerate(specs):
            vol, cfg = configs.build_volume("small", **sp)
            vol.s.mapId = i
            W, H = cfg["res"]
            img = dn.Image(W, H, on_device=True)
            v, p = vol.view_proj(H / W)
            sets[form].append((vol, img, v, p))
            if form == "plain":
                tiles += vol.num_tiles
                nonempty += vol.nonempty_chunks()
                pixels += W * H
    build_s = time.perf_counter() - t0
    log("built 2 x %d maps in %.1f s (%d tiles, %d non-empty chunks, %d pixels per frame per set)"
        % (len(specs), build_s, tiles, nonempty, pixels))
    A, B = sets["plain"], sets["batched"]
    batch = dn.Batch([m[0] for m in B])
    bstream = batch.stream()
    tuned = None

    def plain_frame(t):
        for vol, img, v, p in A:
            vol.draw(img, v, p)
            vol.sync(dn.DN_READ_WRITE, 1)
            vol.update_lighting(1, 1000, t)
            assert vol.finish(), lib.dn_cuda_last_error().decode()

    def batched_frame(t):
        batch.run([dn.Batch.item(vol, img, v, p, sync=(dn.DN_READ_WRITE, 1), light=(1, 1000, t)) for vol, img, v, p in B])
        assert batch.finish(), lib.dn_cuda_last_error().decode()

    for f in range(frames_warm):
        t = 1.0 + 0.25 * f
        plain_frame(t)
        batched_frame(t)
        if f == frames_warm - 1 and autotune:
            # tuned on the last warm-up frame's lighting, past the streaming ramp (the first frames light
            # almost nothing, so timings there say nothing about the timed frames)
            tuned = batch.autotune()
            log("autotuned: %s" % tuned)
    for vol, *_ in A:
        vol.reset_stats()
    batch.reset_stats()
    ev = [ctypes.c_void_p(), ctypes.c_void_p()]
    for e in ev:
        lib.dn_cuda_event_create(e)
    plain_s = batched_s = batched_dev_ms = 0.0
    launches = 0
    clocks = ClockSampler(local)
    barrier(pg)
    clocks.start()
    for k in range(frames_timed):
        t = 1.0 + 0.25 * (frames_warm + k)
        lib.dn_cuda_flush_l2(None, L2_FLUSH_BYTES)
        lib.dn_cuda_device_sync()
        t0 = time.perf_counter()
        plain_frame(t)
        plain_s += time.perf_counter() - t0
        lib.dn_cuda_flush_l2(bstream, L2_FLUSH_BYTES)
        lib.dn_cuda_device_sync()
        l0 = lib.dn_cuda_launch_count()
        t0 = time.perf_counter()
        lib.dn_cuda_event_record(ev[0], bstream)
        batch.run([dn.Batch.item(vol, img, v, p, sync=(dn.DN_READ_WRITE, 1), light=(1, 1000, t)) for vol, img, v, p in B])
        lib.dn_cuda_event_record(ev[1], bstream)
        assert batch.finish(), lib.dn_cuda_last_error().decode()
        batched_s += time.perf_counter() - t0
        launches += lib.dn_cuda_launch_count() - l0
        ms = ctypes.c_float()
        lib.dn_cuda_event_elapsed_ms(ev[0], ev[1], ms)
        batched_dev_ms += ms.value
    barrier(pg)
    clk = clocks.stop()
    pr = {"rays": 0, "litVoxels": 0, "primaryRays": 0}
    for vol, *_ in A:
        st = vol.stats()
        for key in pr:
            pr[key] += st[key]
    br = batch.stats()
    tuning = batch.tuning()
    batch.close()
    for form in sets.values():
        for vol, img, *_ in form:
            img.close()
            vol.close()
    for e in ev:
        lib.dn_cuda_event_destroy(e)
    rays_p = allreduce_sum(pg, pr["rays"])
    rays_b = allreduce_sum(pg, br["rays"])
    plain_s = allreduce_max(pg, plain_s)
    batched_s = allreduce_max(pg, batched_s)
    batched_dev_ms = allreduce_max(pg, batched_dev_ms)
    res_hist = {}
    for sp in specs:
        key = "%dx%d" % sp["res"]
        res_hist[key] = res_hist.get(key, 0) + 1
    return {
        "workload": "batched: %d maps, chunk dims U[8,64] per axis, non-empty fraction U[0.05,0.5], own seeded camera "
                    "each, resolutions 320x180..1920x1080, K=16, 1 diffuse path per voxel per frame" % len(specs),
        "maps": len(specs), "tiles": tiles, "nonempty_chunks": nonempty, "pixels_per_frame": pixels,
        "resolutions": res_hist,
        "method": "two identical map sets; each frame number runs the plain form on one and the batched form on the "
                  "other (same rays: counters compared); frames %d..%d timed after %d warm-up frames; wall clock from "
                  "issue to results on the host, L2 flushed before each form's frame"
                  % (frames_warm, frames_warm + frames_timed - 1, frames_warm),
        "plain_rays_per_s": rays_p / plain_s if plain_s else None,
        "batched_rays_per_s": rays_b / batched_s if batched_s else None,
        "batched_device_rays_per_s": rays_b / (batched_dev_ms / 1e3) if batched_dev_ms else None,
        "ratio": (rays_b / batched_s) / (rays_p / plain_s) if plain_s and batched_s and rays_p else None,
        "rays_per_frame": rays_b / frames_timed,
        "identical_rays": int(rays_p) == int(rays_b),
        "lit_voxels_per_frame": br["litVoxels"] / frames_timed,
        "plain_ms_per_frame": plain_s * 1e3 / frames_timed,
        "batched_ms_per_frame": batched_s * 1e3 / frames_timed,
        "batched_gpu_launches_per_frame": launches / frames_timed,
        "tuning": tuning, "autotuned": tuned is not None, "build_s": build_s, "clocks": clk,
        "plain_form": "per map: DN_draw, DN_sync_gpu, DN_update_lighting, DN_finish (one map at a time)",
        "batched_form": "DN_batch_run over all maps + DN_batch_finish per frame (CUDA graph replay)",
    }


def run_batched(args):
    """The batched workload as its own bench line (value = batched rays/s, wall clock, both forms on
    identical frames: batched_vs_plain)."""
    rank, world, local, pg = dist_setup()
    import doonengine_gb300 as dn
    lib = dn.load()
    if lib.dn_cuda_init(local) != 0:
        raise RuntimeError("dn_cuda_init(%d): %s" % (local, lib.dn_cuda_last_error().decode()))
    dn.init()
    r = batched_vs_plain(args, lib, rank, pg, local, args.warmup, args.steps, autotune=not args.no_autotune)
    result = {
        "metric": METRIC + " (batched)", "value": r["batched_rays_per_s"], "unit": "rays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["batched_ms_per_frame"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded heightfields; the reference publishes no scenes)",
        "config": {"workload": r["workload"], "maps": r["maps"], "tiles": r["tiles"],
                   "frame": "draw -> sync -> lighting for every map",
                   "l2": "flushed before each timed frame of each form (256 MiB write, outside the timed region)",
                   "parallelism": "replicas: own maps per GPU, no collective"},
        "batched_vs_plain": r, "gpu_launches": int(r["batched_gpu_launches_per_frame"] * args.steps),
        "clocks": r["clocks"],
    }
    if rank == 0:
        print(json.dumps(result), flush=True)


# ------------------------------------------------------------ streaming-edits workload

def catmull_rom(p, t):
    """Point at t in [0, 1] on the uniform Catmull-Rom spline through the rows of p (end points repeated)."""
    n = len(p) - 1
    x = min(max(t, 0.0), 1.0) * n
    i = min(int(x), n - 1)
    u = x - i
    p0, p1, p2, p3 = p[max(i - 1, 0)], p[i], p[i + 1], p[min(i + 2, n)]
    return 0.5 * ((2.0 * p1) + (-p0 + p2) * u + (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3) * u * u
                  + (-p0 + 3.0 * p1 - 3.0 * p2 + p3) * u * u * u)


def run_streaming(args):
    """One large map edited every frame: 1-512 chunks re-rolled, the camera on a seeded Catmull-Rom spline,
    and only edited, visible chunks relit (lighting split larger than any frame count, so the split
    filter never selects an unedited chunk)."""
    import ctypes
    rank, world, local, pg = dist_setup()
    import doonengine_gb300 as dn
    from doonengine_gb300 import configs
    lib = dn.load()
    if lib.dn_cuda_init(local) != 0:
        raise RuntimeError("dn_cuda_init(%d): %s" % (local, lib.dn_cuda_last_error().decode()))
    dn.init()
    t0 = time.perf_counter()
    seed = 31 + 1000 * rank
    vol, cfg = configs.build_volume("small", map=(128, 32, 128), seed=seed, mean=0.1, amp=0.05, shapes=0,
                                    res=(1280, 720), K=16, cam=(0.1, 0.8, 0.1, 25.0, 45.0))
    vol.s.mapId = rank
    build_s = time.perf_counter() - t0
    W, H = cfg["res"]
    sx, sy, sz = cfg["map"]
    flags = np.array([vol.s.map[t].flag for t in range(vol.num_tiles)], np.uint8)
    occ = np.nonzero(flags)[0]
    chunk_pos = np.stack([occ % sx, (occ // sx) % sy, occ // (sx * sy)], 1).astype(np.int32)
    nonempty = len(occ) / vol.num_tiles
    rng = np.random.default_rng(seed)
    ctrl = np.stack([rng.uniform(0.05, 0.95, 8) * sx, rng.uniform(0.6, 0.9, 8) * sy, rng.uniform(0.05, 0.95, 8) * sz], 1)
    total = args.warmup + args.steps
    split = 1 << 30
    img = dn.Image(W, H, on_device=True)
    stream = vol.stream()
    edits_per_frame = rng.integers(1, 513, size=total)
    frame = [0]

    def edit_and_camera(f):
        t = f / max(1, total - 1)
        p = catmull_rom(ctrl, t)
        q = catmull_rom(ctrl, min(1.0, t + 1e-3))
        d = q - p
        vol.s.camPos.x, vol.s.camPos.y, vol.s.camPos.z = float(p[0]), float(p[1]), float(p[2])
        vol.s.camOrient.x = 25.0
        vol.s.camOrient.y = float(np.degrees(np.arctan2(d[0], d[2])))
        n = int(edits_per_frame[f])
        sel = np.ascontiguousarray(chunk_pos[rng.integers(len(chunk_pos), size=n)])
        h0 = time.perf_counter()
        lib.dn_scene_reroll(vol.ptr, sel.ctypes.data, n, seed * 7919 + f, 14)
        return n, time.perf_counter() - h0

    host_sync = [0.0]

    def gpu_frame(f):
        v, p = vol.view_proj(H / W)
        vol.draw(img, v, p)
        h0 = time.perf_counter()
        vol.sync(dn.DN_READ_WRITE, split)          # host part: pack the edited chunks, stage one upload
        host_sync[0] += time.perf_counter() - h0
        vol.update_lighting(1, 1000, 1.0 + 0.25 * f)

    for f in range(args.warmup):
        edit_and_camera(f)
        gpu_frame(f)
    assert vol.finish(), lib.dn_cuda_last_error().decode()
    K = args.steps
    evs = []
    for _ in range(2 * K):
        e = ctypes.c_void_p()
        lib.dn_cuda_event_create(e)
        evs.append(e)
    vol.reset_stats()
    launches0 = lib.dn_cuda_launch_count()
    clocks = ClockSampler(local)
    barrier(pg)
    lib.dn_cuda_device_sync()
    clocks.start()
    t0 = time.perf_counter()
    host_edit_s, edited = 0.0, 0
    host_sync[0] = 0.0
    for k in range(K):
        f = args.warmup + k
        n, hs = edit_and_camera(f)
        host_edit_s += hs
        edited += n
        lib.dn_cuda_flush_l2(stream, L2_FLUSH_BYTES)
        lib.dn_cuda_event_record(evs[2 * k], stream)
        gpu_frame(f)
        lib.dn_cuda_event_record(evs[2 * k + 1], stream)
    assert vol.finish(), lib.dn_cuda_last_error().decode()
    lib.dn_cuda_device_sync()
    barrier(pg)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = lib.dn_cuda_launch_count() - launches0 - K
    ms = ctypes.c_float()
    dev_ms = 0.0
    for k in range(K):
        lib.dn_cuda_event_elapsed_ms(evs[2 * k], evs[2 * k + 1], ms)
        dev_ms += ms.value
    st = vol.stats()
    dev_ms_max = allreduce_max(pg, dev_ms)
    rays = allreduce_sum(pg, st["rays"])
    result = {
        "metric": METRIC + " (streaming edits)", "value": rays / (dev_ms_max / 1e3), "unit": "rays/s",
        "n_gpus": world, "steps": K, "warmup": args.warmup, "ms_per_step": dev_ms_max / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded heightfield; seeded chunk re-rolls)",
        "config": {"workload": "streaming edits: %dx%dx%d chunks (~%.0f%% non-empty), %dx%d draw, camera on a "
                               "seeded Catmull-Rom spline, 1-512 chunks re-rolled per frame, only edited and "
                               "visible chunks relit, K=16" % (sx, sy, sz, 100 * nonempty, W, H),
                   "map_chunks": [sx, sy, sz], "nonempty_chunk_frac": round(nonempty, 4), "frames": total,
                   "l2": "flushed between timed steps (256 MiB write, outside the timed events)",
                   "parallelism": "replicas: one map per GPU, no collective"},
        "lit_voxels_per_s": allreduce_sum(pg, st["litVoxels"]) / (dev_ms_max / 1e3),
        "primary_rays_per_s": allreduce_sum(pg, st["primaryRays"]) / (dev_ms_max / 1e3),
        "chunks_edited_per_step": edited / K, "host_edit_ms_per_step": host_edit_s * 1e3 / K,
        "host_sync_ms_per_step": host_sync[0] * 1e3 / K,
        "host_edit_note": "host_edit: the workload generating its edits (dn_scene_reroll re-rolls the voxels of the "
                          "chosen chunks through the edit API); host_sync: DN_sync_gpu's host part (%s)"
                          % ("packing of the edited chunks on the host, pool ranges, one pinned upload of the "
                             "packed voxels" if os.environ.get("DN_HOST_PACKING", "0") not in ("", "0") else
                             "the surface count of each edited chunk, pool ranges, one pinned upload of the "
                             "chunks' voxels; the packing itself runs on the device, k_pack_stage"),
        "packing": "host" if os.environ.get("DN_HOST_PACKING", "0") not in ("", "0") else "device",
        "wall_ms_per_step": wall * 1e3 / K, "build_s": build_s,
        "gpu_launches": int(allreduce_sum(pg, launches)), "clocks": clk,
    }
    img.close()
    vol.close()
    if rank == 0:
        print(json.dumps(result), flush=True)


# ------------------------------------------------------------ shapes workload

def shape_script(rng, map_size, n):
    """n seeded shape calls over the map: every kind, half extents 4-48 voxels, any orientation, a third of
    them removals (two thirds of those with flipped normals)"""
    X, Y, Z = (8 * s for s in map_size)
    ops = []
    for _ in range(n):
        kind = int(rng.integers(0, 8))
        c = tuple(float(x) for x in np.round(rng.uniform((0, 0, 0), (X, Y, Z)) * 4) / 4)
        v = tuple(float(x) for x in np.round(rng.uniform(4.0, 48.0, 3) * 4) / 4)
        a = float(np.round(rng.uniform(4.0, 48.0) * 4) / 4)
        b = float(np.round(rng.uniform(3.0, 40.0) * 4) / 4)
        if kind == 3:
            b = min(b, a - 1.0)
        removal = rng.random() < 1.0 / 3.0
        mat = 255 if removal else int(rng.integers(0, 16))
        ops.append(dict(kind=kind, c=c, v=v, a=a, b=b, orient=tuple(float(x) for x in rng.integers(0, 360, 3)),
                        voxel=(mat, (0.0, 1.0, 0.0), tuple(int(x) for x in rng.integers(0, 256, 3))),
                        flip=bool(removal and rng.random() < 2.0 / 3.0)))
    return ops


def run_shapes(args):
    """The shape functions as an edit source: each step places a script of 16 large shapes into a
    64x32x64-chunk map through DN_shape_* (device evaluation of every voxel of the covered chunks, host
    edits in the reference's order).  value: voxels evaluated per second of device time; e2e: the same
    per second of wall time through the public call (transform, evaluation, copy back, edits)."""
    import ctypes
    rank, world, local, pg = dist_setup()
    import doonengine_gb300 as dn
    lib = dn.load()
    if lib.dn_cuda_init(local) != 0:
        raise RuntimeError("dn_cuda_init(%d): %s" % (local, lib.dn_cuda_last_error().decode()))
    dn.init()
    map_size = (64, 32, 64)
    per_step = 16
    rng = np.random.default_rng(41 + 1000 * rank)
    vol = dn.Volume(map_size, 4096, cpu_only=True)
    total = args.warmup + args.steps
    script = [shape_script(rng, map_size, per_step) for _ in range(total)]

    def step(ops):
        for o in ops:
            vol.shape(o["kind"], o["voxel"], o["c"], o["v"], o["a"], o["b"], o["orient"], o["flip"])

    for f in range(args.warmup):
        step(script[f])
    vox = ctypes.c_uint64()
    dms = ctypes.c_double()
    lib.dn_cuda_shape_stats(vox, dms, 1)
    launches0 = lib.dn_cuda_launch_count()
    clocks = ClockSampler(local)
    barrier(pg)
    lib.dn_cuda_device_sync()
    clocks.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(script[args.warmup + k])
    lib.dn_cuda_device_sync()
    barrier(pg)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = lib.dn_cuda_launch_count() - launches0
    lib.dn_cuda_shape_stats(vox, dms, 0)
    voxels = allreduce_sum(pg, vox.value)
    dev_s = allreduce_max(pg, dms.value) / 1e3
    wall = allreduce_max(pg, wall)
    solid = int((vol.export_voxels()[0] >> 24 != 255).sum())
    result = {
        "metric": "shape voxels evaluated/s", "value": voxels / dev_s, "unit": "voxels/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded shape scripts)",
        "config": {"workload": "shapes: %d DN_shape_* calls per step (all 8 kinds, half extents 4-48 voxels, "
                               "random orientation, 1/3 removals) into a %dx%dx%d-chunk CPU map"
                               % ((per_step,) + map_size),
                   "map_chunks": list(map_size), "shapes_per_step": per_step,
                   "l2": "not flushed (each shape's evaluation reads only its parameters)",
                   "parallelism": "replicas: one map per GPU, no collective"},
        "voxels_evaluated_per_step": voxels / args.steps, "solid_voxels_after": solid,
        "e2e": {"value": voxels / wall, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": None, "path": "DN_shape_* (host transform + device evaluation + host edits)",
                "wall_ms_per_step": wall * 1e3 / args.steps},
        "gpu_launches": int(allreduce_sum(pg, launches)), "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = shapes_cpu_baseline(map_size, script[args.warmup], args.cpu_seconds)
    vol.close()
    if rank == 0:
        print(json.dumps(result), flush=True)


def shapes_cpu_baseline(map_size, ops, seconds):
    """the CPU oracle's restatement of the shape functions (evaluation + edits, one thread) on the first
    timed step's shapes, as many as fit in about the given seconds"""
    import doonengine_gb300 as dn
    from oracle import oracle as O
    lib = dn.load()
    from doonengine_gb300 import _lib as L
    d = O.DenseShapes(map_size)
    done = 0
    voxels = 0
    t0 = time.perf_counter()
    for o in ops:
        q = lib.DN_quaternion_from_euler(L.DNvec3(*o["orient"]))
        rot = lib.DN_quaternion_to_mat4(q)
        at = L.DNvec3(*o["c"])
        if o["kind"] == 6:
            up = lib.DN_mat4_mult_vec4(rot, L.DNvec4(0.0, 1.0, 0.0, 1.0))
            at = lib.DN_vec3_add(at, lib.DN_vec3_scale(L.DNvec3(up.x, up.y, up.z), o["b"]))
        t = lib.DN_mat4_mult(lib.DN_mat4_translate(at), rot)
        it = lib.DN_mat4_inv(t)
        tm = np.array([[t.m[c][r] for r in range(4)] for c in range(4)], np.float32)
        im = np.array([[it.m[c][r] for r in range(4)] for c in range(4)], np.float32)
        so = O.DenseShapes.op(o["kind"], int(o["flip"]), o["voxel"][0], o["voxel"][2], o["voxel"][1], o["c"], o["v"],
                              o["a"], o["b"], tm, im)
        ev = d.apply(so)
        if ev is not None:
            voxels += int(np.prod(ev[1] - ev[0] + 1)) * 512
        done += 1
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    return {"value": voxels / el, "unit": "voxels/s", "cores": 1, "kind": "port",
            "sample": "%d of the first timed step's %d shapes through the CPU oracle (evaluation + edits, %.1f s)"
                      % (done, len(ops), el)}


# ------------------------------------------------------------ serving workload

def serving_sweep(args, lib, rank, world, nmaps, rates, seconds, budget_gb, stop_at_saturation=True):
    """Poisson request streams over many resident maps through the serving loop (serve.h), swept over
    arrival rates: 70% draws, 25% relights of the visible chunks, 5% edit batches of 1-256 chunks.
    Returns the serving line (without printing it)."""
    import doonengine_gb300 as dn
    from doonengine_gb300 import configs
    specs = configs.serving_specs(nmaps, seed=11 + 1000 * rank)
    vols, views = [], []
    t0 = time.perf_counter()
    tiles = 0
    for i, sp in enumerate(specs):
        vol, cfg = configs.build_volume("small", **sp)
        vol.s.mapId = i
        vols.append(vol)
        tiles += vol.num_tiles
    build_s = time.perf_counter() - t0
    log("built %d maps in %.1f s (%d tiles)" % (len(vols), build_s, tiles))
    budget = int(budget_gb * (1 << 30))
    server = dn.Server(vols, budget_bytes=budget)
    # draw targets: a ring of device images per resolution (the bench does not read them back)
    ring = {r: [dn.Image(r[0], r[1], on_device=True, hit_info=True) for _ in range(args.image_ring)]
            for r in configs.RESOLUTIONS}
    ring_pos = {r: 0 for r in ring}
    vp = {}
    for i, vol in enumerate(vols):
        for r in ring:
            vp[(i, r)] = vol.view_proj(r[1] / r[0])
    rng = np.random.default_rng(1234 + rank)

    def make_requests(rate, seconds):
        n = int(rng.poisson(rate * seconds))
        offs = np.sort(rng.uniform(0.0, seconds, size=n))
        kinds = rng.choice(3, size=n, p=[0.70, 0.25, 0.05])
        which = rng.integers(len(vols), size=n)
        reqs = []
        for k, vi in zip(kinds, which):
            vi = int(vi)
            if k == 0:
                r = configs.RESOLUTIONS[int(rng.integers(len(configs.RESOLUTIONS)))]
                img = ring[r][ring_pos[r]]
                ring_pos[r] = (ring_pos[r] + 1) % len(ring[r])
                v, p = vp[(vi, r)]
                reqs.append(server.draw_request(vi, img, v, p, user=1))
            elif k == 1:
                reqs.append(server.relight_request(vi, 1, 1000, float(rng.uniform(0.0, 100.0)), user=2))
            else:
                sx, sy, sz = specs[vi]["map"]
                nch = int(rng.integers(1, 257))
                edits = []
                for _ in range(nch):
                    mp = (int(rng.integers(sx)), int(rng.integers(sy)), int(rng.integers(sz)))
                    for _ in range(4):
                        cp = tuple(int(c) for c in rng.integers(8, size=3))
                        edits.append((mp, cp, int(rng.integers(16)), (0.0, 1.0, 0.0),
                                      tuple(int(c) for c in rng.integers(40, 240, size=3)), False))
                reqs.append(server.edit_request(vi, edits, user=3))
        return reqs, offs

    server.start()
    pinned_start = lib.dn_cuda_host_pinned()
    # warm-up: every map drawn once and relit once
    warm = []
    for vi in range(len(vols)):
        r = specs[vi]["res"]
        v, p = vp[(vi, r)]
        warm.append(server.draw_request(vi, ring[r][0], v, p))
        warm.append(server.relight_request(vi, 1, 1000, 0.5))
    for q in warm:
        server.submit(q)
    assert server.drain(1800.0), "warm-up did not drain"
    server.poll()
    pinned_warm = lib.dn_cuda_host_pinned()
    sweep = []
    lib.DN_batch_reset_stats(lib.DN_server_batch(server.ptr))
    tot_rays, tot_s = 0, 0.0
    for rate in rates:
        reqs, offs = make_requests(rate, seconds)
        st0 = server.stats()
        b0 = server.batch_stats()
        pin0 = lib.dn_cuda_host_pinned()
        t0 = time.perf_counter()
        server.replay(reqs, offs)
        ok = server.drain(args.drain_timeout)
        el = time.perf_counter() - t0
        comps = server.poll()
        b1 = server.batch_stats()
        st1 = server.stats()
        lat = np.array([c["finished"] - c["arrival"] for c in comps]) * 1e3
        by_kind = {}
        for name, kind in (("draw", 0), ("relight", 1), ("edit", 2)):
            lk = np.array([c["finished"] - c["arrival"] for c in comps if c["kind"] == kind]) * 1e3
            if len(lk):
                by_kind[name] = {"n": int(len(lk)), "p50_ms": float(np.percentile(lk, 50)),
                                 "p99_ms": float(np.percentile(lk, 99))}
        rays = b1["rays"] - b0["rays"]
        tot_rays += rays
        tot_s += el
        row = {"offered_rps": rate, "requests": len(reqs), "completed": len(comps), "drained": bool(ok),
               "achieved_rps": len(comps) / el if el else None, "wall_s": el,
               "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
               "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
               "rays_per_s": rays / el if el else None, "by_kind": by_kind,
               "ticks": st1["ticks"] - st0["ticks"], "items": st1["items"] - st0["items"],
               "evictions": st1["evictions"] - st0["evictions"], "restores": st1["restores"] - st0["restores"],
               "evicted_gb": (st1["evictedBytes"] - st0["evictedBytes"]) / 2**30,
               "restored_gb": (st1["restoredBytes"] - st0["restoredBytes"]) / 2**30,
               "server_admit_s": st1["admitSeconds"] - st0["admitSeconds"],
               "server_issue_s": st1["issueSeconds"] - st0["issueSeconds"],
               "server_evict_s": st1["evictSeconds"] - st0["evictSeconds"],
               "server_restore_s": st1["restoreSeconds"] - st0["restoreSeconds"],
               "device_s": st1["deviceSeconds"] - st0["deviceSeconds"],
               "host_pinned_gb": lib.dn_cuda_host_pinned() / 2**30,
               "host_pinned_grown_gb": (lib.dn_cuda_host_pinned() - pin0) / 2**30}
        log("rate %g: %s" % (rate, {k: row[k] for k in ("completed", "achieved_rps", "p50_ms", "p99_ms", "rays_per_s",
                                                       "evictions", "restores", "server_admit_s", "server_evict_s",
                                                       "server_restore_s", "server_issue_s", "device_s",
                                                       "host_pinned_gb", "host_pinned_grown_gb")}))
        sweep.append(row)
        # past saturation the queue only grows: stop the sweep there
        if not ok or (row["achieved_rps"] or 0.0) < 0.9 * rate:
            row["saturated"] = True
            if stop_at_saturation:
                break
    st = server.stats()
    good = [r for r in sweep if r["p99_ms"] is not None and r["p99_ms"] <= 33.0 and r["drained"]]
    best = max(good, key=lambda r: r["achieved_rps"]) if good else None
    result = {
        "metric": METRIC + " (served)", "value": tot_rays / tot_s if tot_s else 0.0, "unit": "rays/s",
        "n_gpus": world, "steps": len(sweep), "warmup": 1, "ms_per_step": tot_s * 1e3 / max(1, len(sweep)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded heightfields; Poisson arrivals)",
        "config": {"workload": "serving: %d resident maps, chunk dims log-uniform 8^3..96x32x96, requests 70%% draw "
                               "(320x180..1920x1080) / 25%% relight / 5%% edit batches of 1-256 chunks, Poisson "
                               "arrivals swept over %s req/s, %.0f s each"
                               % (len(vols), ",".join("%g" % r for r in rates), seconds),
                   "maps": len(vols), "tiles": tiles, "device_budget_gb": budget_gb,
                   "parallelism": "replicas: own maps per GPU, no collective"},
        "sweep": sweep,
        "max_rps_with_p99_le_33ms": best["achieved_rps"] if best else None,
        "resident_bytes": st["residentBytes"], "resident_maps": st["residentVolumes"],
        "evictions": st["evictions"], "restores": st["restores"], "build_s": build_s,
        "host_pinned_gb": {"after_start": pinned_start / 2**30, "after_warmup": pinned_warm / 2**30,
                           "end": lib.dn_cuda_host_pinned() / 2**30},
    }
    server.close()
    for imgs in ring.values():
        for im in imgs:
            im.close()
    for v in vols:
        v.close()
    return result


def run_serving(args):
    rank, world, local, pg = dist_setup()
    import doonengine_gb300 as dn
    lib = dn.load()
    if lib.dn_cuda_init(local) != 0:
        raise RuntimeError("dn_cuda_init(%d): %s" % (local, lib.dn_cuda_last_error().decode()))
    dn.init()
    rates = [float(x) for x in args.rates.split(",")]
    result = serving_sweep(args, lib, rank, world, args.maps, rates, args.seconds, args.budget_gb)
    if rank == 0:
        print(json.dumps(result), flush=True)


# ------------------------------------------------------------ reference arm

def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import doonengine_gb300 as dn
    from doonengine_gb300 import configs, _lib
    from oracle import oracle as O
    lib = dn.load()
    ncores = os.cpu_count() or 1
    vol, cfg = configs.build_volume(args.config, cpu_only=True)
    nonempty = vol.nonempty_chunks() / vol.num_tiles
    W, H = cfg["res"]
    view, proj = vol.view_proj(H / W)
    iv, icv, ip = _lib.DNmat4(), _lib.DNmat4(), _lib.DNmat4()
    lib.DN_draw_matrices(view, proj, iv, icv, ip)
    om = O.OracleMap(vol.map_size)
    rng = np.random.default_rng(0)
    pix_n = args.ref_pixels if args.ref_pixels > 0 else W * H
    req_cap = args.ref_requests if args.ref_requests > 0 else None

    def clear_updated():
        # the product's DN_sync_gpu clears 'updated' after streaming (voxel.c:1534); the oracle only reads it
        for i in range(vol.s.chunkCap):
            if vol.s.chunks[i].updated:
                vol.s.chunks[i].updated = False

    def frame(f):
        if pix_n >= W * H:
            om.draw(vol.s, iv, icv, ip, W, H, nthreads=ncores)
        else:
            pix = rng.choice(W * H, size=pix_n, replace=False).astype(np.uint32)
            om.draw(vol.s, iv, icv, ip, W, H, pixels=pix, nthreads=ncores)
        om.sync(vol.s, 2, 1)
        clear_updated()
        reqs = om.requests()
        if req_cap is None:
            # the whole lighting update, committed like DN_update_lighting's (sample counts grow, so later
            # frames trace K shadow rays per voxel instead of the first sample's one): the GPU arm's work
            om.light(vol.s, 1, 1000, 1.0 + 0.25 * f, nthreads=ncores)
        else:
            p = om.light_params(vol.s, 1, 1000, 1.0 + 0.25 * f)
            sel = rng.permutation(len(reqs))[:req_cap].astype(np.uint32)
            if len(sel):
                om.light_requests(vol.s, p, sel, nthreads=ncores)
        return len(reqs)

    for f in range(args.warmup):
        frame(f)
    om.reset_counters()
    groups = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        groups += frame(args.warmup + k)
    el = time.perf_counter() - t0
    c = om.counters()
    value = c["rays"] / el
    if pix_n >= W * H and req_cap is None:
        sample = ("per step: the whole frame, the same work as the GPU arm's step of the same number: all %dx%d "
                  "pixels of the draw and all %.0f lighting request groups of the frame (mean), the CPU "
                  "restatement of the reference shaders with OpenMP" % (W, H, groups / max(1, args.steps)))
    else:
        sample = ("per step: %d sampled pixels of the %dx%d draw + %s sampled lighting request groups, the CPU "
                  "restatement of the reference shaders with OpenMP" % (pix_n, W, H, req_cap if req_cap else "all"))
    result = {"metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
              "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
              "data": "synthetic (seeded heightfield + boxes/spheres)", "impl": "reference",
              "config": workload_desc(cfg, vol, nonempty, args.config),
              "cpu_baseline": {"value": value, "unit": "rays/s", "cores": ncores, "kind": "port", "sample": sample},
              "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
              "rays_per_step": c["rays"] / args.steps,
              "rays_by_kind_per_step": {"primary": c["primary"] / args.steps,
                                        "lighting": (c["rays"] - c["primary"]) / args.steps},
              "note": "the reference path runs only as GLSL through OpenGL, which is unavailable on this box; "
                      "this arm times the CPU restatement of its algorithm"}
    om.close()
    vol.close()
    print(json.dumps(result), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=24)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="large")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-pixels", type=int, default=0, help="pixels per reference step (0 = the full image)")
    ap.add_argument("--ref-requests", type=int, default=0,
                    help="lighting request groups per reference step (0 = all of the frame's, the GPU arm's mix)")
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "serving", "streaming", "shapes"],
                    help="plain: one map per step (the headline); batched: many maps per step")
    ap.add_argument("--maps", type=int, default=64, help="maps of the batched workload")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--residency", default="keep", choices=["keep", "lru"],
                    help="plain workload: chunk residency (DN_set_residency); lru = the reference's voxel-buffer nodes")
    ap.add_argument("--rates", default="100,200,300,400,500,600,700,850,1000,1100,1200,1300,1400,1500,2000,5000,10000,20000",
                    help="serving: offered req/s, swept upwards until the server saturates")
    ap.add_argument("--seconds", type=float, default=4.0, help="serving: seconds of arrivals per rate")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="serving: device budget")
    ap.add_argument("--image-ring", type=int, default=16, help="serving: draw targets per resolution")
    ap.add_argument("--drain-timeout", type=float, default=20.0)
    ap.add_argument("--no-batched", action="store_true", help="plain workload: skip the batched-vs-plain part")
    ap.add_argument("--no-serving", action="store_true", help="plain workload: skip the serving parts")
    ap.add_argument("--batched-warmup", type=int, default=8, help="plain workload's batched part: warm-up frames")
    ap.add_argument("--batched-frames", type=int, default=4, help="plain workload's batched part: timed frames")
    ap.add_argument("--serving-rates", default="500,800,1000,1200,1400,1600,2000",
                    help="plain workload's serving part: offered req/s")
    ap.add_argument("--serving-seconds", type=float, default=2.0, help="plain workload's serving part: s per rate")
    ap.add_argument("--pressure-budget-gb", type=float, default=60.0,
                    help="plain workload: a second serving sweep under this device budget (below the resident "
                         "set, so whole maps are evicted to pinned host memory under load); 0 skips it")
    ap.add_argument("--pressure-rates", default="300,600,900", help="offered req/s of the eviction sweep")
    ap.add_argument("--pressure-seconds", type=float, default=4.0,
                    help="plain workload's eviction sweep: s per rate (which maps are evicted depends on timing, "
                         "so its tail latency needs more requests than the resident sweep's)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3 (at least three untimed steps)")
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "streaming":
        run_streaming(args)
    elif args.workload == "shapes":
        run_shapes(args)
    elif args.workload == "serving":
        if args.maps == 64:
            args.maps = 256
        run_serving(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
