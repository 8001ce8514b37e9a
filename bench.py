#!/usr/bin/env python3
"""4K frames/s of the plain per-frame rasterization path on GB300.

Workload (default): 2,000,000 triangles in seeded icospheres and displaced
grids (per-object triangle screen area log-uniform over 0.5-5000 px, ~15% of
objects straddling the near plane or a frustum side), 8 value-noise textures
of 2048^2 with full mip chains, one 3840x2160 view. Seeded synthetic data:
no glTF sample assets exist on this machine.

A step is one frame: render_scene + update_auto_exposure(dt = 0) + resolve to
RGBA8 and the visibility buffer, all resident in HBM (`value`). `e2e` is the
same metric through the C ABI with host buffers: every step also copies the
RGBA8 frame and the visibility buffer into pinned host memory.

--impl reference times the CPU restatement of the reference's rayon path (the
oracle) on the host cores over the same workload.

Multi-GPU: frames are independent, so N GPUs run N replicas (weak scaling, no
collective on the data path); rank 0 prints the line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "swraster-viewer_gb300"))

KERNELS_PER_FRAME = 7  # reset, frontend, clip, scan, scatter, raster, shade


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="4k", choices=["4k", "small"])
    ap.add_argument("--cpu-frames", type=int, default=3, help="frames in the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sched-tile", type=int, default=0,
                    help="raster scheduling tile (8, 16, 32, 64; 0 = the library's choice for the frame size)")
    ap.add_argument("--fused-shade", action="store_true",
                    help="served: 32-px tiles shade inside the raster kernel (with --sched-tile 32)")
    ap.add_argument("--gi", action="store_true",
                    help="plain mode: bake the voxel GI at load (the reference's --gi) and shade with it")
    ap.add_argument("--mode", default="plain", choices=["plain", "batched", "hetero", "served"],
                    help="plain: 4K per-frame path (the headline); batched: 64 views of the 81,920-triangle scene "
                         "in one launch; hetero: 16 heterogeneous scenes in one launch; served: request loop")
    ap.add_argument("--rates", default="100,500,1000,2000,3000,5000", help="served arrival rates (requests/s)")
    ap.add_argument("--inflight", type=int, default=3, help="served: batches in flight (one engine and stream each)")
    ap.add_argument("--max-batch", type=int, default=64, help="served: views per batch")
    ap.add_argument("--no-graph", dest="graph", action="store_false",
                    help="served: launch each batch's kernels directly instead of replaying a captured graph")
    ap.add_argument("--seconds", type=float, default=2.0, help="served: arrival window per rate")
    ap.add_argument("--max-tris", type=int, default=0, help="hetero/served: cap on triangles per scene")
    return ap.parse_args()


def workload(name):
    import scenes
    if name == "4k":
        sd, cam = scenes.stress_scene()
        cfg = {"workload": "plain 4K: 2M triangles (icospheres + displaced grids, log-uniform 0.5-5000 px "
                           "triangles), 8x 2048^2 RGBA8 textures, 3840x2160, 64-px tiles",
               "triangles": 2000000, "width": 3840, "height": 2160}
        return sd, cam, cfg
    sd = scenes.spheres_scene()
    return sd, None, {"workload": "plain small: 64 icospheres (81,920 triangles), 256^2 texture, 1280x720",
                      "triangles": 81920, "width": 1280, "height": 720}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, world, device="cuda"):
    """The largest of a per-rank float over all ranks (itself for one rank)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world, units_per_rank, ms_max):
    """Whole-job rate over replicas: the units every rank processed divided by
    the slowest rank's time."""
    return world * units_per_rank / (ms_max / 1000.0)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # nvidia-smi's start-up (NVML initialisation) stalls the process's
        # CUDA calls for a while: let it finish before the timed region.
        t0 = time.time()
        while time.time() - t0 < 10.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for i, n in enumerate(names):
                if r[5 + i].strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(sd, cam_params, cfg, frames, threads=None, warmup=1):
    """The oracle (CPU restatement of the reference's rayon path) on all host
    cores over a bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import scenes
    import swr
    oracle.build()
    threads = threads or os.cpu_count()
    s = swr.Scene(sd, host_only=True)
    cam = swr.make_camera(*cam_params) if cam_params else swr.make_camera(
        *scenes.default_camera_params(s.info(), cfg["width"], cfg["height"]))
    view = s.export()
    for _ in range(warmup):
        oracle.render(view, cam, cfg["width"], cfg["height"], threads=threads)
    t0 = time.perf_counter()
    for _ in range(frames):
        oracle.render(view, cam, cfg["width"], cfg["height"], threads=threads)
    dt = time.perf_counter() - t0
    s.close()
    return frames / dt, threads, "%d frames of the full workload" % frames


def run_reference(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return 0
    sd, cam_params, cfg = workload(args.workload)
    # Bounded sample: at most 20 timed and 3 warm-up frames (a 4K frame takes
    # about 0.3 s on 16 Grace cores).
    steps = max(1, min(args.steps, 20))
    warm = max(1, min(args.warmup, 3))
    fps, cores, sample = cpu_baseline(sd, cam_params, cfg, steps, warmup=warm)
    line = {"metric": "4K frames/s" if args.workload == "4k" else "frames/s", "value": fps, "unit": "frames/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": 1000.0 / fps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": cfg,
            "gtri_per_s": fps * cfg["triangles"] / 1e9,
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _timed(torch, fn, reps):
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(reps):
        fn()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_batched(args, hetero):
    """One launch sequence for many views vs the same views rendered one per
    frame by the plain path, on the same GPU."""
    import numpy as np
    import torch
    import scenes
    import swr
    sh = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(3)
    if hetero:
        items = []
        for sd, cp in scenes.hetero_scenes(max_triangles=args.max_tris or None):
            s = swr.Scene(sd)
            items.append((s, swr.make_camera(*cp), cp[3], cp[4]))
        cfg = {"workload": "16 heterogeneous scenes (10k-4M triangles log-uniform, 1-8 textures of 512-2048 px), "
                           "one view each at 640x480-3840x2160, all in one launch",
               "views": len(items), "triangles": int(sum(s.info().triangle_count for s, *_ in items))}
    else:
        s = swr.Scene(scenes.spheres_scene())
        res = [(320, 240), (640, 480), (1280, 720), (1920, 1080)]
        items = []
        for i in range(64):
            w, h = res[int(rng.integers(4))]
            items.append((s, swr.make_camera(*scenes.sphere_camera(rng, s.info(), w, h)), w, h))
        cfg = {"workload": "64 views of the 81,920-triangle sphere scene on a sphere of radius 15-40, resolutions "
                           "from {320x240, 640x480, 1280x720, 1920x1080}, one launch", "views": 64,
               "triangles": 81920 * 64}
    px = sum(w * h for _, _, w, h in items)
    b = swr.Batch(use_graph=True)
    arr = swr.Batch.views([(sc, cam, w, h, 2.0, swr.RSQRT_AARCH64) for sc, cam, w, h in items])
    tile, _ = b.autotune(arr, sh)
    for _ in range(max(3, args.warmup)):
        b.render(arr, sh)
    b.sync()
    def one():
        b.render(arr, sh)
    ms_batch = _timed(torch, one, args.steps)
    b.sync()
    # Plain path: one renderer per resolution, views one after another.
    rends = {}
    for sc, cam, w, h in items:
        if (w, h) not in rends:
            rends[(w, h)] = swr.Renderer(w, h)
    def seq():
        for sc, cam, w, h in items:
            rends[(w, h)].render(sc, cam, 0.0, sh)
    for _ in range(2):
        seq()
    ms_seq = _timed(torch, seq, max(3, args.steps // 4))
    for r in rends.values():
        r.close()
    n = len(items)
    line = {"metric": "batched views/s", "value": n / (ms_batch / 1000.0), "unit": "views/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_batch,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": dict(cfg, sched_tile=tile, graph=True),
            "plain_sequential": {"value": n / (ms_seq / 1000.0), "unit": "views/s", "ms_per_batch": ms_seq},
            "speedup_vs_plain": ms_seq / ms_batch, "gpix_per_s": px / (ms_batch / 1000.0) / 1e9,
            "gpu_launches": KERNELS_PER_FRAME * args.steps}
    print(json.dumps(line), flush=True)
    b.close()
    return 0


def run_served(args):
    """Poisson request stream over 8 resident scenes: served form (continuous
    batching) vs the plain per-frame path (one request at a time, FIFO)."""
    import threading
    import numpy as np
    import torch
    import scenes
    import swr
    sh = torch.cuda.current_stream().cuda_stream
    scs = [swr.Scene(sd) for sd, _ in scenes.hetero_scenes(seed=31, count=8, max_triangles=args.max_tris or None)]
    res = [(640, 480), (1280, 720), (1920, 1080), (3840, 2160)]
    srv = swr.Server(memory_budget=40 << 30, max_batch_views=args.max_batch, inflight=args.inflight,
                     use_graph=args.graph, sched_tile=args.sched_tile, fused_shade=args.fused_shade)
    ids = [srv.add_scene(s) for s in scs]
    rends = {r: swr.Renderer(r[0], r[1]) for r in res}
    results = {}
    for rate in [float(x) for x in args.rates.split(",")]:
        rng = np.random.default_rng(int(rate))
        n = max(20, min(int(rate * args.seconds), 4000))
        gaps = rng.exponential(1.0 / rate, n)
        reqs = []
        for i in range(n):
            k = int(rng.integers(len(scs)))
            w, h = res[int(rng.integers(len(res)))]
            cam = swr.make_camera(*scenes.sphere_camera(rng, scs[k].info(), w, h, 0.7 * scs[k].info().bounds_diagonal,
                                                        1.5 * scs[k].info().bounds_diagonal))
            reqs.append((k, cam, w, h))
        # Served.
        lat = []
        bviews = []
        done = [0]
        def submit():
            t0 = time.perf_counter()
            t = t0
            for i, (k, cam, w, h) in enumerate(reqs):
                t += gaps[i]
                d = t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                while srv.submit(ids[k], cam, w, h, 2.0, tag=i) is None:
                    time.sleep(0.0005)
        th = threading.Thread(target=submit)
        t_start = time.perf_counter()
        th.start()
        while done[0] < n:
            for c in srv.poll(256, wait_ms=5):
                lat.append(c.latency_ms)
                bviews.append(c.batch_views)
                srv.release(c.ticket)
                done[0] += 1
        t_end = time.perf_counter()
        th.join()
        served = {"completed": n, "frames_per_s": n / (t_end - t_start), "p50_ms": float(np.percentile(lat, 50)),
                  "p99_ms": float(np.percentile(lat, 99)), "mean_batch_views": float(np.mean(bviews))}
        # Plain path: the same arrivals, served one at a time in order.
        plat = []
        t0 = time.perf_counter()
        arr_t = t0 + np.cumsum(gaps)
        for i, (k, cam, w, h) in enumerate(reqs):
            d = arr_t[i] - time.perf_counter()
            if d > 0:
                time.sleep(d)
            r = rends[(w, h)]
            r.render(scs[k], cam, 0.0, sh)
            r.sync()
            plat.append((time.perf_counter() - arr_t[i]) * 1000.0)
        t1 = time.perf_counter()
        plain = {"frames_per_s": n / (t1 - t0), "p50_ms": float(np.percentile(plat, 50)),
                 "p99_ms": float(np.percentile(plat, 99))}
        results[str(int(rate))] = {"served": served, "plain": plain}
    st = srv.stats()
    line = {"metric": "served frames/s + p99 latency vs plain GPU", "unit": "frames/s", "n_gpus": 1,
            "config": {"workload": "8 resident scenes (10k-4M triangles), Poisson arrivals, random scene, camera on "
                                   "a sphere, resolution from {640x480, 1280x720, 1920x1080, 3840x2160}, 40 GB "
                                   "budget, continuous batching",
                       "triangles": int(sum(s.info().triangle_count for s in scs)), "inflight": args.inflight,
                       "max_batch_views": args.max_batch, "graph": bool(args.graph),
                       "sched_tile": args.sched_tile, "fused_shade": bool(args.fused_shade)},
            "rates": results, "batches": st.batches, "device_bytes": st.device_bytes, "data": "synthetic"}
    best_served = max((v["served"]["frames_per_s"] for v in results.values()), default=0.0)
    best_plain = max((v["plain"]["frames_per_s"] for v in results.values()), default=0.0)
    line["value"] = best_served
    line["plain_max_frames_per_s"] = best_plain
    line["speedup_vs_plain"] = best_served / best_plain if best_plain else None
    # Equal p99: the most frames/s each side delivered at a rate whose p99
    # latency stayed within the bound.
    eq = {}
    for bound in (50.0, 100.0, 250.0):
        s_ok = [v["served"]["frames_per_s"] for v in results.values() if v["served"]["p99_ms"] <= bound]
        p_ok = [v["plain"]["frames_per_s"] for v in results.values() if v["plain"]["p99_ms"] <= bound]
        sb, pb = max(s_ok, default=0.0), max(p_ok, default=0.0)
        eq["p99<=%dms" % bound] = {"served": sb, "plain": pb, "ratio": sb / pb if pb else None}
    line["at_equal_p99"] = eq
    print(json.dumps(line), flush=True)
    srv.close()
    for r in rends.values():
        r.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.mode in ("batched", "hetero", "served"):
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if args.mode == "served":
            return run_served(args)
        return run_batched(args, args.mode == "hetero")
    world, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import scenes
    import swr
    sd, cam_params, cfg = workload(args.workload)
    W, H = cfg["width"], cfg["height"]
    scene = swr.Scene(sd, gi=args.gi)
    if args.gi:
        cfg = dict(cfg, workload=cfg["workload"] + ", baked voxel GI", gi=True)
    cam = swr.make_camera(*cam_params) if cam_params else swr.make_camera(
        *scenes.default_camera_params(scene.info(), W, H))
    r = swr.Renderer(W, H, sched_tile=args.sched_tile)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(max(3, args.warmup)):
        r.render(scene, cam, 0.0, sh)
    r.sync()
    st = r.stats()
    # Timed region: K frames, device-resident (inputs > L2: the scene is
    # ~265 MB and each frame writes 100 MB of outputs).
    clocks = Clocks(local)
    clocks.start()
    r.set_profiling(True)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        r.render(scene, cam, 0.0, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    r.sync()
    prof, nprof = r.profile()
    r.set_profiling(False)
    clk = clocks.stop()
    ms = max_over_ranks(ms, world)
    fps = aggregate_rate(world, args.steps, ms)
    # End to end through the C ABI with host buffers (pinned): each step is
    # the reference's frame, render_scene + update_auto_exposure +
    # blit_to_buffer, with the RGBA8 framebuffer in host memory when the
    # blit returns. Headline: the framebuffer is the renderer's blit target,
    # so the shading pass writes it over the host link and the blit waits;
    # also reported: the blit copying it after the frame.
    rgba_h = torch.empty((H, W), dtype=torch.int32, pin_memory=True)
    import ctypes as C
    L = swr.lib()
    e2e_steps = max(5, args.steps // 4)

    def e2e_run():
        barrier()
        torch.cuda.synchronize()
        e2 = torch.cuda.Event(enable_timing=True)
        e3 = torch.cuda.Event(enable_timing=True)
        e2.record(stream)
        for _ in range(e2e_steps):
            r.render(scene, cam, 0.0, sh)
            swr.check(L.swr_blit(r.handle, C.c_void_p(rgba_h.data_ptr()), W, sh))
        e3.record(stream)
        torch.cuda.synchronize()
        barrier()
        return aggregate_rate(world, e2e_steps, max_over_ranks(e2.elapsed_time(e3), world))

    e2e_copy_fps = e2e_run()
    r.set_blit_target(rgba_h.data_ptr(), W, keep=rgba_h)
    e2e_fps = e2e_run()
    r.set_blit_target(None)
    h2d = st.staged_bytes  # per-frame tables: scene/view headers, draws, chunks
    d2h = W * (H & ~1) * 4
    # Roofline for the dominant kernel (HBM: shading reads the 8-B depth key
    # and writes 4-B RGBA8 + 8-B visibility ID per pixel).
    dom = max(("raster", "shade", "frontend"), key=lambda k: prof[k])
    px = W * H
    # raster: bins read (4 B/pair), raster records read (80 B/emitted triangle), depth keys
    # written (8 B per pixel of the 64-px tile grid).
    alg = {"shade": 20.0 * px, "raster": 4.0 * st.bin_pairs + 80.0 * st.setup_triangles + 8.0 * st.tiles * 4096,
           "frontend": 12.0 * st.triangles_in + 48.0 * 3 * st.triangles_in + 256.0 * st.setup_triangles}[dom]
    peak, peak_kind = peaks()
    achieved = alg / (prof[dom] / 1000.0) / 1e9
    traffic = None
    issue = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        tj = json.load(open(tp))
        traffic = tj.get(args.workload, {}).get(dom)
        # The kernel is bound by instruction issue, not HBM: warp instructions
        # per launch (from the ncu capture) over the live duration, against
        # 4 issue slots per SM per cycle at the sampled clock.
        winst = tj.get("warp_instructions", {}).get(args.workload, {}).get(dom)
        if winst and clk.get("sm_mhz"):
            import torch
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            ach = winst / (prof[dom] / 1000.0)
            pk = 4.0 * sms * clk["sm_mhz"] * 1e6
            issue = {"kernel": dom, "warp_instructions_per_launch": winst, "achieved": ach, "peak": pk,
                     "unit": "warp instructions/s", "frac": ach / pk}
    line = {"metric": "4K frames/s" if args.workload == "4k" else "frames/s", "value": fps, "unit": "frames/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene of the configured shape; inputs larger than L2)",
            "config": dict(cfg, parallelism="replicas" if world > 1 else "single", sched_tile=st.sched_tile),
            "gtri_per_s": fps * cfg["triangles"] / 1e9, "gpix_per_s": fps * W * H / 1e9,
            "stage_ms": {k: round(v, 4) for k, v in prof.items()},
            "frame_stats": {"triangles_in": st.triangles_in, "clipped": st.triangles_clipped,
                            "setup_triangles": st.setup_triangles, "bin_pairs": st.bin_pairs,
                            "culled_pairs": st.culled_pairs},
            "issue_roofline": issue,
            "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes": alg},
            "clocks": clk,
            "gpu_launches": KERNELS_PER_FRAME * args.steps,
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "blit": "shading pass writes the pinned host framebuffer (swr_renderer_set_blit_target)",
                    "copy_blit_value": e2e_copy_fps}}
    if rank == 0 and not args.no_cpu_baseline:
        v, cores, sample = cpu_baseline(sd, cam_params, cfg, args.cpu_frames)
        line["cpu_baseline"] = {"value": v, "unit": "frames/s", "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    r.close()
    scene.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
