"""Benchmark of the GB300 path tracer on the ReSTIR workload.

Workload ("Plain method with ReSTIR"): 4x4 chunks (128x32x128 blocks) of the
seeded value-noise heightfield, 0.5% emissive surface blocks, 1920x1080,
64-frame orbit camera path, 3 bounces, light-BVH NEE, ReSTIR with 1 temporal
neighbour (1-slot history), 3 spatial neighbours in a 30-px box, M-cap 20,
FP32 reservoirs.  One step = one frame.

Metric: Mrays/s (closest-hit queries + light any-hit queries issued, the
reference's own ray count) with ms/frame.  `value` is device-timed (CUDA
events on the library stream, scene and frame state resident in HBM);
`e2e` is the same metric through the public C ABI with the frame copied back
to host memory inside the timed region.

--impl reference times the reference's CPU path (the oracle restatement,
OpenMP over pixels on every host core) on a bounded pixel sample of the same
workload.  With N > 1 ranks (torchrun) the frames are rendered by N
independent replicas (the path has no exchange step) and rank 0 prints one
line with the whole-job throughput.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "vulkan-voxel-restir-gi_gb300"))

METRIC = "Mrays/s and ms/frame @1080p ReSTIR; relMSE vs FP64 GT, cache vs plain at equal time"
SEED = 20240601
NX = NZ = 4
EMISSIVE = 0.005
W, H, NB = 1920, 1080, 3
ORBIT = 64


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.ws)
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, window=None):
        """Summary of the samples taken inside window = (t0, t1) (perf_counter
        seconds; all samples if none fell inside it)."""
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = [ln for t, ln in self.lines if window is None or window[0] <= t <= window[1]]
        if not lines:
            lines = [ln for _, ln in self.lines]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


class OracleSampler:
    """The oracle (CPU restatement of the reference's path, OpenMP over pixels)
    on the same workload: world built once, then frames of the orbit rendered
    with `rows` image rows around the centre traced per frame."""

    def __init__(self, world, mats, n, rows):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        t0 = time.perf_counter()
        self.ow = oracle.build_world(mats, n, world)  # meshing, light extraction, SAH builds, commit
        self.build_s = time.perf_counter() - t0
        self.orr = oracle.Renderer(W, H, NB)
        self.rows = min(rows, H)

    def frame(self, f):
        """Renders orbit frame f; returns (seconds, rays)."""
        import oracle
        import vrg  # struct layouts only
        cam = oracle.orbit_camera(NX, NZ, f % ORBIT, ORBIT, W, H)
        p = vrg.RenderParams(1, 1, 3, NB, vrg.MODE_CONFIG, f, 1000 + f, 2000 + f, 30.0, 20, 1, 0, 0)
        y0 = H // 2 - self.rows // 2
        t0 = time.perf_counter()
        self.orr.render(self.ow, cam, p, (y0 * W, (y0 + self.rows) * W))
        dt = time.perf_counter() - t0
        a, b = self.orr.ray_counts()
        return dt, a + b

    def close(self):
        self.orr.close()
        self.ow.close()


def oracle_sample(world, mats, n, rows, frames=1, start_frame=0):
    """Returns (Mrays/s, seconds, rays, scene build seconds) of `frames` oracle frames."""
    smp = OracleSampler(world, mats, n, rows)
    dt, rays = 0.0, 0
    for f in range(frames):
        t, r_ = smp.frame(start_frame + f)
        dt += t
        rays += r_
    smp.close()
    return rays / dt / 1e6, dt, rays, smp.build_s


# The k_trace DRAM traffic comes from a committed ncu capture of the current
# build (dram__bytes_read.sum + dram__bytes_write.sum per launch at 960x540,
# the command that made it stored beside the figures); it is scaled to the
# bench's extent by the pixel count.  The 1080p launches are too large to
# capture with many metrics.
TRACE_PROFILE = os.path.join(ROOT, "profiles", "k_trace_dram_restir540p.json")


def trace_traffic_per_launch(pixels, bounces):
    """(DRAM bytes per k_trace launch scaled to `pixels`, source string), or (None, reason)."""
    try:
        with open(TRACE_PROFILE) as f:
            prof = json.load(f)
    except (OSError, ValueError) as e:
        return None, f"no committed k_trace profile ({e.__class__.__name__})"
    per_frame = sum(prof["dram_bytes_per_launch"])  # one launch per bounce
    scale = pixels / float(prof["pixels"])
    return round(per_frame * scale / bounces), (
        f"ncu dram__bytes_read.sum+dram__bytes_write.sum of k_trace at {prof['resolution']} "
        f"({prof['build']}), scaled by pixels, per launch")


C3_N = 8  # chunks per side of the learned-cache workload
E2E_SLOTS = 4  # host image buffers of the end-to-end loop (frames in flight)
REF_MAX_FRAMES = 48  # full 1080p frames the reference arm times on the host cores

C2_SEED = 20240602
C2_SCENES = 64
C2_RES = [(256, 256), (640, 480), (1280, 720), (1920, 1080)]


def batched_block(ctx, steps, warmup, tuning=None):
    """Batched workload: 64 independent scenes, chunk grids drawn from 1x1..8x8
    and resolutions from {256^2, 640x480, 1280x720, 1920x1080}, each with its
    own terrain seed and orbit camera, 2 bounces + ReSTIR (1 temporal, 3
    spatial, 30 px, M-cap 20).  All chunks of all scenes are built by one
    batched BLAS build; one step = one frame of every view, replayed from a
    CUDA graph (device time from events around the graph launch), next to the
    same frames issued as plain launches."""
    import vrg
    rng = np.random.default_rng(C2_SEED)
    grids = rng.integers(1, 9, size=(C2_SCENES, 2))
    res = [C2_RES[i] for i in rng.integers(0, len(C2_RES), size=C2_SCENES)]
    scenes, keep = [], []
    t0 = time.perf_counter()
    for i in range(C2_SCENES):
        nx, nz = int(grids[i, 0]), int(grids[i, 1])
        blocks = vrg.terrain_blocks(C2_SEED + 1 + i, nx, nz, EMISSIVE)
        sc, objs = vrg.build_world(ctx, blocks)
        scenes.append(sc)
        keep.append(objs)
    t_upload = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.flush()  # every chunk of every scene: one batched extraction + BLAS build
    t_blas = time.perf_counter() - t0
    t0 = time.perf_counter()
    vrg.commit_scenes(scenes)  # all top-level trees in one SAH build, all lamp trees in another
    t_tl = time.perf_counter() - t0
    br = vrg.BatchRenderer(ctx, res, 2)
    if tuning is not None:  # the launch configuration tuned on the single-view workload
        br.set_tuning(tuning)
    seeds = vrg.Pcg32(C2_SEED)

    def cams_of(f):
        return [vrg.orbit_camera(int(grids[i, 0]), int(grids[i, 1]), f % ORBIT, ORBIT, w, h)
                for i, (w, h) in enumerate(res)]

    def params_of(flags):
        return vrg.RenderParams(1, 1, 3, 2, vrg.MODE_CONFIG, 0, 0, 0, 30.0, 20, 1, 0, flags | vrg.RENDER_NO_PACK, 4)

    def step(f, flags, sd=None):
        br.render(scenes, cams_of(f), params_of(flags), sd or [(seeds.next(), seeds.next()) for _ in res])
        st = br.last_stats
        if st.error_flags:
            raise RuntimeError(f"device error flags {st.error_flags:#x}")
        return st.ms_total, st.rays_closest + st.rays_any

    out = {"workload": "batched-64-scenes", "scenes": C2_SCENES, "pixels": br.pixels,
           "tuning": None if tuning is None else tuning.as_dict(),
           "chunks": int((grids[:, 0] * grids[:, 1]).sum()), "bounces": 2,
           "resolutions": {f"{w}x{h}": sum(1 for r in res if r == (w, h)) for w, h in C2_RES},
           "upload_s": round(t_upload, 3), "blas_build_ms": round(1000 * t_blas, 2),
           "tl_commit_ms": round(1000 * t_tl, 2)}
    for name, flags in (("graph", vrg.RENDER_GRAPH), ("launches", 0)):
        for f in range(warmup):
            step(f, flags)
        ms, rays = 0.0, 0
        t0 = time.perf_counter()
        for s_ in range(steps):
            m, r_ = step(warmup + s_, flags)
            ms += m
            rays += r_
        wall = time.perf_counter() - t0
        out[name] = {"mrays_s": round(rays / (ms / 1000.0) / 1e6, 3), "ms_per_step": round(ms / steps, 4),
                     "wall_ms_per_step": round(1000 * wall / steps, 3), "rays_per_step": rays // steps}
    # frames in flight: the steps enqueued back to back without stats (two
    # frames' bounces overlap), CUDA events on the library stream; the ray
    # counts come from a replay of the same frames one at a time
    import torch
    lib_stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", torch.cuda.current_device()))
    f0 = warmup + steps
    sds = [[(seeds.next(), seeds.next()) for _ in res] for _ in range(steps)]
    blob = br.save_state()
    n = len(res)
    p = params_of(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(lib_stream)
    for s_ in range(steps):
        views = (vrg.View * n)()
        for v, cam in enumerate(cams_of(f0 + s_)):
            views[v] = vrg.View(scenes[v].h, cam, sds[s_][v][0], sds[s_][v][1])
        vrg.check(ctx.lib.vrg_render_batched(br.h, views, n, C.byref(p), None, None), "vrg_render_batched")
    e1.record(lib_stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    br.load_state(blob)
    rays = sum(step(f0 + s_, 0, sds[s_])[1] for s_ in range(steps))
    out["in_flight"] = {"mrays_s": round(rays / (ms / 1000.0) / 1e6, 3), "ms_per_step": round(ms / steps, 4),
                        "rays_per_step": rays // steps}
    br.close()
    for sc in scenes:
        sc.close()
    return out


C4_N = 32
C4_EMISSIVE = 0.002
C4_W, C4_H = 3840, 2160


def view_cameras(nx, nz, frame, w, h, n_views=4):
    """Four views from one orbit eye, turned by 90 degrees about the up axis
    (the horizontal faces of a cube map)."""
    import vrg
    base = vrg.orbit_camera(nx, nz, frame % ORBIT, ORBIT, w, h)
    f = np.array(base.front[:], np.float64)
    r = np.array(base.right[:], np.float64)
    cams = []
    for k in range(n_views):
        a = k * np.pi / 2
        fk = np.cos(a) * f + np.sin(a) * r
        rk = np.cos(a) * r - np.sin(a) * f
        c = vrg.Camera()
        c.eye[:] = base.eye[:]
        c.front[:] = [float(x) for x in fk.astype(np.float32)]
        c.right[:] = [float(x) for x in rk.astype(np.float32)]
        c.up[:] = base.up[:]
        c.width, c.height = w, h
        cams.append(c)
    return cams


def update_commit_ms(scene, nx, nz, reps=5):
    """Commit time after moving one chunk (a transform update: the chunk BLASes
    are kept, the top levels and world-space layouts are rebuilt); the chunk
    goes back to its place at the end."""
    key = (nx // 2) * nz + nz // 2
    home = (32 * (nx // 2), 0, 32 * (nz // 2))
    ms = []
    for i in range(reps):
        scene.update_object(key, (home[0], 40 + 8 * i, home[2]))
        t0 = time.perf_counter()
        scene.commit()
        ms.append(1000 * (time.perf_counter() - t0))
    scene.update_object(key, home)
    scene.commit()
    return round(float(np.median(ms)), 3)


def large_block(ctx, steps, warmup, gt_spp, extent=(C4_W, C4_H), cache_warmup=64):
    """Large workload: 32x32 chunks (1024x32x1024 blocks, 0.2% emissive), four
    views of one orbit eye rendered as one batch, 1 spp ReSTIR over paths
    that end into the radiance cache (trained online in the same frames),
    judged against an FP64 plain 8-bounce ground truth of `gt_spp` frames of
    the same views; the plain 3-bounce tracer is measured beside it at >=
    equal time.  Each method is timed one frame at a time (with stats) and
    with its frames in flight (back to back, no stats)."""
    import vrg
    import quality
    import torch
    mats, n = vrg.terrain_materials(SEED)
    ctx.set_materials(mats, n)
    t0 = time.perf_counter()
    world = vrg.terrain_blocks(SEED, C4_N, C4_N, C4_EMISSIVE)
    scene, objs = vrg.build_world(ctx, world)
    ctx.flush()
    t_blas = time.perf_counter() - t0
    t0 = time.perf_counter()
    lt, gtl = scene.get_tlas()
    t_commit = time.perf_counter() - t0
    prims = sum(o.info()["surface_blocks"] for o in objs)
    W4, H4 = extent
    br = vrg.BatchRenderer(ctx, [(W4, H4)] * 4, 8)
    cams = view_cameras(C4_N, C4_N, 0, W4, H4)
    scenes = [scene] * 4
    seeds = vrg.Pcg32(SEED + 4)

    def params(nb, flags, view, accumulate=0):
        return vrg.RenderParams(1, view, 3, nb, vrg.MODE_CONFIG, 0, 0, 0, 30.0, 20, 1, accumulate,
                                flags | vrg.RENDER_NO_PACK, 4)

    def frame(p, want_rad=False):
        _, rads = br.render(scenes, cams, p, [(seeds.next(), seeds.next()) for _ in range(4)],
                            want_radiance=want_rad)
        st = br.last_stats
        if st.error_flags:
            raise RuntimeError(f"device error flags {st.error_flags:#x}")
        return st.ms_total, st.rays_closest + st.rays_any, rads

    # ground truth: plain 8-bounce tracer accumulated in FP64
    br.reset_accumulation()
    t0 = time.perf_counter()
    for f in range(gt_spp):
        frame(params(8, vrg.RENDER_PLAIN_ONLY, 0, accumulate=1))
    gt, n_gt = br.read_accumulation()
    gt_s = time.perf_counter() - t0
    cache = vrg.RadianceCache(ctx, gtl[0]["min"], gtl[0]["max"], seed=7)
    br.set_cache(cache)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", torch.cuda.current_device()))
    clk = ClockSampler(torch.cuda.current_device())  # clocks while the methods are timed
    clk.start()
    out = {}
    methods = (("plain", 3, vrg.RENDER_PLAIN_ONLY, 0), ("restir_cache", 2, vrg.RENDER_CACHE, 1))
    for name, nb, flags, view in methods:
        warm = cache_warmup if name == "restir_cache" else warmup
        for f in range(warm):
            frame(params(nb, flags, view))
        ms, rays, errs = 0.0, 0, []
        for s_ in range(steps):
            m, r_, rads = frame(params(nb, flags, view), want_rad=(s_ < 4))
            ms += m
            rays += r_
            if rads[0] is not None:
                errs.append(np.mean([quality.relmse(rads[v], gt[v]) for v in range(4)]))
        out[name] = {"ms_per_frame": round(ms / steps, 3), "mrays_s": round(rays / (ms / 1000.0) / 1e6, 3),
                     "rays_per_frame": rays // steps, "relmse_1spp": round(float(np.mean(errs)), 5)}
        # the same frames back to back (no stats: frames in flight), CUDA
        # events on the library stream; rays per frame from the frames above
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for s_ in range(steps):
            views = (vrg.View * 4)()
            for v in range(4):
                views[v] = vrg.View(scenes[v].h, cams[v], seeds.next(), seeds.next())
            p = params(nb, flags, view)
            vrg.check(ctx.lib.vrg_render_batched(br.h, views, 4, C.byref(p), None, None), "vrg_render_batched")
        e1.record(stream)
        e1.synchronize()
        ms_f = e0.elapsed_time(e1) / steps
        out[name]["ms_per_frame_in_flight"] = round(ms_f, 3)
        out[name]["mrays_s_in_flight"] = round((rays / steps) / (ms_f / 1000.0) / 1e6, 3)
    # plain accumulated over at least the cache frame's time, with frames
    # timed one at a time and with frames in flight
    rc = out["restir_cache"]
    k = max(1, int(np.ceil(rc["ms_per_frame"] / out["plain"]["ms_per_frame"] - 1e-9)))
    k_f = max(1, int(np.ceil(rc["ms_per_frame_in_flight"] / out["plain"]["ms_per_frame_in_flight"] - 1e-9)))
    br.set_cache(None)
    rel_plain = {}
    for kk in sorted({k, k_f}):
        br.reset_accumulation()
        for f in range(kk):
            frame(params(3, vrg.RENDER_PLAIN_ONLY, 0, accumulate=1))
        acc, _ = br.read_accumulation()
        rel_plain[kk] = float(np.mean([quality.relmse(acc[v], gt[v]) for v in range(4)]))
    rel_plain_k = rel_plain[k]
    res = {
        "workload": f"large-32x32chunks-4x{W4}x{H4}", "chunks": [C4_N, C4_N], "surface_blocks": prims,
        "emissive_fraction": C4_EMISSIVE, "views": 4, "resolution": [W4, H4],
        "method": "2 bounces ending into the radiance cache + ReSTIR (3 spatial, 30 px, M-cap 20), "
                  "1/16 paths trace 4 more bounces and train the cache",
        "scene_build": {"blas_ms": round(1000 * t_blas, 1), "commit_ms": round(1000 * t_commit, 1),
                        "update_commit_ms": update_commit_ms(scene, C4_N, C4_N)},
        "methods": out,
        "ground_truth": {"spp": n_gt, "bounces": 8, "accumulation": "fp64 on the GPU", "seconds": round(gt_s, 1)},
        "equal_time": {"plain_frames": k, "plain_time_ratio": round(k * out["plain"]["ms_per_frame"] /
                                                                    rc["ms_per_frame"], 3),
                       "relmse_plain": round(rel_plain_k, 5), "relmse_restir_cache_1spp": rc["relmse_1spp"],
                       "gain": round(rel_plain_k / max(rc["relmse_1spp"], 1e-12), 3),
                       "gain_lower_bound": round(out["plain"]["relmse_1spp"] / max(
                           1.0, rc["ms_per_frame"] / out["plain"]["ms_per_frame"]) /
                           max(rc["relmse_1spp"], 1e-12), 3),
                       "in_flight": {"plain_frames": k_f, "plain_time_ratio": round(
                           k_f * out["plain"]["ms_per_frame_in_flight"] / rc["ms_per_frame_in_flight"], 3),
                           "relmse_plain": round(rel_plain[k_f], 5),
                           "gain": round(rel_plain[k_f] / max(rc["relmse_1spp"], 1e-12), 3)}},
        "clocks": clk.stop(),
    }
    cache.close()
    br.close()
    scene.close()
    for o in objs:
        o.release()
    return res


def run_large(args, d):
    """The large workload as its own line (--workload large), ground truth at
    --gt-spp frames (4096 by default)."""
    import vrg
    if d.rank != 0:
        d.close()
        return
    ctx = vrg.Context(0)
    ext = (C4_W, C4_H) if not args.resolution else (W, H)
    blk = large_block(ctx, args.steps, args.warmup, args.gt_spp, ext)
    hbm_peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            hbm_peak = json.load(fh).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    rc = blk["methods"]["restir_cache"]
    line = {
        "metric": METRIC, "value": rc["mrays_s"], "unit": "Mrays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": rc["ms_per_frame"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded value-noise voxel terrain, no dataset)",
        "config": {"workload": blk["workload"], "chunks": blk["chunks"], "surface_blocks": blk["surface_blocks"],
                   "emissive_fraction": C4_EMISSIVE, "views": 4, "resolution": blk["resolution"],
                   "method": blk["method"], "parallelism": "single GPU, one batched launch sequence"},
        "scene_build": blk["scene_build"], "methods": blk["methods"], "ground_truth": blk["ground_truth"],
        "equal_time": blk["equal_time"], "hbm_peak_gbs": hbm_peak, "clocks": blk["clocks"],
    }
    print(json.dumps(line), flush=True)
    d.close()


def headline_config(gpus):
    """The workload of the headline line, the same dict in both arms."""
    return {"workload": "restir-1080p-4x4chunks", "resolution": [W, H], "chunks": [NX, NZ],
            "bounces": NB, "temporal_history": 1, "spatial_neighbours": 3, "radius_px": 30,
            "m_cap": 20, "emissive_fraction": EMISSIVE, "orbit_frames": ORBIT,
            "l2": "per-frame state (~1.2 GB of rays, records, reservoirs) exceeds L2; BVH L2-resident",
            "parallelism": f"replicas{gpus}"}


def run_reference(args, d):
    """The reference's CPU path (the oracle restatement, OpenMP over pixels on
    every host core).  Its inputs come from the generator compiled into the
    oracle library, so this process never loads the CUDA library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if d.rank != 0:
        d.close()
        return
    mats, n = oracle.terrain_materials(SEED)
    world = oracle.terrain_blocks(SEED, NX, NZ, EMISSIVE)
    # Full frames (the CPU path's stream passes run over the whole image in any
    # case, so a band of rows would understate its throughput), bounded to the
    # first REF_MAX_FRAMES of the K timed frames: about 12 s on 16 cores.
    rows = min(args.ref_rows, H)
    frames = min(args.steps, REF_MAX_FRAMES)
    threads = cpu_threads()
    smp = OracleSampler(world, mats, n, rows)
    for w in range(min(args.warmup, 2)):
        smp.frame(w)
    times, rays_all = [], 0
    for s in range(frames):
        dt, rays = smp.frame(args.warmup + s)
        times.append(dt)
        rays_all += rays
    smp.close()
    total = sum(times)
    value = rays_all / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s",
        "n_gpus": args.gpus, "steps": frames, "requested_steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * total / frames, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded value-noise voxel terrain, no dataset)",
        "config": headline_config(args.gpus),
        "timing": "wall clock around each frame of the oracle on the host cores",
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{rows} of {H} rows per frame, orbit frames {args.warmup}-"
                                   f"{args.warmup + frames - 1} (the first {frames} of the {args.steps} timed)"},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    d.close()


def run_ours(args, d):
    import vrg
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    ctx = vrg.Context(d.local if args.gpus > 1 else 0)
    mats, n = vrg.terrain_materials(SEED)
    ctx.set_materials(mats, n)
    world = vrg.terrain_blocks(SEED, NX, NZ, EMISSIVE)
    t0 = time.perf_counter()
    scene, objs = vrg.build_world(ctx, world)
    scene.commit()
    build_s = time.perf_counter() - t0
    r = vrg.Renderer(ctx, W, H, NB)
    lib = ctx.lib
    stats = vrg.FrameStats()
    out_dev = vrg.FrameOutput(None, None, 0, 0)

    def frame_params(f):
        return vrg.RenderParams(1, 1, 3, NB, vrg.MODE_CONFIG, f, 1000 + f, 2000 + f, 30.0, 20, 1, 0, 0)

    def render(f, out, st):
        cam = vrg.orbit_camera(NX, NZ, f % ORBIT, ORBIT, W, H)
        p = frame_params(f)
        vrg.check(lib.vrg_render(r.h, scene.h, C.byref(cam), C.byref(p), C.byref(out),
                                 C.byref(st) if st is not None else None), "vrg_render")

    import torch
    dev_ord = d.local if args.gpus > 1 else 0
    torch.cuda.set_device(dev_ord)
    lib_stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", dev_ord))

    def back_to_back_ms(frames, f0):
        """ms per frame of `frames` frames enqueued back to back (CUDA events on the library stream)."""
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        for f in range(frames):
            render(f0 + f, out_dev, None)
        e1.record(lib_stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / frames

    for f in range(args.warmup):
        render(f, out_dev, stats)
    tuning, best_tuning = None, None
    if not args.no_autotune:
        # launch configuration chosen by the autotuner on this workload's
        # frames (scheduling only; the frames it renders are not counted and
        # the renderer's frame counter and history are restored); both times
        # are per frame of frames run back to back (the default over the
        # orbit's first eight views, the tuner's candidates at its first
        # view; 24 frames per run, so that the first frames of a run, which
        # have fewer frames in flight beside them, weigh little in the choice)
        blob0 = r.save_state()
        default_ms = [back_to_back_ms(8, 0) for _ in range(3)]
        r.load_state(blob0)
        cam0 = vrg.orbit_camera(NX, NZ, 0, ORBIT, W, H)
        t0 = time.perf_counter()
        best, best_ms = r.autotune(scene, cam0, frame_params(0), frames=24)
        best_tuning = best
        tuning = {"config": best.as_dict(), "tuned_ms": round(best_ms, 4),
                  "default_ms": round(float(np.median(default_ms)), 4),
                  "tuner_seconds": round(time.perf_counter() - t0, 2)}
    # Timed region: the K frames enqueued back to back (no per-frame stats, so
    # frames are in flight together as in an interactive loop), bracketed by
    # CUDA events on the library's own stream with a synchronize on both sides.
    blob = r.save_state()  # the breakdown pass below replays the same frames from here
    clk = ClockSampler(d.local)
    clk.start()
    time.sleep(0.25)  # the sampler's first reading lands before the region
    # the W warm-up frames again right before the region, so that the GPU does
    # not enter it from the idle wait above; then a synchronize and a barrier
    w0 = time.perf_counter()
    for s in range(args.warmup):
        render(s, out_dev, None)
    torch.cuda.synchronize()
    d.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(lib_stream)
    for s in range(args.steps):
        render(args.warmup + s, out_dev, None)
    ev1.record(lib_stream)
    ev1.synchronize()
    w1 = time.perf_counter()
    time.sleep(0.15)
    clocks = clk.stop((w0, w1 + 0.1))
    total_s = ev0.elapsed_time(ev1) / 1000.0
    # Replay of the same K frames, one at a time with stats: their ray counts
    # (identical frames: the renderer state is restored) and the per-stage
    # CUDA-event breakdown
    r.load_state(blob)
    for s in range(args.warmup):
        render(s, out_dev, None)
    ms, rays, ms_b, ms_res, ms_sp = [], 0, [0.0] * NB, 0.0, 0.0
    ms_tr, ms_sh, ms_ah = [0.0] * NB, [0.0] * NB, [0.0] * NB
    closest, nodes, leaves = 0, 0, 0
    any_rays, l_nodes, l_leaves, l_hits = 0, 0, 0, 0
    for s in range(args.steps):
        render(args.warmup + s, out_dev, stats)
        if stats.error_flags:
            raise RuntimeError(f"device error flags {stats.error_flags:#x}")
        ms.append(stats.ms_total)
        rays += stats.rays_closest + stats.rays_any
        closest += stats.rays_closest
        nodes += stats.nodes_visited
        leaves += stats.leaves_visited
        any_rays += stats.rays_any
        l_nodes += stats.light_nodes_visited
        l_leaves += stats.light_leaves_visited
        l_hits += stats.light_hits
        for b in range(NB):
            ms_b[b] += stats.ms_bounce[b]
            ms_tr[b] += stats.ms_trace[b]
            ms_sh[b] += stats.ms_shade[b]
            ms_ah[b] += stats.ms_anyhit[b]
        ms_res += stats.ms_resolve
        ms_sp += stats.ms_spatial
    d.barrier()
    total_s_max = d.max(total_s)
    rays_all = d.sum(rays)
    value = rays_all / total_s_max / 1e6
    # End to end through the public API: the same K frames again (state
    # restored), each frame's image read back into page-locked host memory
    # (so the device->host copy runs at link speed).  E2E_SLOTS buffers are
    # taken in turn, as the reference's swapchain slots are; every frame's copy
    # is queued behind it (VRG_OUTPUT_HOST_ASYNC), and the host waits on the
    # fence of the oldest frame in flight and reads its image while the newer
    # ones render.  Wall clock, same ray counts.
    host_imgs = [torch.empty(W * H * 4, dtype=torch.uint8, pin_memory=True) for _ in range(E2E_SLOTS)]
    outs = [vrg.FrameOutput(t.data_ptr(), None, vrg.OUTPUT_HOST_ASYNC, 0) for t in host_imgs]
    r.load_state(blob)
    for s in range(0 if args.no_e2e else args.warmup):
        render(s, out_dev, None)
    f0 = r.frame_index()
    checksum = 0
    lag = E2E_SLOTS - 1  # frames in flight behind the one just enqueued
    torch.cuda.synchronize()
    d.barrier()
    t0 = time.perf_counter()
    for s in range(0 if args.no_e2e else args.steps):
        render(args.warmup + s, outs[s % E2E_SLOTS], None)
        if s >= lag:  # the oldest frame in flight: fence, then read its image
            r.wait_frame(f0 + s - lag)
            checksum ^= int(host_imgs[(s - lag) % E2E_SLOTS][(s * 4099) % (W * H * 4)])
    for s in range(max(0, args.steps - lag), 0 if args.no_e2e else args.steps):
        r.wait_frame(f0 + s)
        checksum ^= int(host_imgs[s % E2E_SLOTS][0])
    e2e_s = d.max(time.perf_counter() - t0)
    e2e_value = rays_all / e2e_s / 1e6 if not args.no_e2e else None
    if d.rank != 0:
        d.close()
        return
    # roofline of the dominant kernel, k_trace (closest hit): its compulsory HBM
    # bytes are 16 B of hit record per ray plus 36 B of queue index and ray
    # (origin, direction) for every ray after the primary one; the BVH nodes it
    # walks stay in L1/L2 and are reported separately as traversal bytes
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    trace_s = sum(ms_tr) / 1000.0
    P = W * H
    trace_bytes = 16 * closest + 36 * (closest - P * args.steps)
    achieved = trace_bytes / trace_s / 1e9 if trace_s > 0 else 0.0
    trav_bytes = 128 * nodes + 16 * leaves  # 4-wide nodes (128 B) and surface-block records (16 B)
    stream_bytes = W * H * 252  # ReSTIR compulsory stream bytes per frame (reservoirs + radiance)
    stream_s = (ms_res + ms_sp) / 1000.0
    stream_gbs = stream_bytes * args.steps / stream_s / 1e9 if stream_s > 0 else 0.0
    # L2 read bandwidth of this device, measured now by the library's own
    # sweep kernel: the peak of the BVH walks, whose node and record fetches
    # are L1/L2 traffic (a 32 MiB buffer, 64 sweeps, best of 3)
    l2_peak = max(ctx.l2_read_gbs(32, 64) for _ in range(3))
    trace_l2_gbs = trav_bytes / trace_s / 1e9 if trace_s > 0 else 0.0
    # light-hit collection: 4-wide lamp nodes (112 B: six plane rows and the
    # refs) and lamp-block records (16 B), over the light-pdf walk's time
    any_s = sum(ms_ah) / 1000.0
    walk_bytes = 112 * l_nodes + 16 * l_leaves
    walk_l2_gbs = walk_bytes / any_s / 1e9 if any_s > 0 else 0.0
    # shading, HBM: ray + hit in (48 B) and the bounce record out (32 B) per
    # ray, the next ray and its queue slot (36 B) per continuing ray, and the
    # two vertices of the ReSTIR sample geometry (64 B) per pixel
    shade_s = sum(ms_sh) / 1000.0
    shade_bytes = 80 * closest + 36 * (closest - P * args.steps) + 64 * P * args.steps
    shade_gbs = shade_bytes / shade_s / 1e9 if shade_s > 0 else 0.0
    parts = [("k_trace", trace_s, trace_l2_gbs / l2_peak if l2_peak else 0.0, "l2"),
             ("k_shade", shade_s, shade_gbs / hbm_peak, "hbm"),
             ("light_pdf_walk", any_s, walk_l2_gbs / l2_peak if l2_peak else 0.0, "l2"),
             ("k_resolve+k_spatial", stream_s, stream_gbs / hbm_peak, "hbm")]
    t_all = sum(t for _, t, _, _ in parts)
    weighted = sum(t * f for _, t, f, _ in parts) / t_all if t_all > 0 else 0.0
    traffic, traffic_src = trace_traffic_per_launch(W * H, NB)
    quality_block = None
    if not args.no_quality:
        import quality
        # the learned-cache workload: the same generator on 8x8 chunks at 1080p
        world3 = vrg.terrain_blocks(SEED, C3_N, C3_N, EMISSIVE)
        scene3, objs3 = vrg.build_world(ctx, world3)
        qr = vrg.Renderer(ctx, W, H, 8)
        cam = vrg.orbit_camera(C3_N, C3_N, 0, ORBIT, W, H)
        lt, gtl = scene3.get_tlas()
        # every method of the study runs under one launch configuration, the
        # autotuner's on this scene's ReSTIR frames (the tuner takes no cache
        # frames, whose training changes the cache)
        q_tuning = None
        if not args.no_autotune:
            t0 = time.perf_counter()
            qbest, qms = qr.autotune(scene3, cam, quality.method_params("restir", 0), frames=24)
            q_tuning = {"config": qbest.as_dict(), "tuned_ms": round(qms, 4),
                        "tuner_seconds": round(time.perf_counter() - t0, 2)}
        t0 = time.perf_counter()
        gt = quality.ground_truth(qr, scene3, cam, spp=args.gt_spp, bounces=8)
        gt_s = time.perf_counter() - t0
        study = quality.equal_time_study(ctx, scene3, qr, cam, gt, gtl[0]["min"], gtl[0]["max"], frames=16,
                                         cache_warmup=128)
        quality_block = {"workload": f"learned-cache-1080p-{C3_N}x{C3_N}chunks",
                         "ground_truth": {"spp": args.gt_spp, "bounces": 8, "accumulation": "fp64 on the GPU",
                                          "seconds": round(gt_s, 2), "camera": "orbit frame 0"},
                         "cache": {"levels": 16, "table_entries_per_level": 2 ** 19, "features": 2, "mlp": "5x64 relu",
                                   "train_samples_per_frame": 65536, "train_bounces": 4, "lr": 1e-2},
                         "relmse_eps": quality.EPS, "tuning": q_tuning, **study}
        qr.close()
        scene3.close()
        for o in objs3:
            o.release()
    batched = None
    if not args.no_batched:
        r.close()  # the batch needs the memory of the 1080p renderer
        batched = batched_block(ctx, steps=16, warmup=3, tuning=best_tuning)
    large = None
    if not args.no_large:
        # the large workload, compact: a 256-spp ground truth (the full
        # 4096-spp run is --workload large) and 6 frames per method
        large = large_block(ctx, steps=16, warmup=3, gt_spp=args.large_gt_spp)
        ctx.set_materials(mats, n)
    upd_ms = update_commit_ms(scene, NX, NZ)
    cpu_frames = args.cpu_frames
    cpu_mr, cpu_dt, cpu_rays, cpu_build_s = (oracle_sample(world, mats, n, args.ref_rows, cpu_frames, 0)
                                             if not args.no_cpu else (None, 0, 0, None))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * total_s_max / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded value-noise voxel terrain, no dataset)",
        "config": headline_config(args.gpus),
        "timing": "K frames enqueued back to back on the library stream (frames in flight), bracketed by a "
                  "synchronize and CUDA events on that stream (W warm-up frames just before); ray counts and stage "
                  "times from a replay of the same frames one at a time",
        "ms_breakdown": {"bounce": [round(x / args.steps, 4) for x in ms_b],
                         "k_trace": [round(x / args.steps, 4) for x in ms_tr],
                         "k_shade": [round(x / args.steps, 4) for x in ms_sh],
                         "k_anyhit": [round(x / args.steps, 4) for x in ms_ah],
                         "resolve_temporal": round(ms_res / args.steps, 4),
                         "spatial_finalize_pack": round(ms_sp / args.steps, 4)},
        "ms_per_frame_alone": round(sum(ms) / max(args.steps, 1), 4),
        "rays_per_frame": rays // max(args.steps, 1),
        "scene_build_ms": round(build_s * 1000, 2),
        # the oracle's build of the same 16 chunks on one host core: meshing,
        # light extraction, both SAH BLAS builds per chunk and the commit
        "scene_build_cpu_ms": None if cpu_build_s is None else round(cpu_build_s * 1000, 2),
        "update_commit_ms": upd_ms,
        "roofline": {"bound": "hbm", "kernel": "k_trace", "achieved": round(achieved, 2), "peak": hbm_peak,
                     "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                     "traffic": traffic, "traffic_source": traffic_src,
                     "algorithmic_bytes_per_launch": round(trace_bytes / max(args.steps, 1) / NB),
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else peak_src,
                     "algorithmic_bytes": "16 B hit per ray + 36 B ray/queue per secondary ray",
                     "note": "k_trace is issue/latency bound: its BVH walk is served from L1/L2, see l2",
                     "l2": {"kernel": "k_trace", "achieved": round(trace_l2_gbs, 1), "peak": round(l2_peak, 1),
                            "unit": "GB/s", "frac": round(trace_l2_gbs / l2_peak, 4) if l2_peak else None,
                            "bytes_per_launch": round(trav_bytes / max(args.steps, 1) / NB),
                            "bytes": "128 B per 4-wide node + 16 B per surface-block record visited",
                            "peak_source": "measured in this run (vrg_measure_l2_bandwidth: 32 MiB, 64 sweeps, "
                                           "best of 3)"},
                     "time_weighted": {"frac": round(weighted, 4),
                                       "kernels": {k: {"ms_per_frame": round(1000 * t / max(args.steps, 1), 4),
                                                       "frac": round(f, 4), "peak": pk} for k, t, f, pk in parts}}},
        "traversal": {"kernel": "k_trace", "nodes_per_ray": round(nodes / max(closest, 1), 2),
                      "leaves_per_ray": round(leaves / max(closest, 1), 2),
                      "l1_l2_bytes_per_s_gbs": round(trav_bytes / trace_s / 1e9, 1) if trace_s > 0 else None,
                      "grays_per_s": round(closest / trace_s / 1e9, 3) if trace_s > 0 else None},
        "light_walk": {"kernel": "k_anyhit", "nodes_per_ray": round(l_nodes / max(any_rays, 1), 2),
                       "leaves_per_ray": round(l_leaves / max(any_rays, 1), 2),
                       "hits_per_ray": round(l_hits / max(any_rays, 1), 3)},
        "stream_roofline": {"kernels": "k_resolve+k_spatial", "achieved": round(stream_gbs, 2), "peak": hbm_peak,
                            "unit": "GB/s", "frac": round(stream_gbs / hbm_peak, 4), "bytes_per_px": 252},
        "e2e": {"value": None if e2e_value is None else round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": C.sizeof(vrg.Camera) + C.sizeof(vrg.RenderParams),
                "d2h_bytes_per_step": W * H * 4},
        # per frame: k_trace and k_shade per bounce, k_anyhit + k_hit_eval +
        # k_hit_sum per bounce but the last, k_resolve, k_spatial
        "gpu_launches": (2 * NB + 3 * (NB - 1) + 2) * args.steps,
        "quality": quality_block,
        "autotune": tuning,
        "batched": batched,
        "large": large,
        "clocks": clocks,
        "cpu_baseline": None if cpu_mr is None else {
            "value": round(cpu_mr, 4), "unit": "Mrays/s", "cores": cpu_threads(), "kind": "port",
            "sample": f"{min(args.ref_rows, H)} of {H} rows of orbit frames 0-{cpu_frames - 1} "
                      f"({cpu_dt:.1f} s, {cpu_rays} rays)"},
    }
    print(json.dumps(line), flush=True)
    d.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=512)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-rows", type=int, default=1080, help="image rows the CPU baseline traces per frame")
    ap.add_argument("--cpu-frames", type=int, default=48, help="frames of the CPU baseline sample (about 10 s on 16 cores)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end pass (profiling runs)")
    ap.add_argument("--resolution", default=None, help="WxH override (profiling cases only)")
    ap.add_argument("--no-quality", action="store_true", help="skip the FP64 ground truth / relMSE study")
    ap.add_argument("--gt-spp", type=int, default=None,
                    help="ground-truth samples per pixel (4096)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-scene batched workload")
    ap.add_argument("--no-autotune", action="store_true", help="time the default launch configuration")
    ap.add_argument("--no-large", action="store_true", help="skip the compact large-workload block")
    ap.add_argument("--large-gt-spp", type=int, default=256,
                    help="ground-truth frames of the compact large-workload block")
    ap.add_argument("--workload", default="restir", choices=["restir", "large"],
                    help="restir: the 1080p ReSTIR headline line; large: the 32x32-chunk four-view 4K workload")
    args = ap.parse_args()
    global W, H
    if args.resolution:
        W, H = (int(x) for x in args.resolution.lower().split("x"))
    if args.warmup < 3:
        args.warmup = 3
    if args.gt_spp is None:
        args.gt_spp = 4096
    import vrg
    if not os.path.exists(vrg.LIB_PATH):
        sys.path.insert(0, ROOT)
        import __graft_entry__
        __graft_entry__.build()
    d = Dist()
    if args.impl == "reference":
        run_reference(args, d)
    elif args.workload == "large":
        run_large(args, d)
    else:
        run_ours(args, d)


if __name__ == "__main__":
    main()
