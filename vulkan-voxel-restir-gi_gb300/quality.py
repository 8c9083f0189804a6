"""Image-quality measurement of the renderer: an FP64-accumulated ground truth
of the plain path tracer and the relative MSE of other estimators against it,
with the cache-terminated tracers compared to the plain one at equal frame
time (none of this has a reference counterpart: the reference renders 1 spp
per frame with no error metric).

relMSE(x, gt) = mean over pixels and channels of (x - gt)^2 / (gt^2 + 0.01).

Equal time, two ways:
  * measured: the method's 1-spp frame against the plain tracer accumulated
    over ceil(t_m / t_plain) frames (the plain tracer gets at least the
    method's device time, up to one frame more);
  * lower bound: the mean of N independent plain frames has relMSE
    b + v/N >= (b + v)/N = relMSE_1spp / N (b: its bias against the ground
    truth, v: its one-frame variance), so relMSE_1spp / N_eq with
    N_eq = max(1, t_m / t_plain) bounds the plain tracer's error at exactly
    the method's time from below, and the gain computed with it bounds the
    equal-time gain from below.
"""
import ctypes as C
import math

import numpy as np

import vrg

EPS = 0.01


def relmse(x, gt):
    """Non-finite estimates (the estimator's 0*inf cases) count as 0."""
    x = np.nan_to_num(np.asarray(x, np.float64), nan=0.0, posinf=0.0, neginf=0.0)
    gt = np.asarray(gt, np.float64)
    return float(np.mean((x - gt) ** 2 / (gt * gt + EPS)))


def nonfinite_fraction(x):
    return float(np.mean(~np.isfinite(np.asarray(x))))


def _params(nb, flags, seed, accumulate=1, train_bounces=4):
    return vrg.RenderParams(1, 0, 0, nb, vrg.MODE_CONFIG, seed, seed + 1, seed + 2, 30.0, 20, 1, accumulate,
                            flags | vrg.RENDER_NO_PACK, train_bounces)


def ground_truth(renderer, scene, cam, spp=4096, bounces=8):
    """Plain path tracer, `bounces` bounces, `spp` frames accumulated in FP64 on the GPU."""
    renderer.reset_accumulation()
    for f in range(spp):
        renderer.render_params(scene, cam, _params(bounces, vrg.RENDER_PLAIN_ONLY, f), want_image=False)
    acc, n = renderer.read_accumulation()
    assert n == spp
    return acc


def frame_ms(renderer):
    return float(renderer.last_stats.ms_total)


def run_method(renderer, scene, cam, method, frames, seed0=0, warmup=0, cache=None):
    """Renders `frames` 1-spp frames of `method` at a fixed camera; returns
    (mean image, list of single-frame radiance images, mean device ms/frame).
    method: 'plain' (3 bounces), 'restir' (3 bounces + ReSTIR view), 'cache'
    (2 bounces ending into the radiance cache, 4 more for 1/16 training paths),
    'restir_cache' (the cache-terminated paths resampled by ReSTIR)."""
    if method in ("cache", "restir_cache"):
        renderer.set_cache(cache)
    singles, ms = [], []
    stages = None
    for f in range(warmup + frames):
        p = method_params(method, seed0 + f)
        _, rad = renderer.render_params(scene, cam, p, want_image=False, want_radiance=True)
        if f >= warmup:
            singles.append(rad.astype(np.float32))
            ms.append(frame_ms(renderer))
            st = renderer.last_stats
            stages = {"bounces": [round(st.ms_bounce[b], 4) for b in range(p.num_bounces + (
                p.cache_train_bounces if p.flags & vrg.RENDER_CACHE else 0))],
                "resolve_and_cache": round(st.ms_resolve, 4), "spatial": round(st.ms_spatial, 4)}
    clean = [np.nan_to_num(s, nan=0.0, posinf=0.0, neginf=0.0) for s in singles]
    run_method.last_stages = stages
    return np.mean(clean, axis=0), singles, float(np.mean(ms))


METHODS = ("plain", "restir", "cache", "restir_cache")


def method_params(method, seed):
    """The render parameters run_method uses for `method`."""
    if method == "plain":
        return _params(3, vrg.RENDER_PLAIN_ONLY, seed, accumulate=0)
    if method == "restir":
        p = _params(3, 0, seed, accumulate=0)
    else:
        p = _params(2, vrg.RENDER_CACHE, seed, accumulate=0)
        if method != "restir_cache":
            return p
    p.debug_view = 1
    p.spatial_iterations = 3
    return p


def in_flight_ms(renderer, scene, cam, method, frames, seed0=0, cache=None):
    """Device ms per frame of `frames` frames of `method` enqueued back to back
    (no stats, no outputs: frames in flight), CUDA events on the library's
    stream; None without torch."""
    try:
        import torch
    except ImportError:
        return None
    ctx = renderer.ctx
    renderer.set_cache(cache if method in ("cache", "restir_cache") else None)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", torch.cuda.current_device()))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for f in range(frames):
        p = method_params(method, seed0 + f)
        vrg.check(ctx.lib.vrg_render(renderer.h, scene.h, C.byref(cam), C.byref(p), None, None), "vrg_render")
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / frames


def equal_time_study(ctx, scene, renderer, cam, gt, scene_min, scene_max, frames=16, cache_warmup=64, seed=7):
    """Single-frame and equal-time relMSE of plain, ReSTIR and cache-terminated
    tracing (alone and resampled by ReSTIR) against `gt`.  The cache is
    trained online for `cache_warmup` frames at this camera before the
    measured frames (it keeps training)."""
    cache = vrg.RadianceCache(ctx, scene_min, scene_max, seed=seed)
    out = {}
    for method in METHODS:
        warm = cache_warmup if method == "cache" else 2
        mean_img, singles, ms = run_method(renderer, scene, cam, method, frames, seed0=1000, warmup=warm,
                                           cache=cache)
        out[method] = {"ms_per_frame": round(ms, 4),
                       "relmse_1spp": round(float(np.mean([relmse(s, gt) for s in singles])), 6),
                       "nonfinite": round(float(np.mean([nonfinite_fraction(s) for s in singles])), 8),
                       "relmse_mean_of_frames": round(relmse(mean_img, gt), 6), "frames": frames,
                       "stages_ms_last_frame": run_method.last_stages}
    # the same methods' frames back to back, as an interactive loop renders
    # them (frames in flight); the relMSE figures above do not depend on it
    for method in METHODS:
        t = in_flight_ms(renderer, scene, cam, method, frames, seed0=9000, cache=cache)
        out[method]["ms_per_frame_in_flight"] = None if t is None else round(t, 4)
    renderer.set_cache(None)
    # equal time: each method's 1-spp frame against the plain tracer
    # accumulated over at least the same device time
    t_plain = out["plain"]["ms_per_frame"]
    eq = {}
    plain_acc = {}
    for method in METHODS[1:]:
        t_m = out[method]["ms_per_frame"]
        k = max(1, int(math.ceil(t_m / t_plain - 1e-9))) if t_plain > 0 else 1
        if k not in plain_acc:
            acc_img, _, _ = run_method(renderer, scene, cam, "plain", k, seed0=5000)
            plain_acc[k] = relmse(acc_img, gt)
        n_eq = max(1.0, t_m / t_plain) if t_plain > 0 else 1.0
        rel_m = max(out[method]["relmse_1spp"], 1e-12)
        eq[method] = {"plain_frames": k, "plain_time_ratio": round(k * t_plain / t_m, 3),
                      "relmse_plain": round(plain_acc[k], 6), "relmse_method_1spp": out[method]["relmse_1spp"],
                      "gain": round(plain_acc[k] / rel_m, 3),
                      "gain_lower_bound": round(out["plain"]["relmse_1spp"] / n_eq / rel_m, 3)}
    out["equal_time"] = eq
    # What the trained network adds under ReSTIR: ReSTIR over cache-terminated
    # paths against ReSTIR over plain 3-bounce paths given at least the same
    # device time (the mean of ceil(t_restir_cache / t_restir) consecutive
    # ReSTIR frames; consecutive frames share reservoirs, so this is what
    # ReSTIR reaches in that time, not an independent-sample bound).
    vs = {}
    for key, t_rc, t_r in (("frames_one_at_a_time", out["restir_cache"]["ms_per_frame"], out["restir"]["ms_per_frame"]),
                           ("frames_in_flight", out["restir_cache"].get("ms_per_frame_in_flight"),
                            out["restir"].get("ms_per_frame_in_flight"))):
        if not t_rc or not t_r:
            continue
        k = max(1, int(math.ceil(t_rc / t_r - 1e-9)))
        if ("restir", k) not in plain_acc:
            acc_img, _, _ = run_method(renderer, scene, cam, "restir", k, seed0=6000, warmup=2)
            plain_acc[("restir", k)] = relmse(acc_img, gt)
        rel_m = max(out["restir_cache"]["relmse_1spp"], 1e-12)
        vs[key] = {"restir_frames": k, "restir_time_ratio": round(k * t_r / t_rc, 3),
                   "relmse_restir": round(plain_acc[("restir", k)], 6),
                   "relmse_restir_cache_1spp": out["restir_cache"]["relmse_1spp"],
                   "gain": round(plain_acc[("restir", k)] / rel_m, 3)}
    out["restir_cache_vs_restir"] = vs
    # the same comparison with every method timed in flight
    t_plain_f = out["plain"].get("ms_per_frame_in_flight")
    if t_plain_f:
        eqf = {}
        for method in METHODS[1:]:
            t_m = out[method]["ms_per_frame_in_flight"]
            k = max(1, int(math.ceil(t_m / t_plain_f - 1e-9)))
            if k not in plain_acc:
                acc_img, _, _ = run_method(renderer, scene, cam, "plain", k, seed0=5000)
                plain_acc[k] = relmse(acc_img, gt)
            n_eq = max(1.0, t_m / t_plain_f)
            rel_m = max(out[method]["relmse_1spp"], 1e-12)
            eqf[method] = {"plain_frames": k, "plain_time_ratio": round(k * t_plain_f / t_m, 3),
                           "gain": round(plain_acc[k] / rel_m, 3),
                           "gain_lower_bound": round(out["plain"]["relmse_1spp"] / n_eq / rel_m, 3)}
        out["equal_time_in_flight"] = eqf
    cache.close()
    return out
