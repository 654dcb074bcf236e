"""BVH traversal benchmark: Mrays/s closest-hit + any-hit on one GB300 (per GPU under torchrun).

Workload (the traversal microbenchmark scene, FP32):
  scene   1024 x 1024-cell fBm heightfield (2,097,152 triangles, amplitude 0.2, 6 octaves, seed 1)
          + 200,000 random triangles (centres U([-1,1]x[0,0.5]x[-1,1]), vertex offsets N(0, 0.01^2))
          = 2,297,152 triangles; binned SAH (128 bins, binary leaves of 1), cost-optimal collapse (leaves <= 3) collapsed to 8-wide nodes.
  rays    16,777,216 per step: 8,388,608 primary (4096 x 2048 pinhole at (0,1.5,-2.5) aimed at the
          origin, 30 degree vertical FOV), 4,194,304 cosine-hemisphere bounce rays from primary hits,
          4,194,304 any-hit shadow rays to uniform points on a 0.5 x 0.5 quad at y = 2
          (tmax = distance - 1e-4). Primary rays are emitted in 4x8-pixel tiles (8-row bands); bounce
          and shadow rays follow the order of the primary rays they continue.
A step = the three launches over the resident batch (closest primary, closest bounce, any shadow).
The ray batch (604 MB in, 196 MB out per step) is larger than L2, so no extra flush is done.
Launch configurations are picked per ray class by the autotuner before the timed region.

The same JSON line carries "render": path-tracing workloads on the same GPU (Cornell box samples/s,
many-light ReSTIR DI frames at 1080p, guided against plain path tracing, and 48 batched jobs in one
wavefront with a CUDA graph per iteration); see render_workloads and batch_workload.

--impl reference times the reference's CPU traversal instead (the reference's own code from
oracle/_ref where it was compiled for this machine, else the oracle's restatement of it) on all
host cores over a bounded sample of the same batch.
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

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "hiprt-path-tracer_gb300"))

METRIC = "Mrays/s closest-hit (BVH traversal, 16M-ray batch: 8M primary + 4M bounce closest-hit, 4M shadow any-hit)"
UNIT = "Mrays/s"
WIDTH, HEIGHT, VFOV = 4096, 2048, 30.0
N_BOUNCE = 4 * 1024 * 1024
N_SHADOW = 4 * 1024 * 1024
RAY_IN_BYTES = 36  # origin+tmin, direction+tmax, last_prim
CLOSEST_OUT_BYTES = 16
ANY_OUT_BYTES = 1
NODE_BYTES = 80
KERNEL_NAMES = {1: "trace_ray_kernel", 2: "trace_persistent", 3: "trace_fetch"}
TRI_BYTES = 36  # algorithmic: three float3 vertex records


def workload_config(n_tris):
    return {"workload": "bvh-traversal-microbench", "triangles": n_tris, "rays_per_step": WIDTH * HEIGHT + N_BOUNCE + N_SHADOW,
            "primary": f"{WIDTH}x{HEIGHT} pinhole, vfov {VFOV} deg, emitted in 4x8-pixel tiles (8-row bands)", "bounce": N_BOUNCE, "shadow_any_hit": N_SHADOW,
            "bvh": "binned SAH 128 bins, cost-optimal 8-wide collapse (leaves <= 3 tris), quantised (80 B nodes)",
            "l2": f"inputs larger than L2 ({(WIDTH * HEIGHT + N_BOUNCE + N_SHADOW) * RAY_IN_BYTES / 1e6:.0f} MB of rays per step); no flush"}


def build_workload(seed=1, log=print):
    """Scene + 16M-ray batch (numpy). Bounce/shadow rays need primary hits: traced on the GPU when
    a BVH is given, else (reference arm) on a CPU structure."""
    from gbpt import scenes
    t0 = time.time()
    mesh = scenes.traversal_scene(cells=1024, n_random=200_000, seed=seed)
    log(f"scene: {mesh.n_triangles} triangles in {time.time() - t0:.1f}s")
    primary = scenes.pinhole_rays(WIDTH, HEIGHT, vfov_deg=VFOV, order="bands")
    return mesh, primary


def secondary_rays(mesh, primary, primary_hits, seed=1):
    from gbpt import scenes
    pts, nrm, prim = scenes.hit_points_normals(mesh, primary, primary_hits)
    hit_idx = np.nonzero(prim >= 0)[0]
    rng = np.random.Generator(np.random.PCG64(seed + 100))
    # rays are emitted in the order of the primary rays they continue (as a wavefront's queues
    # keep path order); their directions stay incoherent
    pick_b = np.sort(rng.choice(hit_idx, N_BOUNCE, replace=len(hit_idx) < N_BOUNCE))
    pick_s = np.sort(rng.choice(hit_idx, N_SHADOW, replace=len(hit_idx) < N_SHADOW))
    bounce = scenes.bounce_rays(pts[pick_b], nrm[pick_b], prim[pick_b], seed=seed + 2)
    shadow, _ = scenes.shadow_rays(pts[pick_s], prim[pick_s], seed=seed + 3)
    return bounce, shadow


class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = [l.split(", ") for (t, l) in self.lines if t0 <= t <= t1 + 0.15]
        rows = [r for r in rows if len(r) >= 10]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[6 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[4]) for r in rows if r[4].replace(".", "").isdigit()) if rows else None}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


TRAVERSAL_SOURCES = ("bvh.h", "bvh_build.cpp", "trace.cu", "trace_core.h", "trace_kernels.h")


def kernel_source_hash():
    """SHA-256 (16 hex digits) of the sources that make the traversal kernels and the BVH they
    walk (trace.cu and the headers it includes, the BVH builder), in file-name order."""
    import hashlib
    csrc = os.path.join(REPO, "hiprt-path-tracer_gb300", "csrc")
    h = hashlib.sha256()
    for name in TRAVERSAL_SOURCES:
        h.update(name.encode())
        with open(os.path.join(csrc, name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def ncu_traffic(key="dram_bytes_per_ray"):
    """DRAM (or, key l2_bytes_per_ray, L2) bytes per closest-hit ray from the committed ncu summary
    of the closest-hit kernels, used only when that capture was taken of these very sources (its
    source_hash line matches), else None: a capture of another build says nothing about this one."""
    path = os.path.join(REPO, "profiles", "trace_closest_traffic.txt")
    vals = {}
    try:
        for line in open(path):
            if "=" in line and not line.startswith("#"):
                k, v = line.strip().split("=", 1)
                vals[k] = v
    except OSError:
        return None
    if vals.get("source_hash") != kernel_source_hash() or key not in vals:
        return None
    return float(vals[key])


def l2_copy_peak(dev, sizes_mb=(8, 16, 32, 48), reps=200):
    """Measured L2 bandwidth of this GPU: a device-to-device copy of a buffer pair that fits in the
    129 MB L2 (read + write bytes per second, CUDA events, best over the buffer sizes), the L2
    counterpart of the measured HBM copy peak. Returns (GB/s, {size MB: GB/s})."""
    import torch
    by_size = {}
    for mb in sizes_mb:
        n = mb * (1 << 20) // 4
        a = torch.rand(n, device=dev)
        b = torch.empty_like(a)
        for _ in range(10):
            b.copy_(a)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            b.copy_(a)
        e1.record()
        torch.cuda.synchronize()
        by_size[mb] = 2 * n * 4 / (e0.elapsed_time(e1) / reps * 1e-3) / 1e9
        del a, b
    return max(by_size.values()), by_size


def make_cpu_impl(mesh, log=print):
    """The reference CPU traversal over all host cores: the reference's own code (oracle/_ref) where
    it was compiled for this machine, else the oracle's restatement. Returns (closest, occluded, kind)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    soup = mesh.triangle_soup()
    cores = os.cpu_count() or 1
    if pyoracle.ref_available():
        try:
            ref = pyoracle.RefBVH(soup)
            # the reference's shadow test subtracts 1e-4 from the light distance itself
            return (lambda r: ref.closest(r),
                    lambda r: ref.shadow_occluded(r, (r.dir_tmax[:, 3] + np.float32(1e-4)).astype(np.float32)),
                    "reference", cores)
        except OSError:
            pass
    orc = pyoracle.Oracle()
    t0 = time.time()
    oc = orc.octree(soup)
    log(f"oracle octree build {time.time() - t0:.1f}s ({oc.node_count} nodes)")
    return (lambda r: oc.closest(r, nthreads=cores), lambda r: oc.occluded(r, nthreads=cores), "port", cores)


def cpu_baseline_sample(impl, primary, bounce, shadow, frac):
    """Times the CPU traversal on a strided sample of each ray class."""
    closest, occluded, kind, cores = impl
    step = max(1, int(round(1.0 / frac)))
    samples = [primary.slice(slice(0, None, step)), bounce.slice(slice(0, None, step)),
               shadow.slice(slice(0, None, step))]
    n = sum(len(s) for s in samples)
    t0 = time.perf_counter()
    closest(samples[0])
    closest(samples[1])
    occluded(samples[2])
    dt = time.perf_counter() - t0
    return {"value": n / dt / 1e6, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"every {step}th ray of each class ({n} rays: {len(samples[0])} primary, {len(samples[1])} bounce, "
                      f"{len(samples[2])} shadow), {dt:.2f}s"}, dt


def _orbit(eye, target, deg):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    ex, ez = eye[0] - target[0], eye[2] - target[2]
    return (target[0] + c * ex + s * ez, eye[1], target[2] - s * ex + c * ez)


def _relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


RENDER_WORKLOADS = ("cornell", "envmap", "restir", "guided", "guided_indirect_cornell", "batch")
OPTIONAL_WORKLOADS = ("guided_spec",)  # run only when named in --workloads


def render_workloads(log, guided_res=(480, 270), cpu_baseline=True, only=RENDER_WORKLOADS, restir_res=(1920, 1080)):
    """Path-tracing workloads (one GPU, inputs resident; timed with CUDA events on the current stream):

    cornell     the Cornell box, 256 x 256, 64 launches x 1 spp, 4 bounces, RR from bounce 3, uniform
                light sampling NEE + BSDF MIS, Lambertian; relMSE against a 65536-spp FP64 image;
                cpu_baseline = the oracle's restatement of the reference's CPU estimator on all host
                cores over a bounded sample.
    envmap      the Cornell box under a 2048 x 1024 sky, 512 x 512: envmap table build time and samples/s
                with alias-table envmap sampling, against the same scene without a world.
    restir      the many-light principled scene (16,777,216 + 10,000 emissive triangles), 1920 x 1080,
                8 frames with the camera orbiting 0.5 degrees per frame, 3 indirect bounces, power
                light sampling, ReSTIR DI (32 light + 1 BSDF candidates, visibility reuse, M-cap 20,
                1 spatial pass of 5 neighbours in 30 px).
    guided      the same scene at guided_res, 8 bounces, 64 x 1 spp per image, ReSTIR DI at the primary
                vertex in both arms (configs[2]'s plain method): plain continuations against learned
                guiding (training online every launch, its time included), both over 4 consecutive
                64-spp images after a 64-launch warm-up; relMSE against a 2048-spp plain FP64 image.
                time_to_equal_relmse_speedup = (relMSE x time) plain / (relMSE x time) guided. Also the
                relMSE of the primary vertex's direct light alone (0 bounces, against a direct-only
                reference) and its share of the full image's relMSE.
    """
    import torch
    import gbpt
    from gbpt import guide, scenes
    from gbpt.render import (BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings, guide_render_settings, look_at_camera,
                             restir_di_settings)
    stream = torch.cuda.current_stream()

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    out = {}
    # ---- Cornell box ----
    cb = scenes.cornell_box()
    cscene = gbpt.Scene.from_cornell(cb)
    if "cornell" in only:
        cornell_workload(out, cb, cscene, timed, cpu_baseline)
    # ---- the Cornell box under an importance-sampled environment map ----
    if "envmap" in only:
        out["envmap"] = envmap_workload(timed, cscene)
    del cscene
    if "restir" in only or "guided" in only or "guided_spec" in only:
        many_light_workloads(out, log, timed, guided_res, only, restir_res, cpu_baseline)
    # ---- guided against plain on the indirectly lit Cornell box ----
    if "guided_indirect_cornell" in only:
        out["guided_indirect_cornell"] = guided_indirect_cornell(timed)
    torch.cuda.empty_cache()
    # ---- batched jobs ----
    if "batch" in only:
        out["batch"] = batch_workload(timed, log, cpu_baseline=cpu_baseline)
    return out


def cornell_workload(out, cb, cscene, timed, cpu_baseline):
    import torch
    import gbpt
    # the FP64-accumulated 65,536-spp reference image (256 launches of 256 spp, independent seed)
    ref = gbpt.Renderer(cscene, gbpt.cornell_settings(256, 256, samples_per_launch=256, seed=1000))
    t_ref = timed(lambda: ref.render(256))
    cref = ref.image_sums()[1] / (256 * 256)
    del ref
    r = gbpt.Renderer(cscene, gbpt.cornell_settings(256, 256, samples_per_launch=1, seed=1))
    r.render(3)
    r.reset()
    ms = timed(lambda: r.render(64))
    st = r.stats()
    rays = st["extension_rays"] + st["shadow_rays"] + st["bsdf_light_rays"]
    out["cornell"] = {"config": "256x256, 64 launches x 1 spp, 4 bounces, RR from 3, uniform NEE + BSDF MIS, Lambert",
                      "ms": ms, "samples_per_s": 256 * 256 * 64 / (ms * 1e-3), "mrays_per_s": rays / (ms * 1e-3) / 1e6,
                      "relmse_vs_65536spp_fp64": _relmse(r.image_sums()[1] / 64, cref),
                      "reference_ms": t_ref}
    del r
    if cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import pyoracle
        pyoracle.build(ref=False)
        lt = cscene.light_table()
        cores = os.cpu_count() or 1
        cst = gbpt.cornell_settings(256, 256, samples_per_launch=1, seed=1)
        t0 = time.perf_counter()
        spp = 128
        pyoracle.pt_render(cb.mesh.triangle_soup(), cb.material_of_triangle, cb.albedo, cb.emission, lt["emissive"],
                           lt["probas"], lt["alias"], lt["power_sum"], cst, spp, nthreads=cores)
        dt = time.perf_counter() - t0
        out["cornell"]["cpu_baseline"] = {"value": 256 * 256 * spp / dt, "unit": "samples/s", "cores": cores,
                                          "kind": "port", "sample": f"256x256 x {spp} spp, {dt:.2f}s"}


def many_light_workloads(out, log, timed, guided_res, only, restir_res=(1920, 1080), cpu_baseline=True):
    RW, RH = restir_res
    import numpy as np
    import torch
    import gbpt
    from gbpt import guide, scenes
    from gbpt.render import (BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings, guide_render_settings, look_at_camera,
                             restir_di_settings)
    # ---- many-light principled scene ----
    t0 = time.time()
    S = scenes.many_light_scene()
    scene = gbpt.Scene(S.mesh.positions, S.mesh.indices, S.material_of_triangle, principled=S.materials)
    torch.cuda.synchronize()
    log(f"many-light scene: {S.mesh.n_triangles} triangles, scene + BVH {time.time() - t0:.1f}s")

    def settings(w, h, spp, nb, seed, eye=None):
        iv, ip = look_at_camera(eye or S.eye, S.target, vfov_deg=S.vfov_deg, aspect=w / h)
        return RenderSettings(width=w, height=h, samples_per_launch=spp, nb_bounces=nb, light_sampling=LIGHT_POWER,
                              bsdf=BSDF_PRINCIPLED, seed=seed, inverse_view=iv, inverse_projection=ip)

    def restir_frames(**extra):
        r = gbpt.Renderer(scene, settings(RW, RH, 1, 3, 1))
        r.set_restir_di(restir_di_settings(light_candidates=32, bsdf_candidates=1, m_cap=20, spatial_passes=1,
                                           spatial_neighbors=5, spatial_radius=30, **extra))
        r.render(3)
        r.reset()
        frame_ms = []
        for f in range(8):
            iv, ip = look_at_camera(_orbit(S.eye, S.target, 0.5 * f), S.target, vfov_deg=S.vfov_deg, aspect=RW / RH)
            r.set_camera(iv, ip)
            frame_ms.append(timed(lambda: r.render(1)))
        st = r.stats()
        del r
        return frame_ms, st["extension_rays"] + st["shadow_rays"] + st["bsdf_light_rays"]

    if "restir" in only:
        restir_workload(out, restir_frames, RW, RH)
    if "guided" in only:
        guided_workload(out, scene, S, settings, timed, guided_res, log)
    if cpu_baseline and ("restir" in out or "guided" in out):
        many_light_cpu_baselines(out, scene, S, settings, log)
    if "guided_spec" in only:
        guided_spec_workload(out, scene, S, settings, timed, log)
    del scene


def oracle_principled_scene(mesh, material_of, materials, light_table, log, cores):
    """The oracles' view of a principled scene for a CPU baseline: the triangle soup, the
    coat-roughened material records, the light table, and an octree over the triangles set as
    the oracles' scene accelerator (the exhaustive test would not finish on these scenes).
    Returns (pyoracle, scene dict, effective materials, octree, build seconds)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    from gbpt import materials as M
    soup = np.ascontiguousarray(mesh.triangle_soup(), np.float32)
    eff = M.pack_many([M.coat_roughened(M.unpack(materials[i])) for i in range(len(materials))])
    t0 = time.time()
    oc = pyoracle.Oracle().octree(soup)
    build_s = time.time() - t0
    pyoracle.set_scene_accel(oc)
    sc = dict(soup=soup, material_of=np.ascontiguousarray(material_of, np.int32),
              emission=np.ascontiguousarray(materials[:, 4:7], np.float32), emissive=light_table["emissive"],
              alias_prob=light_table["probas"], alias_idx=light_table["alias"], power_sum=light_table["power_sum"])
    log(f"CPU baseline: octree over {len(soup)} triangles in {build_s:.1f}s ({cores} threads)")
    return pyoracle, sc, eff, oc, build_s


def many_light_cpu_baselines(out, scene, S, settings, log, W=480, H=270):
    """CPU baselines of the many-light workloads: the oracles (the reference's estimator restated,
    tracing through an octree restating the reference's CPU BVH, shading with the library's
    principled BSDF compiled for the host: the reference's own BSDF needs the reference tree) on
    all host cores, on a W x H rendering of the same camera:
      restir: one frame's ReSTIR DI passes (G-buffer, 32 + 1 initial candidates with visibility
        reuse, spatial reuse of 5 neighbours) plus the path's 3 bounces of MIS next-event
        estimation, in samples (pixels) per second;
      guided: plain path tracing with 8 bounces, 1 spp (the reference has no guiding), in samples
        per second."""
    cores = os.cpu_count() or 1
    pyoracle, sc, eff, oc, build_s = oracle_principled_scene(S.mesh, S.material_of_triangle, S.materials,
                                                               scene.light_table(), log, cores)
    try:
        from gbpt.render import look_at_camera
        iv, ip = look_at_camera(S.eye, S.target, vfov_deg=S.vfov_deg, aspect=W / H)
        ivm = np.asarray(iv, np.float32).reshape(4, 4)
        cam = [float(ivm[0, 3]), float(ivm[1, 3]), float(ivm[2, 3])]
        if "restir" in out:
            si = [W, H, 1, 0, 0, 1, 32, 1, 1, 0, 8, 1, 5, 20, 1, 1]
            sf = [4.0, 30.0, 0.906307787, 0.1, *cam, *cam]
            t0 = time.perf_counter()
            gb = pyoracle.restir_gbuffer(sc["soup"], sc["material_of"], eff, W, H, 1, 0, True, iv, ip, nthreads=cores)
            init = pyoracle.restir_pass(0, sc, eff, si, sf, None, gb, nthreads=cores, bsdf="host")
            pyoracle.restir_pass(2, sc, eff, si, sf, None, gb, inp=init, spatial_index=0, spatial_seed=1,
                                 nthreads=cores, bsdf="host")
            t_restir = time.perf_counter() - t0
            st = settings(W, H, 1, 3, 1)
            t0 = time.perf_counter()
            pyoracle.pt_render_principled(sc["soup"], sc["material_of"], eff, sc["emission"], sc["emissive"],
                                          sc["alias_prob"], sc["alias_idx"], sc["power_sum"], st, 1, nthreads=cores,
                                          bsdf="host")
            t_pt = time.perf_counter() - t0
            dt = t_restir + t_pt
            out["restir"]["cpu_baseline"] = {
                "value": W * H / dt, "unit": "samples/s", "cores": cores, "kind": "port",
                "sample": f"{W}x{H}, 1 frame: ReSTIR DI passes {t_restir:.2f}s + 3-bounce path tracing {t_pt:.2f}s "
                          f"(octree built in {build_s:.1f}s, not timed)"}
        if "guided" in out:
            st = settings(W, H, 1, 8, 2)
            t0 = time.perf_counter()
            pyoracle.pt_render_principled(sc["soup"], sc["material_of"], eff, sc["emission"], sc["emissive"],
                                          sc["alias_prob"], sc["alias_idx"], sc["power_sum"], st, 1, nthreads=cores,
                                          bsdf="host")
            dt = time.perf_counter() - t0
            out["guided"]["cpu_baseline"] = {"value": W * H / dt, "unit": "samples/s", "cores": cores, "kind": "port",
                                             "sample": f"{W}x{H} x 1 spp, 8 bounces, plain path tracing, {dt:.2f}s"}
    finally:
        pyoracle.set_scene_accel(None)
        del oc


def restir_workload(out, restir_frames, RW=1920, RH=1080):
    frame_ms, rays = restir_frames()
    tot = sum(frame_ms)
    fused_ms, _ = restir_frames(do_fused_spatiotemporal=1)
    fused_ps_ms, _ = restir_frames(do_fused_spatiotemporal=1, do_light_presampling=1)
    out["restir"] = {"config": f"many-light scene 16.8M + 10k emissive tris, {RW}x{RH}, 8 frames orbiting 0.5 deg, 3 bounces, "
                               "ReSTIR DI 32+1 candidates, visibility reuse, M-cap 20, 1 spatial pass 5 neighbours 30 px",
                     "ms_per_frame": tot / 8, "frame_ms": frame_ms, "samples_per_s": RW * RH * 8 / (tot * 1e-3), "resolution": [RW, RH],
                     "mrays_per_s_traced": rays / (tot * 1e-3) / 1e6,
                     "fused_spatiotemporal_ms_per_frame": sum(fused_ms) / 8,
                     "fused_and_light_presampling_ms_per_frame": sum(fused_ps_ms) / 8,
                     "light_presampling": "128 subsets x 1024 lights, 8x8-pixel tiles"}



def guided_workload(out, scene, S, settings, timed, guided_res, log):
    import numpy as np
    import torch
    import gbpt
    from gbpt import guide
    from gbpt.render import guide_render_settings, restir_di_settings
    # ---- guided against plain, both with ReSTIR DI at the primary vertex (configs[2]'s plain
    # method; the guide acts on the continuations and on later bounces' BSDF technique) ----
    W, H = guided_res
    ref = gbpt.Renderer(scene, settings(W, H, 64, 8, 1000))
    ref.render(32)
    torch.cuda.synchronize()
    gref = ref.image_sums()[1] / 2048
    del ref
    rs = restir_di_settings(light_candidates=32, bsdf_candidates=1, m_cap=20, spatial_passes=1, spatial_neighbors=5,
                            spatial_radius=30)

    def arm(guided, seed, nb=8, ref_img=None, images=4):
        r = gbpt.Renderer(scene, settings(W, H, 1, nb, seed))
        r.set_restir_di(rs)
        gd = None
        if guided:
            gd = guide.Guide(scene_min=S.box[0], scene_max=S.box[1])
            r.set_guide(gd, guide_render_settings())
        r.render(64)  # warm-up: temporal reservoirs and, guided, 64 training steps
        res = []
        for _ in range(images):
            torch.cuda.synchronize()
            prev = r.image_sums()[1]
            t = timed(lambda: r.render(64))
            res.append((t, _relmse((r.image_sums()[1] - prev) / 64, gref if ref_img is None else ref_img)))
        return res, gd

    plain, _ = arm(False, 100)
    guided, gd = arm(True, 200)
    # how much of the error the primary vertex's direct light carries: the same estimator with no
    # bounce, against a direct-only reference
    dref = gbpt.Renderer(scene, settings(W, H, 64, 0, 1001))
    dref.render(32)
    torch.cuda.synchronize()
    direct_ref = dref.image_sums()[1] / 2048
    del dref
    direct, _ = arm(False, 300, nb=0, ref_img=direct_ref, images=2)
    tp, ep = np.mean([a for a, _ in plain]), np.mean([b for _, b in plain])
    tg, eg = np.mean([a for a, _ in guided]), np.mean([b for _, b in guided])
    out["guided"] = {"config": f"many-light scene, {W}x{H}, 8 bounces, 64 x 1 spp per image, ReSTIR DI at the primary vertex "
                               "(32+1 candidates, M-cap 20, 1 spatial pass x 5 in 30 px) and power NEE + MIS after it "
                               "in both arms; guide: 16-level hash grid + 3x64 MLP, 8 vMF lobes + learned selection, "
                               "2^18 records/launch, Adam 1e-2; relMSE vs a 2048-spp plain FP64 image",
                     "plain_ms": tp, "plain_relmse": ep, "guided_ms": tg, "guided_relmse": eg,
                     "plain_relmse_each": [b for _, b in plain], "guided_relmse_each": [b for _, b in guided],
                     "time_to_equal_relmse_speedup": (ep * tp) / (eg * tg), "guide_error_flag": gd.error_flag(),
                     # the mean over 4 images is what the speedup uses; one firefly image can dominate
                     # it, so the medians are reported beside it
                     "plain_relmse_median": float(np.median([b for _, b in plain])),
                     "guided_relmse_median": float(np.median([b for _, b in guided])),
                     "primary_direct_only_relmse": float(np.mean([b for _, b in direct])),
                     "primary_direct_share_of_relmse": float(np.mean([b for _, b in direct])) / ep}


def guided_spec_workload(out, scene, S, settings, timed, log, W=1920, H=1080, spp=256, nb=8, ref_spp=4096):
    """Guided against plain at the guided-rendering configuration's size: the many-light scene at
    1920 x 1080, 8 bounces, one 256-spp image per arm (256 launches of 1 spp; ReSTIR DI at the
    primary vertex in both, the guide trained online from the first launch), relMSE against an
    FP64-accumulated plain image of ref_spp samples per pixel (64 launches of 64 spp). Not in the
    default workload list: the reference alone is ~8.5G path samples."""
    import numpy as np
    import torch
    import gbpt
    from gbpt import guide
    from gbpt.render import guide_render_settings, restir_di_settings
    ref = gbpt.Renderer(scene, settings(W, H, 64, nb, 5000))
    t_ref = timed(lambda: ref.render(ref_spp // 64))
    gref = ref.image_sums()[1] / ref_spp
    del ref
    torch.cuda.empty_cache()
    rs = restir_di_settings(light_candidates=32, bsdf_candidates=1, m_cap=20, spatial_passes=1, spatial_neighbors=5,
                            spatial_radius=30)
    res = {}
    for name, guided, seed in (("plain", False, 5100), ("guided", True, 5200)):
        r = gbpt.Renderer(scene, settings(W, H, 1, nb, seed))
        r.set_restir_di(rs)
        gd = None
        if guided:
            gd = guide.Guide(scene_min=S.box[0], scene_max=S.box[1])
            r.set_guide(gd, guide_render_settings())
        t = timed(lambda: r.render(spp))
        res[name] = (t, _relmse(r.image_sums()[1] / spp, gref), gd.error_flag() if gd else 0)
        log(f"guided_spec {name}: {t / 1e3:.1f} s, relMSE {res[name][1]:.4f}")
        del r, gd
        torch.cuda.empty_cache()
    (tp, ep, _), (tg, eg, flag) = res["plain"], res["guided"]
    out["guided_spec"] = {"config": f"many-light scene, {W}x{H}, {nb} bounces, {spp} spp per arm (launches of 1 spp), "
                                    "ReSTIR DI at the primary vertex in both arms, guide trained online from the first "
                                    f"launch; relMSE vs a {ref_spp}-spp plain FP64 image",
                          "plain_ms": tp, "plain_relmse": ep, "guided_ms": tg, "guided_relmse": eg,
                          "time_to_equal_relmse_speedup": (ep * tp) / (eg * tg), "reference_ms": t_ref,
                          "guide_error_flag": flag}


def envmap_workload(timed, cscene, res=512, launches=32):
    """The Cornell box (open side facing the camera, 60 degree FOV) under a seeded 2048 x 1024 sky
    with a sun: table build time (RGB9E5 packing, FP64 CDF and sum on the device, Vose alias table
    on the host; 2M and 8M texels), then res^2 x launches x 1 spp with the envmap sampled by alias
    table (envmap pass + shade + shadow / BSDF-light / envmap any-hit rays), against the same scene
    without a world."""
    import torch
    import gbpt
    from gbpt import scenes
    from gbpt.render import AMBIENT_ENVMAP, World
    iv, ip = gbpt.look_at_camera((2.75, 2.75, -8.0), (2.75, 2.75, 0.0), vfov_deg=60.0)
    st = gbpt.cornell_settings(res, res, samples_per_launch=1, seed=1, inverse_view=iv, inverse_projection=ip)
    build_ms = {}
    for w, h in ((2048, 1024), (4096, 2048)):
        sky = scenes.sky_envmap(w, h, seed=3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cscene.set_world(World(ambient=AMBIENT_ENVMAP, envmap=sky))
        build_ms[f"{w}x{h}"] = (time.perf_counter() - t0) * 1e3
    cscene.set_world(World(ambient=AMBIENT_ENVMAP, envmap=scenes.sky_envmap(2048, 1024, seed=3)))
    res_out = {}
    for tag in ("envmap", "no_world"):
        if tag == "no_world":
            cscene.set_world(World())
        r = gbpt.Renderer(cscene, st)
        r.render(3)
        r.reset()
        ms = timed(lambda: r.render(launches))
        s = r.stats()
        rays = s["extension_rays"] + s["shadow_rays"] + s["bsdf_light_rays"]
        res_out[tag] = {"ms": ms, "samples_per_s": res * res * launches / (ms * 1e-3),
                        "mrays_per_s": rays / (ms * 1e-3) / 1e6}
        del r
    return {"config": f"Cornell box under a 2048x1024 sky (sun), {res}x{res}, {launches} x 1 spp, 4 bounces, "
                      "alias-table envmap sampling + BSDF MIS, uniform NEE + BSDF MIS, Lambert",
            "table_build_ms": build_ms, **res_out}


def batch_jobs(n_jobs=48, seed=1):
    """The batched workload's jobs, drawn from seed: resolution uniform over {128, 256, 512, 1024}^2,
    a heightfield of 64^2..512^2 cells (fBm amplitude 0.2, 8k-524k triangles) plus 0..2000 emissive
    triangles above it, random principled materials (the many-light distribution), bounces
    U[2, 16], spp U[4, 64], camera above the tile looking at its centre, power light sampling."""
    import gbpt
    from gbpt import materials as M, scenes
    from gbpt.render import BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings, look_at_camera
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        res = int(rng.choice([128, 256, 512, 1024]))
        cells = int(rng.integers(64, 513))
        n_emit = int(rng.integers(0, 2001))
        hf = scenes.heightfield(cells=cells, amplitude=0.2, seed=int(rng.integers(1, 1 << 30)))
        parts, mat_of = [hf], [rng.integers(0, 4, hf.n_triangles)]
        mats = M.random_principled(rng, 4)
        if n_emit:
            em = scenes.random_triangles(n_emit, seed=int(rng.integers(1, 1 << 30)), lo=(-1.0, 0.35, -1.0),
                                         hi=(1.0, 1.2, 1.0), sigma=0.02)
            parts.append(em)
            rad = np.exp(rng.uniform(0.0, np.log(1000.0), n_emit))
            mats += [dict(base_color=(0.0, 0.0, 0.0), emission=(float(r), float(r) * 0.8, float(r) * 0.6)) for r in rad]
            mat_of.append(4 + np.arange(n_emit))
        else:  # no emitters: a single bright emissive quad-like triangle pair keeps the job lit
            em = scenes.Mesh(np.array([[-0.3, 1.5, -0.3], [0.3, 1.5, -0.3], [0.3, 1.5, 0.3], [-0.3, 1.5, 0.3]], np.float32),
                             np.array([[0, 1, 2], [0, 2, 3]], np.int32))
            parts.append(em)
            mats.append(dict(base_color=(0.0, 0.0, 0.0), emission=(20.0, 18.0, 15.0)))
            mat_of.append(np.array([4, 4]))
        mesh = scenes.merge(*parts)
        scene = gbpt.Scene(mesh.positions, mesh.indices, np.concatenate(mat_of).astype(np.int32),
                           principled=M.pack_many(mats))
        ang = rng.uniform(0, 2 * np.pi)
        eye = (2.2 * np.cos(ang), 1.6, 2.2 * np.sin(ang))
        iv, ip = look_at_camera(eye, (0.0, 0.0, 0.0), vfov_deg=50.0, aspect=1.0)
        st = RenderSettings(width=res, height=res, samples_per_launch=int(rng.integers(4, 65)),
                            nb_bounces=int(rng.integers(2, 17)), light_sampling=LIGHT_POWER, bsdf=BSDF_PRINCIPLED,
                            seed=int(rng.integers(1, 1 << 30)), inverse_view=iv, inverse_projection=ip)
        jobs.append((scene, st, {"res": res, "triangles": int(mesh.n_triangles), "emitters": n_emit,
                                 "bounces": st.nb_bounces, "spp": st.samples_per_launch},
                     (mesh, np.concatenate(mat_of).astype(np.int32), M.pack_many(mats))))
    return jobs


def batch_cpu_baseline(jobs, picks, log):
    """CPU baseline of the batch: the path-tracing oracle (the reference's estimator restated,
    tracing through an octree restating the reference's CPU BVH, shading with the library's
    principled BSDF compiled for the host) on all host cores, `spp` samples per pixel of each picked
    job at its own settings; samples per second over the picked jobs."""
    cores = os.cpu_count() or 1
    spp = 32
    total_px, total_s, notes = 0, 0.0, []
    for j in picks:
        sc, st, info, (mesh, mat_of, recs) = jobs[j]
        pyoracle, osc, eff, oc, build_s = oracle_principled_scene(mesh, mat_of, recs, sc.light_table(), log, cores)
        try:
            from gbpt.render import RenderSettings
            one = RenderSettings(**{**st.__dict__, "samples_per_launch": 1})
            t0 = time.perf_counter()
            pyoracle.pt_render_principled(osc["soup"], osc["material_of"], eff, osc["emission"], osc["emissive"],
                                          osc["alias_prob"], osc["alias_idx"], osc["power_sum"], one, spp,
                                          nthreads=cores, bsdf="host")
            dt = time.perf_counter() - t0
        finally:
            pyoracle.set_scene_accel(None)
            del oc
        total_px += st.width * st.height * spp
        total_s += dt
        notes.append(f"job {j} ({info['res']}^2, {info['triangles']} tris, {info['bounces']} bounces) {dt:.2f}s")
    if not picks:
        return None
    return {"value": total_px / total_s, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": f"{spp} spp of " + "; ".join(notes)}


def batch_workload(timed, log, ref_factor=4, cpu_baseline=True):
    """48 jobs in one batched wavefront (one launch per stage for all jobs, one iteration captured
    as a CUDA graph and replayed). samples_per_iteration is picked by timing candidates on the jobs
    clipped to 8 spp; per-job relMSE against an FP64 image of ref_factor x the job's spp (the same
    batch machinery, other seeds), and for the first four 128 x 128 jobs against FP64 65,536-spp
    images; job-completion latency from device timer stamps."""
    import torch
    import gbpt
    from gbpt.render import RenderSettings
    t0 = time.time()
    jobs = batch_jobs()
    log(f"batch: {len(jobs)} jobs built in {time.time() - t0:.1f}s")
    pairs = [(sc, st) for sc, st, _, _ in jobs]
    # autotune samples_per_iteration on the jobs clipped to 8 spp
    clip = [(sc, RenderSettings(**{**st.__dict__, "samples_per_launch": min(8, st.samples_per_launch)})) for sc, st in pairs]
    tune = {}
    for k in (1, 2, 4, 8):
        b = gbpt.Batch(clip, samples_per_iteration=k)
        b.render()
        tune[k] = timed(lambda: b.render())
        del b
    k_best = min(tune, key=tune.get)
    b = gbpt.Batch(pairs, samples_per_iteration=k_best)
    b.render()
    ms = timed(lambda: b.render())
    secs = b.job_seconds()
    st = b.stats()
    imgs = [b.image_sums(j)[1] / pairs[j][1].samples_per_launch for j in range(len(pairs))]
    del b
    ref_pairs = [(sc, RenderSettings(**{**s.__dict__, "samples_per_launch": ref_factor * s.samples_per_launch,
                                       "seed": s.seed + 7919})) for sc, s in pairs]
    rb = gbpt.Batch(ref_pairs, samples_per_iteration=k_best)
    t_ref = timed(lambda: rb.render())
    rel = []
    for j in range(len(pairs)):
        ref = rb.image_sums(j)[1] / ref_pairs[j][1].samples_per_launch
        rel.append(_relmse(imgs[j], ref))
    del rb
    # FP64 65,536-spp references (64 launches of 1,024 spp, other seeds) for the first four 128 x 128
    # jobs: a full-set 65,536-spp reference would be ~10^12 samples
    small = [j for j in range(len(pairs)) if pairs[j][1].width == 128][:4]
    rel64k, t64k = [], 0.0
    for j in small:
        sc, s = pairs[j]
        rr = gbpt.Renderer(sc, RenderSettings(**{**s.__dict__, "samples_per_launch": 1024, "seed": s.seed + 104729}))
        t64k += timed(lambda: rr.render(64))
        rel64k.append(_relmse(imgs[j], rr.image_sums()[1] / 65536))
        del rr
    samples = st["samples"]
    rays = st["extension_rays"] + st["shadow_rays"] + st["bsdf_light_rays"]
    return {"config": "48 jobs from seed 1: res {128,256,512,1024}^2, heightfield 64^2..512^2 cells + 0..2000 emitters, "
                      "principled, bounces U[2,16], spp U[4,64]; one wavefront, one graph per iteration",
            "samples_per_iteration": k_best, "autotune_ms_8spp": tune, "ms": ms, "samples": samples,
            "samples_per_s": samples / (ms * 1e-3), "mrays_per_s": rays / (ms * 1e-3) / 1e6,
            "job_latency_s": {"p50": float(np.percentile(secs, 50)), "p99": float(np.percentile(secs, 99)),
                              "max": float(secs.max())},
            "relmse_vs_fp64": {"reference_spp_factor": ref_factor, "reference_ms": t_ref,
                               "median": float(np.median(rel)), "max": float(np.max(rel)),
                               "each": [round(x, 5) for x in rel]},
            "relmse_vs_65536spp_fp64": {"jobs": small, "each": [round(x, 5) for x in rel64k],
                                        "median": float(np.median(rel64k)) if rel64k else None,
                                        "reference_ms": t64k},
            "jobs": [j for _, _, j, _ in jobs],
            "cpu_baseline": batch_cpu_baseline(jobs, small[:2], log) if cpu_baseline else None}


def indirect_cornell_scene():
    """The Cornell box with its light lowered to y = 4.5 and turned to face the ceiling: the room is
    lit almost only by the bright patch the light makes on the ceiling."""
    import gbpt
    from gbpt import scenes
    cb = scenes.cornell_box()
    pos = cb.mesh.positions.copy()
    for t in cb.emissive_triangles:
        i = cb.mesh.indices[t]
        pos[i, 1] = 4.5
        pos[[i[1], i[2]]] = pos[[i[2], i[1]]]
    return gbpt.Scene(pos, cb.mesh.indices, cb.material_of_triangle, cb.albedo, cb.emission)


def guided_indirect_cornell(timed, res=128, warm_launches=100):
    """Plain against guided path tracing on the indirectly lit Cornell box, res x res, 4 bounces,
    Lambertian: 4 independent 64-spp images each after the guide's warm-up of warm_launches x 4 spp
    (not timed); relMSE against a 16384-spp plain FP64 image."""
    import torch
    import gbpt
    from gbpt import guide
    from gbpt.render import guide_render_settings
    scene = indirect_cornell_scene()
    ref = gbpt.Renderer(scene, gbpt.cornell_settings(res, res, samples_per_launch=256, seed=1000))
    ref.render(64)
    torch.cuda.synchronize()
    cref = ref.image_sums()[1] / 16384
    del ref
    plain = []
    for k in range(4):
        p = gbpt.Renderer(scene, gbpt.cornell_settings(res, res, samples_per_launch=4, seed=100 + k))
        t = timed(lambda: p.render(16))
        plain.append((t, _relmse(p.image_sums()[1] / 64, cref)))
    g = gbpt.Renderer(scene, gbpt.cornell_settings(res, res, samples_per_launch=4, seed=200))
    gd = guide.Guide(scene_min=(0, 0, 0), scene_max=(5.5, 5.5, 5.5))
    g.set_guide(gd, guide_render_settings())
    g.render(warm_launches)
    guided = []
    for k in range(4):
        torch.cuda.synchronize()
        prev = g.image_sums()[1]
        t = timed(lambda: g.render(16))
        guided.append((t, _relmse((g.image_sums()[1] - prev) / 64, cref)))
    tp, ep = np.mean([a for a, _ in plain]), np.mean([b for _, b in plain])
    tg, eg = np.mean([a for a, _ in guided]), np.mean([b for _, b in guided])
    return {"config": f"Cornell box lit through the ceiling, {res}x{res}, 4 bounces, Lambert, 64 spp per image, guide warm-up "
                      f"{warm_launches} x 4 spp (untimed); training continues during the timed images",
            "plain_ms": tp, "plain_relmse": ep, "guided_ms": tg, "guided_relmse": eg,
            "equal_spp_relmse_ratio": eg / ep, "time_to_equal_relmse_speedup": (ep * tp) / (eg * tg),
            "guide_error_flag": gd.error_flag()}


def run_reference(args, rank, world):
    if rank != 0:
        return
    mesh, primary = build_workload(log=lambda *a: print(*a, file=sys.stderr))
    impl = make_cpu_impl(mesh, log=lambda *a: print(*a, file=sys.stderr))
    # the secondary rays are derived as on the GPU arm, from the hits of every primary ray (here
    # found by the CPU traversal itself: the same hits, bit for bit, but for exact ties)
    bounce, shadow = secondary_rays(mesh, primary, impl[0](primary))
    frac = args.ref_fraction
    for _ in range(args.warmup):
        cpu_baseline_sample(impl, primary, bounce, shadow, frac / 4)
    vals, times = [], []
    base = None
    for _ in range(args.steps):
        base, dt = cpu_baseline_sample(impl, primary, bounce, shadow, frac)
        vals.append(base["value"])
        times.append(dt)
    value = statistics.median(vals)
    base["value"] = value
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * statistics.median(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene and rays)",
            "config": workload_config(mesh.n_triangles), "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def guide_kernels_case(n, data_seed=1, guide_seed=3):
    """The guide's training and inference kernels on n seeded random samples (positions in the unit
    box, random unit normals / view / incident directions, exponential weights with a fifth zero,
    cosine BSDF pdfs): the case the guide's ncu captures run."""
    import numpy as np
    import torch
    from gbpt import guide
    rng = np.random.default_rng(data_seed)
    P = rng.uniform(0.0, 1.0, (n, 3))
    N, V, D = (rng.normal(size=(n, 3)) for _ in range(3))
    for a in (N, V, D):
        a /= np.linalg.norm(a, axis=1, keepdims=True)
    w = rng.exponential(1.0, n) * (rng.random(n) < 0.8)
    pb = np.maximum((N * D).sum(1), 0.0) / np.pi
    t = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in (P, N, V, D, w, pb)]
    g = guide.Guide(seed=guide_seed)
    for _ in range(2):
        loss = g.train(*t)
        rows = g.infer(t[0], t[1], t[2])
    torch.cuda.synchronize()
    if g.error_flag() != 0:
        raise SystemExit(f"guide kernels reported error flag {g.error_flag()}")
    print(json.dumps({"guide_kernels": n, "loss": float(loss), "rows": list(rows.shape)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbpt", choices=["gbpt", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-fraction", type=float, default=0.5)
    ap.add_argument("--ref-fraction", type=float, default=1.0 / 16,
                    help="reference arm: fraction of each ray class timed per step (1/16: 1,048,576 rays)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-render", action="store_true", help="skip the path-tracing workloads")
    ap.add_argument("--restir-res", default="1920x1080",
                    help="WxH of the ReSTIR workload (a smaller one for ncu captures of its kernels)")
    ap.add_argument("--workloads", default=",".join(RENDER_WORKLOADS),
                    help="comma-separated path-tracing workloads to run (default: all)")
    ap.add_argument("--configs", default=None,
                    help="JSON {primary, bounce, shadow} launch configurations to use instead of autotuning")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: 2048x1024 primary + 1M bounce + 1M shadow rays, no e2e/CPU legs")
    ap.add_argument("--guide-kernels", type=int, default=0, metavar="N",
                    help="profiling case: two training steps and two queries of the guide on N seeded random "
                         "samples, then exit")
    args = ap.parse_args()
    if args.guide_kernels:
        guide_kernels_case(args.guide_kernels)
        return
    if args.warmup < 3:
        args.warmup = 3
    global WIDTH, HEIGHT, N_BOUNCE, N_SHADOW
    if args.small:
        WIDTH, HEIGHT, N_BOUNCE, N_SHADOW = 2048, 1024, 1024 * 1024, 1024 * 1024
        args.no_cpu_baseline = True
        args.no_render = True
        args.e2e_steps = 0

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import gbpt
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def log(*a):
        if rank == 0:
            print(*a, file=sys.stderr)

    gbpt.load()
    mesh, primary = build_workload(log=log)
    t0 = time.time()
    bvh = gbpt.BVH(mesh.indices, mesh.positions)
    st = bvh.stats()
    log(f"bvh: {st['n_nodes']} nodes, depth {st['wide_depth']}, build {st['build_seconds']:.2f}s "
        f"(wall {time.time() - t0:.2f}s)")

    def to_dev(r):
        return (torch.from_numpy(r.origin_tmin).to(dev), torch.from_numpy(r.dir_tmax).to(dev),
                torch.from_numpy(r.last_prim).to(dev))

    P = to_dev(primary)
    hits_p = bvh.closest(*P)
    torch.cuda.synchronize()
    bounce, shadow = secondary_rays(mesh, primary, hits_p.cpu().numpy())
    B, S = to_dev(bounce), to_dev(shadow)
    hits_b = torch.empty((len(bounce), 4), dtype=torch.float32, device=dev)
    occ_s = torch.empty((len(shadow),), dtype=torch.uint8, device=dev)
    n_rays = len(primary) + len(bounce) + len(shadow)
    hit_frac = float((gbpt.hit_prim(hits_p) >= 0).float().mean())

    # traversal statistics (counting build of the same kernels on the same batch)
    cp = bvh.count(*P)
    cb = bvh.count(*B)
    cs = bvh.count(*S, any_hit=True)
    alg_closest = (len(primary) + len(bounce)) * (RAY_IN_BYTES + CLOSEST_OUT_BYTES) + \
        (cp[0] + cb[0]) * NODE_BYTES + (cp[1] + cb[1]) * TRI_BYTES
    alg_any = len(shadow) * (RAY_IN_BYTES + ANY_OUT_BYTES) + cs[0] * NODE_BYTES + cs[1] * TRI_BYTES

    stream = torch.cuda.current_stream()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]

    # launch configurations picked by the autotuner per ray class (outside the timed region)
    t0 = time.time()
    if args.configs:
        given = json.loads(args.configs)
        cfg_p, cfg_b, cfg_s = given["primary"], given["bounce"], given["shadow"]
    else:
        cfg_p, _ = bvh.autotune(*P, store=False)
        cfg_b, _ = bvh.autotune(*B, store=False)
        cfg_s, _ = bvh.autotune(*S, any_hit=True, store=False)
    log(f"launch configurations ({'given' if args.configs else f'autotuned in {time.time() - t0:.1f}s'}): "
        f"primary {cfg_p}, bounce {cfg_b}, shadow {cfg_s}")
    bvh.set_trace_config(False, **cfg_b)
    bvh.set_trace_config(True, **cfg_s)

    def step(e=None):
        if e is not None:
            e[0].record(stream)
        bvh.closest_cfg(*P, out=hits_p, **cfg_p)
        if e is not None:
            e[1].record(stream)
        bvh.closest_cfg(*B, out=hits_b, **cfg_b)
        if e is not None:
            e[2].record(stream)
        bvh.occluded_cfg(*S, out=occ_s, **cfg_s)
        if e is not None:
            e[3].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(1.0)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.time()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for k in range(args.steps):
        step(ev[k])
    end.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    t_wall1 = time.time()
    time.sleep(0.3)
    sampler.stop()
    total_ms = start.elapsed_time(end)
    if dist is not None:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    closest_ms = sum(e[0].elapsed_time(e[2]) for e in ev) / args.steps
    primary_ms = sum(e[0].elapsed_time(e[1]) for e in ev) / args.steps
    bounce_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / args.steps
    any_ms = sum(e[2].elapsed_time(e[3]) for e in ev) / args.steps
    value = world * n_rays / (ms_step * 1e-3) / 1e6
    clocks = sampler.summary(t_wall0, t_wall1)

    # the production (watertight) triangle test on the same batch and launch configurations: its
    # throughput (outside the timed region, a few steps) and how its closest hits differ from the
    # parity test's, classified (gbpt.trace.classify_hit_differences)
    wcfg = [dict(c, triangle_test=1) for c in (cfg_p, cfg_b, cfg_s)]
    hits_pw = torch.empty_like(hits_p)
    hits_bw = torch.empty_like(hits_b)
    occ_sw = torch.empty_like(occ_s)

    def wt_step():
        bvh.closest_cfg(*P, out=hits_pw, **wcfg[0])
        bvh.closest_cfg(*B, out=hits_bw, **wcfg[1])
        bvh.occluded_cfg(*S, out=occ_sw, **wcfg[2])

    for _ in range(2):
        wt_step()
    w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0.record(stream)
    for _ in range(5):
        wt_step()
    w1.record(stream)
    torch.cuda.synchronize()
    wt_ms = w0.elapsed_time(w1) / 5
    from gbpt.trace import classify_hit_differences
    hp_np, hb_np = hits_p.cpu().numpy(), hits_b.cpu().numpy()
    dif_p = classify_hit_differences(mesh, primary, hp_np, hits_pw.cpu().numpy())
    dif_b = classify_hit_differences(mesh, bounce, hb_np, hits_bw.cpu().numpy())
    occ_diff = int((occ_s != occ_sw).sum().item())
    watertight = {"mrays_s": world * n_rays / (wt_ms * 1e-3) / 1e6, "ms_per_step": wt_ms,
                  "vs_moller_trumbore_primary": dif_p, "vs_moller_trumbore_bounce": dif_b,
                  "shadow_decisions_differing": occ_diff}

    # end to end through the host-buffer C entry points (pinned host memory, copies in the call)
    hp = [torch.from_numpy(x).pin_memory() for x in (primary.origin_tmin, primary.dir_tmax, primary.last_prim)]
    hb = [torch.from_numpy(x).pin_memory() for x in (bounce.origin_tmin, bounce.dir_tmax, bounce.last_prim)]
    hs = [torch.from_numpy(x).pin_memory() for x in (shadow.origin_tmin, shadow.dir_tmax, shadow.last_prim)]
    out_p = torch.empty((len(primary), 4), dtype=torch.float32).pin_memory()
    out_b = torch.empty((len(bounce), 4), dtype=torch.float32).pin_memory()
    out_s = torch.empty((len(shadow),), dtype=torch.uint8).pin_memory()

    def e2e_step():
        bvh.set_trace_config(False, **cfg_p)
        bvh.closest_host(*hp, out=out_p.numpy())
        bvh.set_trace_config(False, **cfg_b)
        bvh.closest_host(*hb, out=out_b.numpy())
        bvh.occluded_host(*hs, out=out_s.numpy())

    e2e_s = float("nan")
    if args.e2e_steps > 0:
        for _ in range(2):
            e2e_step()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    if dist is not None:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    if args.e2e_steps > 0:
        assert np.array_equal(out_p.numpy().view(np.uint32), hits_p.cpu().numpy().view(np.uint32))

    peak, peak_kind = measured_peaks()
    achieved = alg_closest / (closest_ms * 1e-3) / 1e9
    traffic_per_ray = ncu_traffic()
    l2_per_ray = ncu_traffic("l2_bytes_per_ray")
    l2_peak, l2_by_size = l2_copy_peak(dev)
    l2_roofline = None
    if l2_per_ray:
        l2_achieved = l2_per_ray * (len(primary) + len(bounce)) / (closest_ms * 1e-3) / 1e9
        l2_roofline = {"bound": "l2", "achieved": l2_achieved, "peak": l2_peak, "unit": "GB/s",
                       "frac": l2_achieved / l2_peak,
                       "peak_source": "measured here: L2-resident device copy, best of " +
                                      ", ".join(f"{k} MB {v:.0f}" for k, v in l2_by_size.items()),
                       "bytes_per_ray": l2_per_ray,
                       "bytes_source": "ncu lts__t_sectors x 32 B per closest-hit ray (profiles/trace_closest_traffic.txt)"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene and rays)", "config": workload_config(mesh.n_triangles),
        "breakdown": {"primary_mrays_s": len(primary) / primary_ms / 1e3, "bounce_mrays_s": len(bounce) / bounce_ms / 1e3,
                      "shadow_mrays_s": len(shadow) / any_ms / 1e3, "primary_hit_fraction": hit_frac,
                      "nodes_per_ray": {"primary": cp[0] / len(primary), "bounce": cb[0] / len(bounce),
                                        "shadow": cs[0] / len(shadow)},
                      "tris_per_ray": {"primary": cp[1] / len(primary), "bounce": cb[1] / len(bounce),
                                       "shadow": cs[1] / len(shadow)},
                      "bvh_build_s": st["build_seconds"], "bvh_nodes": st["n_nodes"], "bvh_depth": st["wide_depth"]},
        "roofline": {"bound": "hbm", "kernel": "closest-hit traversal (primary + bounce launches: "
                     f"{KERNEL_NAMES[cfg_p['kernel']]} + {KERNEL_NAMES[cfg_b['kernel']]})",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": alg_closest / 2,
                     "traffic": (traffic_per_ray * (len(primary) + len(bounce)) / 2) if traffic_per_ray else None,
                     "l2": l2_roofline},
        "e2e": {"value": world * n_rays / e2e_s / 1e6, "unit": UNIT,
                "h2d_bytes_per_step": n_rays * RAY_IN_BYTES,
                "d2h_bytes_per_step": (len(primary) + len(bounce)) * CLOSEST_OUT_BYTES + len(shadow) * ANY_OUT_BYTES},
        "watertight": watertight,
        "gpu_launches": 3 * args.steps,
        "trace_configs": {"primary": cfg_p, "bounce": cfg_b, "shadow": cfg_s},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        del P, B, S
        base, _ = cpu_baseline_sample(make_cpu_impl(mesh, log=log), primary, bounce, shadow, args.cpu_fraction)
        line["cpu_baseline"] = base
    if rank == 0 and not args.no_render:
        del bvh
        torch.cuda.empty_cache()
        only = tuple(w for w in args.workloads.split(",") if w)
        unknown = [w for w in only if w not in RENDER_WORKLOADS + OPTIONAL_WORKLOADS]
        if unknown:
            raise SystemExit(f"unknown workloads {unknown}; choose from {RENDER_WORKLOADS + OPTIONAL_WORKLOADS}")
        rw, rh = (int(v) for v in args.restir_res.split("x"))
        line["render"] = render_workloads(log, cpu_baseline=not args.no_cpu_baseline, only=only, restir_res=(rw, rh))
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
