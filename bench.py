"""Benchmark: Mrays/s of the path tracer on the incoherent-ray stress scene at 1920x1080, 64 spp, depth 8.

A step is one 64-spp render: 64 progressive frames of one sample per pixel through spk_render (exactly the
reference cpu pipeline's 64 Render() calls at spp=1), over the resident scene (fBm terrain 2,097,152
triangles + 64 level-5 icospheres of 20,480 triangles, Lambertian / GGX metal / dielectric materials, sky
cube with a baked sun). Rays = traced segments (extension + shadow).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's CPU path tracer (the restated oracle: the reference itself does not
build here) on this machine's host cores over a bounded sample of the same workload.

The line also carries `nee`: the same workload with next-event estimation on, the occlusion rays in the
wavefront's shadow stage and walked inline (`--no-nee` skips it); `spatial`: the same workload with the
reference's default DenoisePass spatial fill on, multi-frame and frame by frame (`--no-spatial` skips it); `denoise`: the wall time to relMSE 0.01 / 0.003 at 1920x1080 on the same scene for
denoised 1 / 4 / 16 spp rendering (the committed U-Net) vs plain path tracing, against a 16384-spp reference
(`--no-denoise` skips it); and `batch`: 32 uneven render requests over 3 scenes in one batched wavefront
against the same requests rendered one by one (`--no-batch` skips it, `--batch-autotune` adds a tuned run).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WIDTH, HEIGHT, SPP, BOUNCE = 1920, 1080, 64, 8
METRIC = "Mrays/s on 1 GB300 (path tracer, stress scene 1920x1080, 64 spp, depth 8)"
UNIT = "Mrays/s"
NODE_BYTES, TRI_BYTES, RAY_BYTES, HIT_BYTES = 80, 36, 32, 20


def workload_config():
    return {"workload": "stress scene path tracing: fBm terrain 1024^2 cells (2,097,152 tris) + 64 level-5 "
                        "icospheres (20,480 tris each), 1920x1080, 64 spp (64 frames x 1 spp), max depth 8, "
                        "xoshiro256** per-pixel RNG, Lambertian/GGX-metal/dielectric, sky cube with sun",
            "width": WIDTH, "height": HEIGHT, "spp": SPP, "max_depth": BOUNCE, "triangles": 3_407_872,
            "l2_policy": "inputs larger than L2 (BVH + triangles ~127 MB resident, frame buffers 50 MB, path "
                         "state 180 MB per step touched), no explicit flush"}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 4 + k and
                          s[4 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples),
                "power_w_max": max((float(s[2]) for s in self.samples if re.match(r"^[0-9.]+$", s[2])), default=None)}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def init_dist(world: int, backend: str):
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)
        return dist
    return None


def max_over_ranks(dist, value: float) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, value: float) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_ray():
    """DRAM bytes per extension ray of the extend kernel from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "k_wf_extend_stress.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        m = re.search(r"dram_bytes_per_ray\s*=\s*([0-9.]+)", f.read())
    return float(m.group(1)) if m else None


def ncu_issue_profile():
    """The extend kernel's issue-slot use and lanes per instruction from the committed ncu summary (its
    bulk-iteration table), which say what bounds the walk: it is issue-bound, not HBM-bound."""
    path = os.path.join(ROOT, "profiles", "k_wf_extend_stress.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        text = f.read()
    issue = re.search(r"smsp__issue_active \(% of peak\) \| ([0-9.]+) %", text)
    lanes = re.search(r"smsp__thread_inst_executed_per_inst_executed \| ([0-9.]+)", text)
    dram = re.search(r"gpu__dram_throughput \(% of peak\) \| ([0-9.]+) %", text)
    if not (issue and lanes and dram):
        return None
    return {"issue_active": round(float(issue.group(1)) / 100.0, 3), "lanes_per_instruction": float(lanes.group(1)),
            "dram_throughput": round(float(dram.group(1)) / 100.0, 3), "source": "profiles/k_wf_extend_stress.md"}


# The CPU sample both CPU figures time (the reference arm's steps and the line's cpu_baseline): every
# CPU_ROW_STEP-th row of the 1920x1080 frame (rows spread over the whole image, not a central band) for
# CPU_FRAMES frames of 1 spp, i.e. 270 x 1920 x 4 = 2,073,600 path samples of the 132.7 M of one 64-spp step.
CPU_ROW_STEP, CPU_FRAMES = 4, 4


def ncu_warp_inst_per_ray():
    """Warp instructions the extend kernel issues per extension ray, from the committed ncu summary of the
    same walk (smsp__inst_executed.sum over its launches / the rays they walked)."""
    path = os.path.join(ROOT, "profiles", "k_wf_extend_stress.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        m = re.search(r"warp_inst_per_ray\s*=\s*([0-9.]+)", f.read())
    return float(m.group(1)) if m else None


def issue_roofline(rays: float, trace_s: float, sm_mhz, num_sms: int):
    """The walk's issue-side bound: warp instructions issued per second (ncu's instructions per ray x the
    timed rays / the extend kernels' time) against the SMs' issue peak (4 schedulers x 1 warp instruction
    per cycle per SM at the sampled SM clock)."""
    ipr = ncu_warp_inst_per_ray()
    if ipr is None or not sm_mhz or trace_s <= 0:
        return None
    achieved = ipr * rays / trace_s / 1e9
    peak = num_sms * 4 * sm_mhz * 1e6 / 1e9
    return {"bound": "issue", "achieved": round(achieved, 1), "peak": round(peak, 1), "unit": "G warp-inst/s",
            "frac": round(achieved / peak, 4), "warp_inst_per_ray": ipr,
            "source": "profiles/k_wf_extend_stress.md (smsp__inst_executed.sum / rays)"}


def cpu_sample_text(threads: int) -> str:
    rows = len(range(0, HEIGHT, CPU_ROW_STEP))
    return (f"{CPU_FRAMES} frames x every {CPU_ROW_STEP}th row ({rows} rows spread over the image) x {WIDTH} px of "
            f"the same scene/config ({CPU_FRAMES * rows * WIDTH} of the {WIDTH * HEIGHT * SPP} path samples of a "
            f"64-spp step; Mrays/s over the traced segments, which extrapolates to the step at the same rate), "
            f"oracle restatement of the reference cpu path tracer, faithful traversal (no tmax shrink), "
            f"{threads} threads")


def cpu_sample(osc, camera, threads: int, traversal: int):
    """Times the oracle (reference cpu pipeline restated, scene `osc` already built) on the CPU sample;
    returns (Mrays/s, rays, seconds)."""
    import oracle
    from sparkle_gb300 import abi
    cfg = abi.make_config(WIDTH, HEIGHT, spp=1, bounce=BOUNCE, rng=abi.SPK_RNG_XOSHIRO256SS, seed=0)
    r = oracle.OracleRenderer(osc, cfg, camera)
    t0 = time.perf_counter()
    r.render(CPU_FRAMES, traversal=traversal, threads=threads, rows=(0, HEIGHT), row_step=CPU_ROW_STEP)
    dt = time.perf_counter() - t0
    ext, shadow, paths = r.counts()
    return (ext + shadow) / dt / 1e6, ext + shadow, dt


def cpu_rate(osc, camera, threads: int, traversal: int, repeats: int):
    """One untimed sample, then `repeats` timed ones: (Mrays/s over them, rays, seconds)."""
    cpu_sample(osc, camera, threads, traversal)
    rays, secs = 0, 0.0
    for _ in range(repeats):
        _, n, dt = cpu_sample(osc, camera, threads, traversal)
        rays += n
        secs += dt
    return rays / secs / 1e6, rays, secs


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    from sparkle_gb300 import scenes
    threads = os.cpu_count() or 1
    scene, cam_args = scenes.terrain_spheres(0)
    camera = scenes.make_camera(cam_args, WIDTH, HEIGHT)
    osc = oracle.OracleScene(scene)
    for _ in range(args.warmup):
        cpu_sample(osc, camera, threads, oracle.FAITHFUL)
    rays_tot, t_tot = 0, 0.0
    for _ in range(args.steps):
        _, n, dt = cpu_sample(osc, camera, threads, oracle.FAITHFUL)
        rays_tot += n
        t_tot += dt
    value = rays_tot / t_tot / 1e6
    sample = "per step: " + cpu_sample_text(threads)
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * t_tot / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def parse_tune(text: str) -> dict:
    """"knob=value,knob=value" -> spk_tuning fields."""
    out = {}
    for item in filter(None, text.split(",")):
        k, v = item.split("=")
        out[k.strip()] = int(v)
    return out


def run_ours(args):
    rank, world, local_rank = dist_env()
    import numpy as np
    import torch
    from sparkle_gb300 import abi, native, scenes
    torch.cuda.set_device(local_rank)
    dist = init_dist(world, "nccl")
    scene, cam_args = scenes.terrain_spheres(0)
    camera = scenes.make_camera(cam_args, WIDTH, HEIGHT)
    ctx = native.Context(local_rank)
    if args.tune:
        ctx.set_tuning(**parse_tune(args.tune))
    ctx.set_scene(scene)
    # Replica `rank` renders samples rank*64 .. rank*64+63 of the view (same seed, its own sample offset): N
    # replicas draw what one renderer draws in 64*N frames.
    from sparkle_gb300 import replicas
    cfg = abi.make_config(WIDTH, HEIGHT, spp=1, max_spp=4096, bounce=BOUNCE, rng=abi.SPK_RNG_XOSHIRO256SS,
                          seed=0, kernel=args.kernel, sample_offset=replicas.replica_sample_offset(rank, SPP))
    ctx.set_config(cfg)
    ctx.set_camera(camera)

    # Traffic accounting (untimed): count visited wide nodes and tested triangles over one step's frames
    # (a packet walk counts a node or triangle once per packet: one fetch serves its rays).
    ctx.set_instrumentation(True)
    ctx.render(SPP)
    cs = ctx.stats()
    ctx.set_instrumentation(False)
    bytes_per_ray = (NODE_BYTES * cs["node_visits"] + TRI_BYTES * cs["triangle_tests"]) / cs["extension_rays"] \
        + RAY_BYTES + HIT_BYTES

    for _ in range(args.warmup):
        ctx.set_camera(camera)
        ctx.render(SPP)
        ctx.synchronize()

    # Device-timed steps (inputs resident).
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    device_ms = trace_ms = 0.0
    rays = ext_rays = launches = trace_launches = errors = 0
    with ClockSampler(local_rank) as clocks:
        for _ in range(args.steps):
            ctx.set_camera(camera)
            ctx.render(SPP)
            st = ctx.stats()
            device_ms += st["device_ms"]
            trace_ms += st["trace_kernel_ms"]
            rays += st["extension_rays"] + st["shadow_rays"]
            ext_rays += st["extension_rays"]
            launches += st["kernel_launches"]
            trace_launches += st["trace_launches"]
            errors |= st["error_flags"]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    elapsed_s = max_over_ranks(dist, device_ms / 1000.0)
    total_rays = sum_over_ranks(dist, float(rays))
    value = total_rays / elapsed_s / 1e6

    # End to end through the C ABI: camera in, 64 frames, HDR + RGBA16F frame buffers out to pinned memory.
    hdr_host = torch.empty((HEIGHT, WIDTH, 4), dtype=torch.float32, pin_memory=True)
    out_host = torch.empty((HEIGHT, WIDTH, 4), dtype=torch.int16, pin_memory=True)
    d2h = hdr_host.numel() * 4 + out_host.numel() * 2
    h2d = 96  # spk_camera
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e2e_rays = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.set_camera(camera)
        ctx.render(SPP)
        ctx.read_framebuffer_into(hdr_host.data_ptr(), out_host.data_ptr())
        e2e_rays += ctx.stats()["extension_rays"]
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e_value = sum_over_ranks(dist, float(e2e_rays)) / e2e_s / 1e6
    if dist:
        dist.barrier()

    if rank != 0:
        ctx.close()
        return
    peak, peak_kind = measured_peaks()
    rays_per_launch = rays / max(1, trace_launches)
    achieved = bytes_per_ray * rays / (trace_ms / 1000.0) / 1e9
    traffic_per_ray = ncu_traffic_per_ray()
    hdr = np.asarray(hdr_host)
    assert np.all(np.isfinite(hdr)), "non-finite frame buffer"

    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        import oracle
        threads = os.cpu_count() or 1
        osc = oracle.OracleScene(scene)
        v_f, n_f, dt_f = cpu_rate(osc, camera, threads, oracle.FAITHFUL, 4)
        v_p, _, _ = cpu_rate(osc, camera, threads, oracle.PRUNED, 2)
        # the reference's own pool size: min(max_threads = 64, hardware threads) minus the main and render
        # threads it reserves (TaskDispatcher.cpp:18-20, AppFramework.cpp:129-130)
        ref_workers = max(1, min(64, threads) - 2)
        v_w, _, _ = cpu_rate(osc, camera, ref_workers, oracle.FAITHFUL, 2)
        cpu = {"value": round(v_f, 4), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"4 repeats (after one untimed) of the reference arm's step, {cpu_sample_text(threads)}: "
                         f"{n_f} rays in {dt_f:.2f} s; pruned traversal: {v_p:.3f} Mrays/s",
               "pruned_value": round(v_p, 4),
               "reference_workers": {"threads": ref_workers, "value": round(v_w, 4)}}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(elapsed_s * 1000.0 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(), kernel={0: "auto(wavefront)", 1: "megakernel", 2: "wavefront"}[args.kernel],
                       parallelism=f"replicas x{world}" if world > 1 else "single GPU", tuning=ctx.tuning()),
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "kernel": "k_wf_extend (closest-hit walk)" if args.kernel != 1 else "k_render_mega",
                     "algorithmic_bytes_per_ray": round(bytes_per_ray, 1),
                     "nodes_per_ray": round(cs["node_visits"] / cs["extension_rays"], 2),
                     "triangles_per_ray": round(cs["triangle_tests"] / cs["extension_rays"], 2),
                     "rays_per_launch": round(rays_per_launch, 1),
                     "traffic": (round(traffic_per_ray * rays_per_launch) if traffic_per_ray else None),
                     "traffic_unit": "DRAM bytes per launch (ncu per-ray figure x rays per launch)",
                     "ncu_issue": ncu_issue_profile()},
        "trace_kernel_ms_per_step": round(trace_ms / args.steps, 3),
        "device_error_flags": errors,
        "clocks": clocks.summary(),
    }
    line["roofline"]["issue"] = issue_roofline(ext_rays, trace_ms / 1000.0, line["clocks"].get("sm_mhz"),
                                               torch.cuda.get_device_properties(local_rank).multi_processor_count)
    if cpu:
        line["cpu_baseline"] = cpu
    if world == 1 and not args.no_nee:
        line["nee"] = nee_metric(ctx, camera)
    if world == 1 and not args.no_spatial:
        line["spatial"] = spatial_metric(ctx, camera)
    if world == 1 and not args.no_denoise:
        line["denoise"] = denoise_metric(ctx)
    if world == 1 and not args.no_batch:
        line["batch"] = batch_metric(args.batch_autotune)
    if world == 1 and not args.no_scene_update:
        line["scene_update"] = scene_update_metric(scene, camera)
    print(json.dumps(line), flush=True)
    ctx.close()


def nee_metric(ctx, camera, steps: int = 3):
    """The same workload with next-event estimation on (a light and a sky occlusion ray per diffuse vertex):
    Mrays/s over extension + shadow rays by device time, with the occlusion rays in the wavefront's shadow
    stage (persistent any-hit walk with lane refill, the default) and walked inline by the shade kernel."""
    from sparkle_gb300 import abi
    cfg = abi.make_config(WIDTH, HEIGHT, spp=1, max_spp=4096, bounce=BOUNCE, rng=abi.SPK_RNG_XOSHIRO256SS,
                          seed=0, enable_nee=True)
    ctx.set_config(cfg)
    out = {"spp": SPP, "steps": steps}
    for name, stage in (("shadow_stage", 1), ("inline", 0)):
        ctx.set_tuning(shadow_stage=stage)
        ctx.set_camera(camera)
        ctx.render(SPP)  # warm-up (allocations, graph capture)
        ms = ext = shadow = 0.0
        errors = 0
        for _ in range(steps):
            ctx.set_camera(camera)
            ctx.render(SPP)
            st = ctx.stats()
            ms += st["device_ms"]
            ext += st["extension_rays"]
            shadow += st["shadow_rays"]
            errors |= st["error_flags"]
        out[name] = {"mrays_s": round((ext + shadow) / (ms * 1e3), 1), "ms_per_step": round(ms / steps, 2),
                     "extension_rays_per_step": int(ext / steps), "shadow_rays_per_step": int(shadow / steps),
                     "error_flags": errors}
    ctx.set_tuning(shadow_stage=1)
    out["speedup"] = round(out["shadow_stage"]["mrays_s"] / out["inline"]["mrays_s"], 3)
    return out


def spatial_metric(ctx, camera, steps: int = 3):
    """The same workload through the reference's default cpu pipeline, whose DenoisePass spatial fill is on
    (RenderConfig.cpp:38): Mrays/s by device time with every frame of the call in one wavefront (the
    default) and frame by frame (spk_tuning.multi_frame = 0)."""
    from sparkle_gb300 import abi
    cfg = abi.make_config(WIDTH, HEIGHT, spp=1, max_spp=4096, bounce=BOUNCE, rng=abi.SPK_RNG_XOSHIRO256SS,
                          seed=0, spatial_denoise=True)
    ctx.set_config(cfg)
    out = {"spp": SPP, "steps": steps}
    for name, mf in (("multi_frame", 1), ("frame_by_frame", 0)):
        ctx.set_tuning(multi_frame=mf)
        ctx.set_camera(camera)
        ctx.render(SPP)  # warm-up
        ms = rays = 0.0
        errors = 0
        for _ in range(steps):
            ctx.set_camera(camera)
            ctx.render(SPP)
            st = ctx.stats()
            ms += st["device_ms"]
            rays += st["extension_rays"] + st["shadow_rays"]
            errors |= st["error_flags"]
        out[name] = {"mrays_s": round(rays / (ms * 1e3), 1), "ms_per_step": round(ms / steps, 2), "error_flags": errors}
    ctx.set_tuning(multi_frame=1)
    out["speedup"] = round(out["multi_frame"]["mrays_s"] / out["frame_by_frame"]["mrays_s"], 3)
    return out


def scene_update_metric(scene, camera):
    """Scene build and incremental updates on the stress scene (wall time through the C ABI, host arrays in):
    spk_set_scene with the host SAH and with the device LBVH BLAS builder and the Mrays/s each tree traces at
    (16 frames of the bench workload, device time), spk_set_scene reusing a spk_save_bvh blob, spk_update_mesh
    of the 2.1M-triangle terrain (device refit of its BLAS + TLAS rebuild) and spk_set_instance_transforms of
    the 64 spheres (TLAS rebuild)."""
    import numpy as np
    from sparkle_gb300 import abi, native
    c = native.Context(0)
    cfg = abi.make_config(WIDTH, HEIGHT, spp=1, max_spp=4096, bounce=BOUNCE, rng=abi.SPK_RNG_XOSHIRO256SS, seed=0)
    out = {}
    for name, builder in (("host_sah", 0), ("device_lbvh", 1)):
        c.set_tuning(bvh_builder=builder)
        c.set_scene(scene)  # warm (allocations, table set-up)
        t0 = time.perf_counter()
        c.set_scene(scene)
        build_ms = (time.perf_counter() - t0) * 1e3
        c.set_config(cfg)
        c.set_camera(camera)
        c.render(4)
        c.set_camera(camera)
        c.render(16)
        st = c.stats()
        out[name] = {"set_scene_ms": round(build_ms, 1), "bvh_nodes": st["bvh_nodes"],
                     "mrays": round((st["extension_rays"] + st["shadow_rays"]) / (st["device_ms"] * 1e3), 1)}
    c.set_tuning(bvh_builder=0)
    c.set_scene(scene)
    blob = c.save_bvh()
    r = native.Context(0)
    r.set_bvh(blob)
    t0 = time.perf_counter()
    r.set_scene(scene)
    out["set_scene_from_bvh_blob_ms"] = {"value": round((time.perf_counter() - t0) * 1e3, 1),
                                         "blas_reused": r.stats()["blas_reused"], "blob_bytes": len(blob)}
    r.close()
    terrain = scene.meshes[0]
    moved = terrain.positions.copy()
    moved[:, 2] += np.float32(0.5) * np.sin(moved[:, 0] * np.float32(0.3)).astype(np.float32)
    c.update_mesh(0, moved)  # warm
    t0 = time.perf_counter()
    c.update_mesh(0, terrain.positions)
    refit_ms = (time.perf_counter() - t0) * 1e3
    xf = np.stack([i.transform for i in scene.instances[1:]])
    t0 = time.perf_counter()
    c.set_instance_transforms(1, xf)
    c.synchronize()
    xf_ms = (time.perf_counter() - t0) * 1e3
    out["update_mesh_ms"] = {"terrain_triangles": int(terrain.num_faces), "value": round(refit_ms, 2)}
    out["set_instance_transforms_ms"] = {"instances": len(xf), "value": round(xf_ms, 3)}
    c.close()
    return out


def batch_metric(autotune: bool = False):
    """Batched workload: 32 requests over 3 scenes (about 10k, 200k and 2.1M triangles), pixel counts
    log-uniform in [128^2, 1920x1080], spp in {1, 4, 16, 64}, depth 8 with roulette, xoshiro256**. The
    batch (spk_render_batch, one regenerating wavefront) against the same requests rendered one after
    another (spk_render per request on per-scene contexts); both by device time (CUDA events)."""
    from sparkle_gb300 import abi, autotune as at, native, scenes
    sc = scenes.batch_scenes()
    reqs = scenes.batch_requests([c for _, c in sc])
    ctx = native.Context(0)
    ctx.set_scenes([s for s, _ in sc])

    def run_batch(c):
        c.render_batch(reqs, rng=abi.SPK_RNG_XOSHIRO256SS, enable_nee=False)
        return c.stats()

    run_batch(ctx)  # warm-up (allocations)
    best = at.measure(ctx, run_batch, repeats=2)
    out = {"requests": len(reqs), "scene_triangles": [s.num_triangles for s, _ in sc],
           "sample_items": int(sum(r["width"] * r["height"] * r["spp"] for r in reqs)),
           "batched": {"mrays_s": round(best[0] / (best[1] * 1e3), 1), "device_ms": round(best[1], 2),
                       "rays": int(best[0])}}
    if autotune:
        knobs, hist = at.autotune(ctx, run_batch, rebuild=lambda: ctx.set_scenes([s for s, _ in sc]), log=None)
        tuned = at.measure(ctx, run_batch, repeats=2)
        out["autotuned"] = {"knobs": knobs, "mrays_s": round(tuned[0] / (tuned[1] * 1e3), 1),
                            "evaluations": len(hist)}
    ctx.close()
    singles = []
    for s, _ in sc:
        c = native.Context(0)
        c.set_scene(s)
        singles.append(c)
    rays = ms = walk_ms = 0.0
    for r in reqs:
        c = singles[r["scene"]]
        c.set_config(abi.make_config(r["width"], r["height"], spp=1, max_spp=4096, bounce=r["bounce"],
                                     rng=abi.SPK_RNG_XOSHIRO256SS, seed=r["seed"], kernel=abi.SPK_KERNEL_WAVEFRONT))
        c.set_camera(r["camera"])
        c.render(r["spp"])
        st = c.stats()
        rays += st["extension_rays"] + st["shadow_rays"]
        ms += st["device_ms"]
        walk_ms += st["trace_kernel_ms"]
    for c in singles:
        c.close()
    # The walk (extend kernels) takes walk_ms of the requests' device time one by one; batching shares the
    # launches of the rest (shading, generation, resolves, launch gaps), so it can save at most the remainder.
    out["sequential"] = {"mrays_s": round(rays / (ms * 1e3), 1), "device_ms": round(ms, 2), "rays": int(rays),
                         "walk_ms": round(walk_ms, 2), "walk_share": round(walk_ms / ms, 3)}
    out["speedup"] = round(out["batched"]["mrays_s"] / out["sequential"]["mrays_s"], 3)
    return out


def denoise_metric(ctx):
    """Second half of the metric: wall time to relMSE 0.01 (and 0.003) at 1920x1080 on the same scene,
    denoised 1 / 4 / 16 spp (committed U-Net weights, tcgen05 inference, per-tile fallback) vs plain path
    tracing at 1 .. 512 spp, both scored against a 16384-spp plain reference (about 70 s of the run)."""
    from sparkle_gb300 import denoise, eval_denoiser
    import os as _os
    if not _os.path.exists(denoise.WEIGHTS):
        return {"unavailable": "no trained weights at " + _os.path.relpath(denoise.WEIGHTS, ROOT)}
    r = eval_denoiser.run(WIDTH, HEIGHT, ref_spp=16384, plain_max=512, den_spp=(1, 4, 16), ctx=ctx)
    out = {"ref_spp": r["ref_spp"], "nee": True, "threshold": r["threshold"], "tile": r["tile"],
           "plain": [[p["spp"], round(p["relmse"], 6), p["wall_s"]] for p in r["plain"]],
           "denoised": [[d["spp"], round(d["relmse"], 6), d["wall_s"], d["fallback_tiles"]] for d in r["denoised"]]}
    for k in ("time_to_0.01", "time_to_0.003"):
        out[k] = r[k]
    return out


def run_profile_small(args):
    """The bench workload cut to `--frames` frames (default 2; stress scene, 127 MB of nodes + triangles,
    larger than L2, at 1920x1080; `--nee` turns next-event estimation on): the case the ncu captures run on
    (one kernel, a few launches, ~0.3 GB on the device per frame). With F frames a packet of 32 primary rays
    holds 32 / F pixels' samples (one pixel's at F >= 32, as in the 64-frame bench step)."""
    from sparkle_gb300 import abi, native, scenes
    scene, cam_args = scenes.terrain_spheres(0)
    w, h = WIDTH, HEIGHT
    ctx = native.Context(0)
    ctx.set_scene(scene)
    ctx.set_config(abi.make_config(w, h, spp=1, bounce=BOUNCE, rng=abi.SPK_RNG_XOSHIRO256SS, kernel=args.kernel,
                                   enable_nee=args.nee))
    ctx.set_camera(scenes.make_camera(cam_args, w, h))
    ctx.render(args.frames)
    st = ctx.stats()
    assert st["error_flags"] == 0, st
    print(json.dumps({"profile_small": True, "frames": args.frames, "nee": args.nee,
                      "extension_rays": st["extension_rays"],
                      "shadow_rays": st["shadow_rays"], "device_ms": st["device_ms"]}))
    ctx.close()


def run_profile_unet(args):
    """ncu capture case for the U-Net's tcgen05 convolutions: one inference at 1920x1080 (padded to
    1920x1088; about 1.1 GB of activations), ten more of the same input (their median is the warm time),
    and one training step on a 4 x 128 x 128 batch, on seeded random features, with the committed weights
    when present."""
    import numpy as np
    import torch
    from sparkle_gb300 import denoise, native
    dn = native.Denoiser(0, seed=1)
    if os.path.exists(denoise.WEIGHTS):
        denoise.load_weights(dn)
    rng = np.random.default_rng(5)
    feat = torch.from_numpy(rng.uniform(0, 1, (1, HEIGHT, WIDTH, 10)).astype(np.float32)).cuda()
    out = dn.infer(feat)
    ms_infer = dn.last_ms()
    reps = []
    for _ in range(10):  # warm inferences after the first (same input, same output)
        dn.infer(feat)
        reps.append(dn.last_ms())
    fb = torch.from_numpy(rng.uniform(0, 1, (4, 128, 128, 10)).astype(np.float32)).cuda()
    tb = torch.from_numpy(rng.uniform(0, 2, (4, 128, 128, 3)).astype(np.float32)).cuda()
    loss = dn.train_step(fb, tb, 1e-4)
    ms_train = dn.last_ms()
    assert np.isfinite(loss) and torch.isfinite(out).all().item()
    print(json.dumps({"profile_unet": True, "infer_ms": ms_infer, "infer_ms_median_warm": float(np.median(reps)),
                      "train_step_ms": ms_train, "loss": loss}))
    dn.close()


def run_profile_scene(args):
    """ncu capture case for the scene-build kernels: the stress scene's BLASes built on the device (LBVH),
    then the terrain's BLAS refitted once and the 1080p output converted for a screenshot and scored with
    FLIP against itself. `--grid` shrinks the terrain (cells per side) for multi-pass captures."""
    import numpy as np
    from sparkle_gb300 import abi, evaluate, native, scenes
    scene, cam_args = scenes.terrain_spheres(0, grid=args.grid)
    ctx = native.Context(0)
    ctx.set_tuning(bvh_builder=1)
    t0 = time.perf_counter()
    ctx.set_scene(scene)
    build_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    ctx.update_mesh(0, scene.meshes[0].positions)
    refit_ms = (time.perf_counter() - t0) * 1e3
    ctx.set_config(abi.make_config(WIDTH, HEIGHT, spp=1, bounce=BOUNCE, rng=abi.SPK_RNG_XOSHIRO256SS))
    ctx.set_camera(scenes.make_camera(cam_args, WIDTH, HEIGHT))
    ctx.render(1)
    shot = ctx.read_rgba8()
    rgb = shot[..., :3].astype(np.float32) / np.float32(255)
    t0 = time.perf_counter()
    mean = evaluate.flip(rgb, rgb[::-1].copy())
    flip_ms = (time.perf_counter() - t0) * 1e3
    print(json.dumps({"profile_scene": True, "triangles": scene.num_triangles, "set_scene_ms": round(build_ms, 1),
                      "update_mesh_ms": round(refit_ms, 2), "flip_1080p_ms": round(flip_ms, 2),
                      "flip_mean": round(mean, 5)}), flush=True)
    ctx.close()


def run_profile_rays(args):
    """ncu capture case for the ray-set walk: 4M random rays (origins uniform in the scene box, isotropic
    directions) on the stress scene through spk_trace_device, twice."""
    import torch
    from sparkle_gb300 import native, scenes
    scene, _ = scenes.terrain_spheres(0)
    ctx = native.Context(0)
    ctx.set_scene(scene)
    n = 4 * 1024 * 1024
    rays = torch.from_numpy(scenes.random_rays(*scene.world_bounds(), n, seed=21)).cuda()
    hits = torch.empty((n, 5), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        ctx.trace_device(rays.data_ptr(), n, hits.data_ptr())
        st = ctx.stats()
        assert st["error_flags"] == 0, st
    print(json.dumps({"profile_rays": True, "rays": n, "device_ms": st["device_ms"],
                      "mrays_per_s": n / st["device_ms"] / 1e3}))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--kernel", type=int, default=0, help="0 auto, 1 megakernel, 2 wavefront")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-denoise", action="store_true", help="skip the denoised-vs-plain time-to-relMSE leg")
    ap.add_argument("--no-nee", action="store_true", help="skip the next-event-estimation leg")
    ap.add_argument("--no-spatial", action="store_true", help="skip the spatial-fill (default pipeline) leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-requests leg")
    ap.add_argument("--batch-autotune", action="store_true", help="autotune the batched leg's launch knobs")
    ap.add_argument("--no-scene-update", action="store_true", help="skip the scene build / incremental update leg")
    ap.add_argument("--tune", default="", help="spk_tuning knobs, e.g. cuda_graph=0,material_sort=1,bvh_width=4")
    ap.add_argument("--profile-small", action="store_true",
                    help="ncu capture case: the bench workload cut to --frames frames, no timing output")
    ap.add_argument("--nee", action="store_true", help="with --profile-small: next-event estimation on")
    ap.add_argument("--frames", type=int, default=2, help="with --profile-small: frames rendered (1..64)")
    ap.add_argument("--profile-unet", action="store_true",
                    help="ncu capture case: one 1080p U-Net inference and one training step")
    ap.add_argument("--profile-scene", action="store_true",
                    help="ncu capture case: device BLAS build + refit of the stress scene, screenshot + FLIP")
    ap.add_argument("--grid", type=int, default=1024, help="terrain cells per side for --profile-scene")
    ap.add_argument("--profile-rays", action="store_true",
                    help="ncu capture case: 4M random rays through spk_trace_device on the stress scene")
    args = ap.parse_args()
    if args.profile_unet:
        run_profile_unet(args)
    elif args.profile_rays:
        run_profile_rays(args)
    elif args.profile_scene:
        run_profile_scene(args)
    elif args.profile_small:
        run_profile_small(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
