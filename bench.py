"""Traversal benchmark: closest-hit Mrays/s of the GB300 LBVH path.

Workload (the reference's traversal micro-benchmark configuration):
1,048,576 FP32 triangles with seeded centroids uniform in the unit cube and
vertices offset by U[-0.01, 0.01]; 16,777,216 rays with origins uniform in
[-0.2, 1.2]^3 and directions uniform on the sphere, tmax unbounded.  One
step = one closest-hit pass over all rays (Accelerator::intersect
semantics, bit-exact IDs/t/uv).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbrt|reference]

`value`: rays/s with rays resident in HBM (CUDA events on the launching
stream).  `e2e`: the same through the host-buffer C ABI entry
(gbrt_trace_closest_host) with rays in pinned host memory, the upload and
the hit download inside the timed region.  The rays (512 MiB) exceed L2
(129 MB), so no explicit flush is done between steps.
Under torchrun each rank traces its own 16,777,216 rays on its own GPU
(weak scaling, no collective on the data path); value sums over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRI = 1 << 20
N_RAY = 1 << 24
ALG_BYTES_PER_RAY = 32 + 16          # ray record in + hit record out
ALG_BYTES_PER_TRI = 36               # three FP32 vertices, read once per pass
FALLBACK_HBM_GBS = 6800.0
METRIC = "Mrays/s closest-hit (1M-triangle traversal micro-benchmark)"


# ---- the multi-rank (replica) path: each rank traces its own seeded rays
# over the replicated scene; the only exchange is the max of the ranks'
# times (no collective on the data path) ----

def rank_rays(n, rank):
    """The n rays rank `rank` traces (its own seeded batch)."""
    from libyafaray_gb300 import scenes
    return scenes.random_rays(n, seed=2 + 1000 * rank)


def max_over_ranks(x, dist, device=None):
    """x reduced with MAX over the process group (x itself with no group)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """Whole-job throughput in millions of units per second: every rank
    processes units_per_rank in (at most) `seconds`."""
    return units_per_rank * world / seconds / 1e6


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic_per_ray():
    """DRAM bytes per ray of the closest-hit kernel from the committed ncu
    summary (a line 'dram_bytes_per_ray: X'), or None."""
    p = os.path.join(ROOT, "profiles", "traverse_closest_1M.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_ray:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(verts, faces, rays, budget_s=12.0, threads=None):
    """Oracle port (CPU restatement, front-to-back BVH, all host threads) on a
    bounded sample of the same rays.  Returns rays/s and details."""
    from oracle import orc
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    scene = orc.OracleScene(verts, faces)
    build_s = time.perf_counter() - t0
    probe = rays[: 20000 * threads]
    t0 = time.perf_counter(); scene.trace(probe, 0, threads=threads); dt = time.perf_counter() - t0
    n = int(min(len(rays), max(len(probe), len(probe) * budget_s / max(dt, 1e-6))))
    sample = rays[len(probe):len(probe) + n] if len(probe) + n <= len(rays) else rays[:n]
    t0 = time.perf_counter(); scene.trace(sample, 0, threads=threads); dt = time.perf_counter() - t0
    return len(sample) / dt, {"cores": threads, "rays": len(sample), "seconds": dt, "build_s": build_s}


def run_reference(args, rank, world):
    """--impl reference: the CPU restatement of the reference's traversal
    (kind 'port'; the reference's own kd-tree is not compiled on this host)
    timed on all host threads, each step a bounded sample of the workload."""
    if rank != 0:
        return
    from libyafaray_gb300 import scenes
    from oracle import orc
    threads = os.cpu_count() or 1
    verts, faces = scenes.random_triangles(N_TRI, seed=1)
    scene = orc.OracleScene(verts, faces)
    sample = max(20000, 40000 * threads)
    rays = scenes.random_rays(sample * 2, seed=2)
    for _ in range(args.warmup):
        scene.trace(rays[:sample], 0, threads=threads)
    times = []
    for k in range(args.steps):
        chunk = rays[(k % 2) * sample:(k % 2 + 1) * sample]
        t0 = time.perf_counter(); scene.trace(chunk, 0, threads=threads); times.append(time.perf_counter() - t0)
    per_step = float(np.mean(times))
    v = sample / per_step / 1e6
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "config": {"workload": "traversal micro-benchmark: 1,048,576 triangles, incoherent rays, closest hit",
                      "triangles": N_TRI, "rays_per_step": sample, "sample_of": N_RAY},
           "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": threads, "kind": "port",
                            "sample": f"{sample} of the {N_RAY} rays per step"},
           "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def coherent_traversal_section():
    """The micro-benchmark's second mesh: a 2,097,152-triangle unit sphere with
    seeded Perlin displacement (amplitude 0.05) and camera-coherent primary
    rays at 1920x1080 (one per pixel centre), closest hit; a 20,000-ray
    sample is checked against the oracle."""
    import torch
    from libyafaray_gb300 import gbrt, scenes
    from oracle import orc
    v, f = scenes.perlin_sphere()
    rays = scenes.camera_rays(1920, 1080, (0.0, 0.6, 3.2), (0.0, 0.0, 0.0))
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    v_d = torch.from_numpy(v).cuda()
    f_d = torch.from_numpy(f.view(np.int32)).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bvh = gbrt.Bvh.build_device(v_d.data_ptr(), len(v), f_d.data_ptr(), len(f), stream=sp)
    torch.cuda.synchronize()
    build_ms = (time.perf_counter() - t0) * 1e3
    n = len(rays)
    r_d = torch.from_numpy(rays).cuda()
    h_d = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    for _ in range(3):
        bvh.trace_closest_device(r_d.data_ptr(), n, h_d.data_ptr(), stream=sp)
    steps = 50
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(steps):
        bvh.trace_closest_device(r_d.data_ptr(), n, h_d.data_ptr(), stream=sp)
    ev[1].record(stream)
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / steps
    hits = h_d.cpu().numpy()
    prim = hits[:, 0].view(np.int32)
    sel = np.random.default_rng(4).choice(n, 20000, replace=False)
    o = orc.OracleScene(v, f)
    ep, et, _, _ = o.trace(rays[sel], 0)
    agree = float(np.mean((ep == prim[sel]) & (np.where(ep >= 0, et == hits[sel, 1], True))))
    return {"workload": "2,097,152-triangle unit sphere, Perlin displacement amplitude 0.05 (seed 3), 1920x1080 pinhole "
                        "primary rays (pixel centres), closest hit",
            "bvh_build_ms": build_ms, "rays": n, "ms_per_launch": ms, "mrays_s": n / ms / 1e3,
            "hit_fraction": float((prim >= 0).mean()),
            "oracle_sample_agreement": agree, "oracle_sample": 20000}


def next_rows_section():
    """The rows built beyond the core path, each at 512x512 on the Cornell
    box: adaptive anti-aliasing passes, transparent shadows, image textures
    and SPPM; device time per frame beside the reference's CPU time for the
    same configuration."""
    import torch
    from libyafaray_gb300 import gbrt, scenes
    out = {}
    ref_note = "reference: oracle/_ref render_dump, same configuration, 8 x86 cores (16 threads)"

    def frame_ms(r, spp, reps=3):
        film = torch.zeros(512 * 512 * 3, dtype=torch.float32, device="cuda")
        r.render_device(spp, film.data_ptr())
        return min(r.render_device(spp, film.data_ptr(), base_offset=spp * (k + 1), stats=True)["ms"] for k in range(reps))

    # adaptive AA: gauss film, AA_passes 4 from 8 samples, inc 4, threshold 0.02
    sc = scenes.cornell_scene(res=512)
    sc["film"] = {"filter_type": "gauss", "AA_pixelwidth": 1.5, "AA_passes": 4, "AA_minsamples": 8, "AA_inc_samples": 4,
                  "AA_threshold": 0.02}
    r = gbrt.Renderer(sc)
    film = torch.zeros(512 * 512 * 3, dtype=torch.float32, device="cuda")
    w = torch.zeros(512 * 512, dtype=torch.float32, device="cuda")
    r.render_aa_device(film.data_ptr(), w.data_ptr())
    times, res = [], None
    for k in range(3):
        film.zero_(); w.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = r.render_aa_device(film.data_ptr(), w.data_ptr(), base_offset=1000 * (k + 1))
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    out["adaptive_aa_cornell"] = {"workload": "Cornell 512x512, gauss film 1.5, AA_passes 4, AA_minsamples 8, AA_inc_samples 4, "
                                              "AA_threshold 0.02", "ms_per_frame": 1e3 * min(times), "pixels_per_pass": res,
                                  "reference_s": 6.34, "reference_note": ref_note}
    del r
    r = gbrt.Renderer(scenes.cornell_scene(res=512, shiny=("transparent",), glass=True, transparent_shadows=4))
    out["transparent_shadows_cornell"] = {"workload": "Cornell 512x512 16 spp, transparent box + fake_shadows glass balls, "
                                                      "transpShad, shadowDepth 4", "ms_per_frame": frame_ms(r, 16),
                                          "reference_s": 17.2, "reference_note": ref_note}
    del r
    r = gbrt.Renderer(scenes.textured_cornell_scene(res=512))
    out["textured_cornell"] = {"workload": "Cornell 512x512 16 spp, UV-mapped mirrored checker, cube-mapped global texture "
                                                 "through a layer node, checker-clipped global texture",
                               "ms_per_frame": frame_ms(r, 16), "reference_s": 4.39, "reference_note": ref_note}
    del r
    r = gbrt.Renderer(scenes.cornell_sppm_scene(res=512, photons=1_000_000, passes=16))
    r.render(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, st = r.render(1, base_offset=16)
    torch.cuda.synchronize()
    out["sppm_glass_cornell"] = {"workload": "glass Cornell 512x512, SPPM 1,000,000 photon paths x 16 passes",
                                 "ms_per_frame": 1e3 * (time.perf_counter() - t0), "reference_s": 19.8,
                                 "reference_note": ref_note}
    del r
    return out


def render_sections(args):
    """Cornell path tracing throughput and the guided-vs-plain time to
    relMSE 0.01 on the indoor scene (against an FP64-accumulated plain
    render of args.ref_spp samples per pixel)."""
    import torch
    from libyafaray_gb300 import convergence, gbrt, scenes
    out = {}
    # Cornell box, 512x512, 16 spp, path_samples 1, bounces 5, RR from 3
    r = gbrt.Renderer(scenes.cornell_scene(res=512))
    film = torch.zeros(512 * 512 * 3, dtype=torch.float32, device="cuda")
    for _ in range(3):
        r.render_device(16, film.data_ptr())
    best = None
    for k in range(5):
        st = r.render_device(16, film.data_ptr(), base_offset=16 * k, stats=True)
        if best is None or st["ms"] < best["ms"]:
            best = st
    rays = best["extension_rays"] + best["shadow_rays"]
    out["pathtracing_cornell"] = {
        "workload": "Cornell box 34 triangles + emitter, 512x512, 16 spp, pathtracing path_samples 1 bounces 5 rr_min 3",
        "ms_per_frame": best["ms"], "mrays_s": rays / best["ms"] / 1e3,
        "msamples_s": best["camera_samples"] / best["ms"] / 1e3,
        "rays_per_frame": rays, "reference_cpu_note": "reference renders this frame in 3.37 s on 8 x86 threads"}
    del r
    # photonmapping: glass ball (200,000-triangle geodesic sphere) on a plane under
    # a pointlight, 10M diffuse + 10M caustic photon paths, final gather 32, 1024x1024, 1 spp
    sc = scenes.caustic_scene(res=1024, geodesic=100, diffuse_photons=10_000_000, caustic_photons=10_000_000,
                              final_gather=True, fg_samples=32, radius=0.02, search=50)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = gbrt.Renderer(sc)
    build_s = time.perf_counter() - t0
    film = torch.zeros(1024 * 1024 * 3, dtype=torch.float32, device="cuda")
    for k in range(2):
        r.render_device(1, film.data_ptr(), base_offset=k)
    frames = []
    for k in range(5):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = r.render_device(1, film.data_ptr(), base_offset=2 + k, stats=True)
        torch.cuda.synchronize()
        st["wall_ms"] = (time.perf_counter() - t0) * 1e3
        frames.append(st)
    best = min(frames, key=lambda x: x["wall_ms"])
    rays = best["extension_rays"] + best["shadow_rays"]
    out["photon_mapping"] = {
        "workload": "glass geodesic sphere r 0.5 (200,000 triangles, IOR 1.5) on a 4x4 m plane, pointlight power 1000; photonmapping "
                    "10M diffuse + 10M caustic photon paths, radius 0.02, search 50, final gather 32, 1024x1024, 1 spp",
        "scene_bvh_build_and_upload_s": build_s,
        "photon_paths": best["photon_paths"], "photons_stored": best["photons_stored"],
        "radiance_photons": best["radiance_photons"],
        "photon_maps_ms": best["photon_ms"], "render_ms": best["ms"], "frame_wall_ms": best["wall_ms"],
        "photon_paths_per_s": best["photon_paths"] / (best["photon_ms"] / 1e3),
        "render_mrays_s": rays / best["ms"] / 1e3,
        "reference_cpu_note": "reference: 4.32 s per frame (photon maps + render, scene tree already built), "
                              "8 x86 threads, oracle/_ref render_dump, threads_photons auto"}
    del r, film
    # 64 random scenes (spheres / tori, shinydiffuse / glossy / rough glass,
    # 1-4 area lights), 64 spp, bounces 8, rendered as one batch
    t0 = time.perf_counter()
    rs = [gbrt.Renderer(scenes.batch_scene(i)) for i in range(64)]
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    films = [torch.zeros(r.scene["camera"]["resx"] * r.scene["camera"]["resy"] * 3, dtype=torch.float32, device="cuda")
             for r in rs]
    ptrs = [f.data_ptr() for f in films]
    # the autotuner's trial renders (1 spp of the whole batch per candidate)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, tuning = gbrt.render_multi(rs, 1, ptrs)
    torch.cuda.synchronize()
    tune_wall_s = time.perf_counter() - t0
    for f in films:
        f.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, _ = gbrt.render_multi(rs, 64, ptrs, tuning=tuning)
    torch.cuda.synchronize()
    batch_s = time.perf_counter() - t0
    rays = st["extension_rays"] + st["shadow_rays"]
    samples = st["camera_samples"]
    out["batch_64_scenes"] = {
        "workload": "64 seeded scenes (seed 1000+i): round(10^U[3, log10 2e6]) triangles of spheres / tori on a plane, "
                    "50 % shinydiffuse, 30 % glossy, 20 % rough_glass, 1-4 area lights, 256/512/1024 square, 64 spp, bounces 8",
        "triangles": int(sum(len(r.faces) for r in rs)), "camera_samples": samples, "rays": rays,
        "scene_setup_s": setup_s, "batch_wall_s": batch_s, "batch_device_ms": st["ms"], "mrays_s": rays / batch_s / 1e6,
        "msamples_s": samples / batch_s / 1e6,
        "execution": "one wavefront over all 64 scenes (gbrt_pt_render_multi)",
        "autotuned": {k: tuning[k] for k in ("wave_paths", "shade_block", "trace_blocks_per_sm", "streams")},
        "autotune_wall_s": tune_wall_s, "autotune_device_ms": tuning["tune_ms"],
        "reference_cpu_note": "reference, extrapolated: 8 of the 64 scenes (every 8th) at 1 spp took 4.49 s on 8 x86 threads "
                              "(oracle/_ref render_dump, scene trees already built) -> about 2,300 s for 64 scenes x 64 spp"}
    del rs, films
    # indoor scene lit through a door gap: guided vs plain time to relMSE 0.01
    r = gbrt.Renderer(scenes.indoor_scene())
    t0 = time.perf_counter()
    ref = convergence.reference_image(r, spp=args.ref_spp)
    ref_s = time.perf_counter() - t0
    plain = convergence.time_to_relmse(r, ref, target=0.01, spp_pass=16, max_time=90)
    runs = {}
    for frac in (0.25, 0.1):
        guide = r.make_guide()
        runs[frac] = convergence.time_to_relmse(r, ref, target=0.01, spp_pass=4, max_time=90, guide=guide,
                                                alpha=0.6, train_fraction=frac, train_steps=16, batch=65536,
                                                max_vertex=4, expected_time=plain["time_s"], spp_pass_after=16)
        del guide
    guided, short = runs[0.25], runs[0.1]
    ok = plain["reached"]
    out["guided_vs_plain"] = {
        "workload": "indoor room 10x4x6 m, door ajar 0.1 m, outdoor 2x2 m light radiance 200, 200,036 triangles, "
                    "960x540, bounces 12",
        "reference": {"spp": args.ref_spp, "accumulation": "fp64", "seconds": ref_s},
        "target_relmse": 0.01, "relmse": "mean (x - r)^2 / (r^2 + 1e-2) over pixels and RGB",
        "plain": {k: plain[k] for k in ("time_s", "spp", "relmse", "reached")},
        "guided": {k: guided[k] for k in ("time_s", "spp", "relmse", "reached")},
        "guided_settings": {"alpha": 0.6, "train_fraction_of_plain_time": 0.25, "adam_steps_per_wave": 16,
                            "batch": 65536, "spp_per_pass": "4 while training, then 16",
                            "target": "incident radiance x BSDF cosine", "guided_vertices": "first 4 path vertices (camera hit and 3 bounces)"},
        "speedup_wall_time": plain["time_s"] / guided["time_s"] if guided["reached"] and ok else None,
        "speedup_samples": plain["spp"] / guided["spp"] if guided["reached"] and ok else None,
        "guided_training_10pct": {**{k: short[k] for k in ("time_s", "spp", "relmse", "reached")},
                                  "train_fraction_of_plain_time": 0.1,
                                  "speedup_wall_time": plain["time_s"] / short["time_s"] if short["reached"] and ok
                                  else None},
    }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbrt", choices=["gbrt", "reference"])
    ap.add_argument("--rays", type=int, default=N_RAY)
    ap.add_argument("--tris", type=int, default=N_TRI)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-render", action="store_true", help="skip the path-tracing and guided-vs-plain sections")
    ap.add_argument("--ref-spp", type=int, default=16384, help="spp of the FP64 reference of the guided-vs-plain run")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    from libyafaray_gb300 import gbrt, scenes
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    gbrt.load()

    verts, faces = scenes.random_triangles(args.tris, seed=1)
    rays_np = rank_rays(args.rays, rank)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    v_d = torch.from_numpy(verts).cuda()
    f_d = torch.from_numpy(faces.view(np.int32)).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bvh = gbrt.Bvh.build_device(v_d.data_ptr(), len(verts), f_d.data_ptr(), len(faces), stream=sp)
    build_s = time.perf_counter() - t0
    info = bvh.info()
    rays_d = torch.from_numpy(rays_np).cuda()
    hits_d = torch.empty((args.rays, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    for _ in range(args.warmup):
        bvh.trace_closest_device(rays_d.data_ptr(), args.rays, hits_d.data_ptr(), stream=sp)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        ev[0].record(stream)
        for k in range(args.steps):
            bvh.trace_closest_device(rays_d.data_ptr(), args.rays, hits_d.data_ptr(), stream=sp)
            ev[k + 1].record(stream)
        torch.cuda.synchronize()
    launch_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    total_ms = max_over_ranks(total_ms, dist, "cuda")
    per_step_s = total_ms / 1e3 / args.steps
    value = whole_job_rate(args.rays, world, per_step_s)
    hits_np = hits_d[:, 0].cpu().numpy().view(np.int32)
    hit_frac = float((hits_np >= 0).mean())

    # any-hit pass over the same rays (reported beside the headline)
    occ_d = torch.empty(args.rays, dtype=torch.int32, device="cuda")
    bvh.trace_shadow_device(rays_d.data_ptr(), args.rays, occ_d.data_ptr(), stream=sp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(3):
        bvh.trace_shadow_device(rays_d.data_ptr(), args.rays, occ_d.data_ptr(), stream=sp)
    e1.record(stream)
    torch.cuda.synchronize()
    anyhit_mrays = args.rays * 3 / (e0.elapsed_time(e1) / 1e3) / 1e6

    e2e = None
    if not args.no_e2e:
        rays_pin = torch.from_numpy(rays_np).pin_memory()
        hits_pin = torch.empty((args.rays, 4), dtype=torch.float32).pin_memory()
        rp, hp = rays_pin.numpy(), hits_pin.numpy()
        import ctypes
        L = gbrt.load()

        def e2e_step():
            gbrt.check(L.gbrt_trace_closest_host(bvh.handle, ctypes.c_void_p(rp.ctypes.data), args.rays,
                                                 ctypes.c_void_p(hp.ctypes.data)))
        for _ in range(2):
            e2e_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / args.steps
        e2e_s = max_over_ranks(e2e_s, dist, "cuda")
        assert np.array_equal(hp[:, 0].view(np.int32), hits_np), "host path disagrees with device path"
        direct = gbrt.host_path_direct(rp.ctypes.data, args.rays, hp.ctypes.data)
        e2e = {"value": whole_job_rate(args.rays, world, e2e_s), "unit": "Mrays/s",
               "h2d_bytes_per_step": int(rp.nbytes), "d2h_bytes_per_step": int(hp.nbytes),
               "ms_per_step": e2e_s * 1e3,
               "host_path": "direct: the kernel reads the pinned rays and writes the pinned hits in place" if direct
               else "staged: 2,097,152-ray chunks copied through device buffers on two streams",
               "gpu_launches_per_step": 1 if direct else (args.rays + (1 << 21) - 1) >> 21}

    render = None if args.no_render else render_sections(args)
    if render is not None:
        render["traversal_coherent_2M"] = coherent_traversal_section()
        render["beyond_core_path"] = next_rows_section()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peak, peak_kind = peaks()
    avg_launch_s = float(np.mean(launch_ms)) / 1e3
    alg_bytes = args.rays * ALG_BYTES_PER_RAY + args.tris * ALG_BYTES_PER_TRI
    achieved = alg_bytes / avg_launch_s / 1e9
    tpr = ncu_traffic_per_ray()
    cpu = None
    if not args.no_cpu_baseline:
        cv, cinfo = cpu_baseline(verts, faces, rays_np)
        cpu = {"value": cv / 1e6, "unit": "Mrays/s", "cores": cinfo["cores"], "kind": "port",
               "sample": f"{cinfo['rays']} of the {args.rays} rays on the same scene "
                         f"({cinfo['seconds']:.1f} s, CPU restatement with a front-to-back BVH)"}
    out = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": "traversal micro-benchmark: 1,048,576 triangles (centroids U[0,1]^3, vertex offsets "
                               "U[-0.01,0.01]), 16,777,216 incoherent rays (origins U[-0.2,1.2]^3, directions "
                               "uniform on S^2), closest hit",
                   "triangles": args.tris, "rays_per_gpu": args.rays, "l2": "inputs (512 MiB rays) larger than L2; no flush",
                   "max_leaf_size": 4, "sah_intersect_cost": 2.0, "hit_fraction": hit_frac, "bvh_build_s": build_s,
                   "bvh_nodes": info["n_nodes"], "bvh_depth": info["max_depth"], "bvh_sah": info["sah_cost"]},
        "gpu_launches": args.steps,
        "anyhit_mrays_s": anyhit_mrays,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": f"{peak_kind} (HBM copy bandwidth)",
                     "traffic": (tpr * args.rays) if tpr is not None else None,
                     "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_launch_s * 1e3},
        "clocks": clocks.summary(),
    }
    if e2e:
        out["e2e"] = e2e
    if cpu:
        out["cpu_baseline"] = cpu
    if render:
        out.update(render)
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
