"""Benchmark of the NMH traversal hot path on GB300.

Workload (the traversal microbench): 1,000,000 triangles with centroids
U[0,1]^3 and LogNormal(-4, 0.5) edges, 2^24 rays (half coherent pinhole rays
of a 4096x4096 image, even rows; half random origin / uniform direction),
tmax 1e6. One step = one closest-hit pass over all 2^24 device-resident rays;
the metric is Mrays/s closest-hit. Inputs are seeded synthetic data.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {gb300,reference}]

Prints one JSON line. `e2e` measures the same metric through the C ABI's
host-buffer call (aur_trace_closest_host: rays copied in from pinned host
memory and hits copied back inside the timed region). A trace is two
launches: warp packets for the 32-ray chunks of one direction octant (the
pinhole half), then one ray per thread for the other chunks. `roofline`
divides the algorithmic bytes of a trace by its CUDA-event duration, with the
reference algorithm's bytes: 24 B ray in + 16 B hit out + 72 B per node that
the reference's intersect() visits (two triangles of 36 B), the visits
counted by the same traversal without box pruning. This traversal's own
reads per ray (fewer nodes, 128-byte records) are reported beside it, and
the DRAM traffic of one trace (both launches) from the committed ncu summary
when that summary was captured from the current traversal sources. `cpu_baseline` times the
oracle's C++ restatement of the reference traversal on a sample of the same
rays on all host cores. With --gpus N > 1 (under torchrun) every rank runs
an independent replica of the workload.

The same line carries the other workloads (Cornell, MIS, pixel filter, the
64-scene wavefront batch at all 64 spp, the adjoint, the terrain at
1920x1080), each with its correctness checks against the oracle or central
differences; bench.py prints the line and exits with status 1 when any
check fails (the failures are listed under "parity").
"""
import argparse
import hashlib
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

N_TRIS = 1_000_000
N_RAYS = 1 << 24
RAY_IN_BYTES = 28      # origin, direction, tmax (this traversal's own reads)
REF_RAY_IN_BYTES = 24  # origin, direction: the reference algorithm's ray
HIT_OUT_BYTES = 16     # t, u, v, prim
NODE_BYTES = 72        # two triangles, as the reference fetches per visited node
SLAB_BYTES = 16        # first word of a node record: slab lo/hi (+ 8 B of triangle)
TRI_BYTES = 64         # rest of the two triangles, read when the slab is crossed
BOX_BYTES = 48         # children's subtree boxes, read before descending
NMH_LEVEL_BYTES = 32   # NMH build, per triangle per level: 16 B read + 16 B written
METRIC = "Mrays/s closest-hit"
WORKLOAD = ("traversal microbench: 1M triangles (centroid U[0,1]^3, edges LogNormal(-4,0.5)), 2^24 rays "
            "(half coherent pinhole 4096x4096 even rows, half random origin/direction), closest hit")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1 << 22)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-extras", action="store_true", help="headline traversal only")
    ap.add_argument("--terrain", action="store_true",
                    help="only the large terrain workload (plain vs wavefront, full frame)")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="rays per step (profiling cases only)")
    ap.add_argument("--profile", nargs="?", const="trace", default=None,
                    choices=["trace", "render", "mis", "loop", "wavefront", "adjoint", "build", "filter", "emitters",
                             "prep", "stages"],
                    help="small profiling case: trace = one closest-hit and one any-hit launch; render = Cornell "
                         "+ sphere frames; mis = one MIS frame of the emissive Cornell box; loop = the "
                         "reference-structured loop (65,536-ray tiles) on the Cornell + sphere scene; "
                         "wavefront = stepped 8-scene batch; adjoint = one adjoint; "
                         "build = NMH build of the 1M-triangle soup; filter = pixel filter of a 3840x2160 frame; "
                         "emitters = emitter table and MIS light-selection table of a 1M-triangle soup whose "
                         "triangles all emit; prep = object-to-world transform and tangent frames of 4M triangles; "
                         "stages = per-stage time split of the 64-scene batch (samples [0, 2) of 64) and of the "
                         "terrain (sample 0 of 256), the wavefront's kernels launched stepped")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value, world, device="cpu"):
    """Maximum of a per-rank time over all ranks (replicas time the slowest)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, world, seconds):
    """Whole-job throughput of `world` independent replicas timed together."""
    return world * units_per_rank / seconds


def workload(n_rays=N_RAYS):
    from aurora_gb300 import scenes
    V = scenes.random_soup(N_TRIS, seed=0)
    rays = scenes.microbench_rays(n_rays, seed=1)
    return V, rays


def run_profile(args):
    """Small cases for ncu captures (see --profile)."""
    import torch
    from aurora_gb300 import api, build as abuild, scenes, types as T
    abuild.build()
    ctx = api.Context(0)
    if args.profile == "render":
        for sd, p in ((scenes.cornell(), T.render_params(256, 256, 16, 4, mode=T.MODE_PATH)),
                      (scenes.cornell_sphere(seed=0), T.render_params(256, 256, 16, 4, mode=T.MODE_PATH))):
            sc = api.Scene(ctx, sd)
            sc.render(p)
            torch.cuda.synchronize()
        print(json.dumps({"profile_case": "render"}))
        return
    if args.profile == "mis":
        sc = api.Scene(ctx, scenes.cornell_emissive(area_light=True))
        sc.render(T.render_params(256, 256, 16, 3, mode=T.MODE_PATH_MIS))
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "mis"}))
        return
    if args.profile == "loop":
        sd = scenes.cornell_sphere(seed=0)
        sc = api.Scene(ctx, sd)
        W = H = 256
        spp = 4
        p = T.render_params(W, H, spp, 4, mode=T.MODE_PATH)
        rays = torch.zeros((W * H, 9), dtype=torch.float32, device="cuda")
        hits = torch.zeros((W * H, 12), dtype=torch.float32, device="cuda")
        accum = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        api.clear_pixels(ctx, W, H, accum)
        for s_ in range(spp):
            api.generate_rays(ctx, W, H, s_, spp, sd.camera, rays, hits)
            api.raytrace_monte_carlo(ctx, sc, p, s_, 0, W * H, rays, hits)
            api.draw_pixels(ctx, W, H, 1.0 / spp, hits, accum)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "loop"}))
        return
    if args.profile == "wavefront":
        sds = [scenes.sphere_scene(i) for i in range(8)]
        scs = [api.Scene(ctx, sd) for sd in sds]
        prm = [T.render_params(256, 256, 64, 6, mode=T.MODE_PATH, sample_end=2, scene_id=i) for i in range(8)]
        b = api.Batch(ctx, scs, prm, tuning=api.make_tuning(1 << 20, 0, 128, 8))
        st = b.profile([torch.zeros((256, 256, 4), device="cuda") for _ in range(8)])
        print(json.dumps({"profile_case": "wavefront", "stage_ms": st}))
        return
    if args.profile == "adjoint":
        sd = scenes.cornell_sphere(seed=0)
        sc = api.Scene(ctx, sd)
        p = T.render_params(128, 128, 16, 4, mode=T.MODE_PATH)
        img = sc.render(p)
        sc.adjoint(p, img.contiguous())
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "adjoint"}))
        return
    if args.profile == "filter":
        src = torch.rand((2160, 3840, 4), device="cuda")
        out = torch.empty_like(src)
        for _ in range(2):
            api.filter_pixels(ctx, 3840, 2160, src, out)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "filter"}))
        return
    if args.profile == "stages":
        out = {"profile_case": "stages"}
        sds = [scenes.sphere_scene(i) for i in range(64)]
        scs = [api.Scene(ctx, sd) for sd in sds]
        prm = [T.render_params(512, 512, 64, 6, seed=0, mode=T.MODE_PATH, sample_end=2, scene_id=i)
               for i in range(64)]
        b = api.Batch(ctx, scs, prm, tuning=api.make_tuning(1 << 25, 0, 256, 4))
        frames = [torch.zeros((512, 512, 4), device="cuda") for _ in range(64)]
        b.profile(frames)                              # warm-up
        out["spheres_64_scenes_2spp_ms"] = b.profile(frames)
        b.close()
        del scs, frames
        sd = scenes.terrain(res=2048, seed=0)
        sc = api.Scene(ctx, sd)
        p = T.render_params(1920, 1080, 256, 8, seed=0, mode=T.MODE_PATH, sample_end=1)
        b = api.Batch(ctx, [sc], [p], tuning=api.make_tuning(1 << 21, 0, 128, 16))
        f = [torch.zeros((1080, 1920, 4), device="cuda")]
        b.profile(f)
        out["terrain_1spp_ms"] = b.profile(f)
        b.close()
        print(json.dumps(out))
        return
    if args.profile == "emitters":
        V = scenes.random_soup(1_000_000, seed=0)
        n = V.shape[0]
        sh = np.stack([T.lambert((0.5, 0.5, 0.5), emission=(1.0, 0.8, 0.6))])
        sh["emission"] = 1.0
        corners = [np.stack([V[:, k], V[:, 3 + k], V[:, 6 + k]], 1) for k in range(3)]   # p1, p2, p3
        fn = scenes.face_normals(*corners)
        sd = scenes.SceneData("emissive_soup", V, scenes.normals_to_aos(fn, fn, fn), np.ones(n, np.uint16), sh,
                              np.zeros(0, T.light_dtype), scenes.cornell_camera())
        sc = api.Scene(ctx, sd)
        for _ in range(2):
            sc.emitters()
            sc.mis_table()
            sc.set_shaders(sh)                    # a shader change rebuilds the light-selection table
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "emitters", "triangles": n}))
        return
    if args.profile == "prep":
        n = 1 << 22
        src = torch.rand((n * 9,), device="cuda")
        nrm = torch.rand((n * 9,), device="cuda")
        dv, dn = torch.empty_like(src), torch.empty_like(src)
        tb, bt = torch.empty_like(src), torch.empty_like(src)
        xf = np.zeros(4, T.object_transform_dtype)
        for i in range(4):
            xf[i]["offset"], xf[i]["size"] = i * (n // 4), n // 4
            xf[i]["world_matrix"] = np.eye(4) * (1.0 + i)
            xf[i]["normal_matrix"] = np.eye(4) / (1.0 + i)
        for _ in range(2):
            api.transform(ctx, src, nrm, xf, dv, dn)
            api.generate_tb(ctx, dn, tb, bt)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "prep", "triangles": n}))
        return
    if args.profile == "build":
        V, _ = workload(16)
        Vd = torch.from_numpy(V.reshape(-1)).cuda()
        for _ in range(2):
            api.Nmh(ctx, Vd, count=V.shape[0])
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "build"}))
        return
    V, rays = workload(args.rays)
    nmh = api.Nmh(ctx, torch.from_numpy(V.reshape(-1)).cuda(), count=V.shape[0])
    rays_d = api.rays_tensor(rays)
    hits_d = api.trace_closest(ctx, nmh, rays_d)
    torch.cuda.synchronize()
    api.trace_closest(ctx, nmh, rays_d, hits_d)
    occ = api.trace_any(ctx, nmh, rays_d)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "closest + any hit", "rays": int(args.rays), "triangles": N_TRIS,
                      "hit_rate": float((hits_d[:, 3].view(torch.int32) != -1).float().mean().item()),
                      "occluded": float((occ != -1).float().mean().item())}), flush=True)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


TRAVERSAL_SOURCES = ("aurora_gb300/csrc/trace.cu", "aurora_gb300/csrc/aur_traverse.cuh",
                     "aurora_gb300/csrc/aur_math.cuh")
TRAFFIC_PROFILE = "profiles/k_trace_microbench_full.md"


def traversal_source_sha():
    """First 16 hex digits of the SHA-256 of the closest-hit kernel's sources."""
    h = hashlib.sha256()
    for rel in TRAVERSAL_SOURCES:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def load_traffic():
    """(DRAM bytes of one closest-hit trace, both launches; where they come from).

    The committed ncu summary holds 'traffic_bytes_per_trace: N' and
    'source_sha256_16: H', H being traversal_source_sha() of the sources it
    was captured from. The figure is used only when H equals the hash of the
    sources now; otherwise traffic is None and the source says why."""
    p = os.path.join(ROOT, TRAFFIC_PROFILE)
    if not os.path.exists(p):
        return None, "no ncu summary (%s)" % TRAFFIC_PROFILE
    vals = {}
    for line in open(p):
        k, sep, v = line.strip().partition(":")
        if sep and k in ("traffic_bytes_per_trace", "source_sha256_16"):
            vals[k] = v.strip()
    now = traversal_source_sha()
    if vals.get("source_sha256_16") != now:
        return None, ("stale: %s was captured from traversal sources %s, the current ones hash to %s"
                      % (TRAFFIC_PROFILE, vals.get("source_sha256_16", "(unrecorded)"), now))
    try:
        return int(vals["traffic_bytes_per_trace"]), "%s (ncu dram__bytes_read.sum + dram__bytes_write.sum of " \
            "both launches of a trace, traversal sources %s)" % (TRAFFIC_PROFILE, now)
    except (KeyError, ValueError):
        return None, "no traffic_bytes_per_trace line in %s" % TRAFFIC_PROFILE


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
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
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(verts, perm, rays, sample, seed=7):
    """The oracle's restatement of intersect() on a random sample of the rays,
    all host threads."""
    import oracle
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(rays.shape[0], size=min(sample, rays.shape[0]), replace=False))
    sub = np.ascontiguousarray(rays[idx])
    nth = os.cpu_count() or 1
    oracle.trace_closest(verts, perm, sub[:1024], nthreads=nth)       # warm the library
    t0 = time.perf_counter()
    oracle.trace_closest(verts, perm, sub, nthreads=nth)
    dt = time.perf_counter() - t0
    return {"value": sub.shape[0] / dt / 1e6, "unit": "Mrays/s", "cores": nth, "kind": "port",
            "sample": "%d rays drawn uniformly from the 2^24 (seed %d), closest hit, oracle C++ restatement of "
                      "intersect(), %d host threads, %.1f s" % (sub.shape[0], seed, nth, dt)}


class Checks:
    """Correctness checks of the workloads: every check is recorded, and a
    failed one makes bench.py exit with status 1 after printing its line."""

    def __init__(self):
        self.names, self.failures = [], []

    def add(self, name, ok):
        self.names.append(name)
        if not bool(ok):
            self.failures.append(name)
        return bool(ok)

    def summary(self):
        return {"checks": len(self.names), "passed": len(self.names) - len(self.failures),
                "failures": self.failures}


def cpu_build_baseline(V, gpu_perm):
    """The oracle's NMH build (C++ restatement of rebuilder.cu's algorithm,
    one host thread) of the whole soup, timed; its permutation must equal the
    GPU's."""
    import oracle
    t0 = time.perf_counter()
    perm, levels = oracle.nmh_build(V)
    dt = time.perf_counter() - t0
    return {"ms": dt * 1e3, "mtris_per_s": V.shape[0] / dt / 1e6, "cores": 1, "kind": "port",
            "sample": "the whole %d-triangle soup, %d levels, oracle C++ restatement, 1 host thread" % (V.shape[0], levels),
            "equal": bool(np.array_equal(perm, gpu_perm))}


def _render_rate(n_samples, ms):
    return n_samples / (ms * 1e-3)


def _rmse(a, ref):
    return float(((a[..., :3].double() - ref[..., :3].double()) ** 2).mean().sqrt())


def _rmse_16384(ctx, sc, p, tuning):
    """RMSE at the workload's spp of a small view of the same camera, plain
    renderer and wavefront, against a 16384-spp render of that view (seed 1)."""
    from aurora_gb300 import api, types as T
    pr = np.array(p, copy=True)
    pr["spp"], pr["seed"] = 16384, 1
    rb = api.Batch(ctx, [sc], [pr], tuning=tuning)
    t0 = time.perf_counter()
    ref = rb.render()[0]
    rb.status()
    ref_s = time.perf_counter() - t0
    rb.close()
    plain = sc.render(p)
    wb = api.Batch(ctx, [sc], [p], tuning=tuning)
    wf = wb.render()[0]
    wb.status()
    wb.close()
    return {"view": "%dx%d" % (int(p["width"]), int(p["height"])), "spp": int(p["spp"]),
            "reference": "16384 spp, seed 1 (%.1f s)" % ref_s, "plain": _rmse(plain, ref), "wavefront": _rmse(wf, ref)}


def bench_batched(ctx, checks, n_scenes=64, size=512, spp=64, depth=6, loop_samples=8, rmse_scene=0,
                  ref_spp=4096):
    """Batched workload: 64 sphere scenes (1k-500k triangles each), 512x512,
    64 spp, depth 6, path mode, all 64 samples of every scene timed with CUDA
    events in two forms whose frames must be identical:
      * this library's fused plain renderer (one aur_render per scene, all
        samples of a scene in one launch), the plain GPU path;
      * the wavefront batch (one graph launch for all scenes).
    `speedup` is wavefront over fused plain. Beside them, the plain path as
    the reference structures it (render/monteCarloRaytracer.cpp:81-120: per
    scene and sample, generate rays, the megakernel over 65,536-ray tiles,
    draw pixels) on samples [0, loop_samples), with its frames checked
    against the fused renderer's at that sample count. RMSE: the 64-spp
    frames of scene `rmse_scene` from both forms against a `ref_spp`-spp
    render of that scene (seed 1)."""
    import torch
    from aurora_gb300 import api, scenes, types as T
    sds = [scenes.sphere_scene(i) for i in range(n_scenes)]
    scs = [api.Scene(ctx, sd) for sd in sds]
    prm = [T.render_params(size, size, spp, depth, seed=0, mode=T.MODE_PATH, scene_id=i) for i in range(n_scenes)]
    n_samples = n_scenes * size * size * spp
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    frames = [torch.zeros((size, size, 4), dtype=torch.float32, device="cuda") for _ in range(n_scenes)]

    scs[0].render(T.render_params(size, size, spp, depth, seed=0, mode=T.MODE_PATH, sample_end=1))   # warm-up
    torch.cuda.synchronize()
    e0.record(stream)
    for sc, p, f in zip(scs, prm, frames):
        sc.render(p, accum=f)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_img = frames

    # the reference-structured loop on samples [0, loop_samples)
    tile = 65536
    rays_b = torch.empty((size * size * 9,), dtype=torch.float32, device="cuda")     # aur_path_ray, 36 B
    hits_b = torch.empty((size * size * 12,), dtype=torch.float32, device="cuda")    # aur_hitpoint, 48 B
    loop_frames = [torch.zeros((size, size, 4), dtype=torch.float32, device="cuda") for _ in range(n_scenes)]
    torch.cuda.synchronize()
    e0.record(stream)
    for sc, p, f in zip(scs, prm, loop_frames):
        for smp in range(loop_samples):
            api.generate_rays(ctx, size, size, smp, spp, sc.data.camera, rays_b, hits_b)
            for off in range(0, size * size, tile):
                api.raytrace_monte_carlo(ctx, sc, p, smp, off, min(tile, size * size - off), rays_b, hits_b)
            api.draw_pixels(ctx, size, size, 1.0 / spp, hits_b, f)
    e1.record(stream)
    torch.cuda.synchronize()
    loop_ms = e0.elapsed_time(e1)
    del rays_b, hits_b
    loop_same = True
    for i in (0, n_scenes - 1):
        part = scs[i].render(T.render_params(size, size, spp, depth, seed=0, mode=T.MODE_PATH, scene_id=i,
                                             sample_end=loop_samples))
        loop_same = loop_same and bool(torch.equal(part, loop_frames[i]))
    del loop_frames
    checks.add("batch: the reference-structured loop's frames equal the fused renderer's", loop_same)

    t0 = time.perf_counter()
    tuning, tune_ms = api.autotune(ctx, scs, prm)
    tune_s = time.perf_counter() - t0
    batch = api.Batch(ctx, scs, prm, tuning=tuning)
    wf = [torch.zeros_like(f) for f in frames]
    batch.render(wf)                                     # warm-up (graph upload)
    batch.status()
    for f in wf:
        f.zero_()
    e0.record(stream)
    batch.render(wf)
    e1.record(stream)
    iters = batch.status()
    wf_ms = e0.elapsed_time(e1)
    ext, shadow, _ = batch.counters()
    batch.close()
    same = all(torch.equal(a, b) for a, b in zip(wf, plain_img))
    checks.add("batch: wavefront frames equal the fused renderer's (64 scenes, 64 spp)", same)

    # RMSE against a high-spp frame of one scene
    rp = T.render_params(size, size, ref_spp, depth, seed=1, mode=T.MODE_PATH, scene_id=rmse_scene)
    rb = api.Batch(ctx, [scs[rmse_scene]], [rp], tuning=tuning)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = rb.render()[0]
    rb.status()
    ref_s = time.perf_counter() - t0
    rb.close()
    rmse_plain, rmse_wf = _rmse(plain_img[rmse_scene], ref), _rmse(wf[rmse_scene], ref)
    checks.add("batch: equal RMSE of plain and wavefront", rmse_plain == rmse_wf)
    small = _rmse_16384(ctx, scs[rmse_scene], T.render_params(128, 128, spp, depth, seed=0, mode=T.MODE_PATH,
                                                              scene_id=rmse_scene), tuning)
    checks.add("batch: equal RMSE against the 16384-spp view", small["plain"] == small["wavefront"])
    tris = [sd.count for sd in sds]
    return {"workload": "%d sphere scenes (%d-%d triangles, %d total), %dx%d, %d spp, depth %d, path mode; all "
                        "samples timed" % (n_scenes, min(tris), max(tris), sum(tris), size, size, spp, depth),
            "plain_samples_per_s": _render_rate(n_samples, plain_ms), "plain_ms": plain_ms,
            "wavefront_samples_per_s": _render_rate(n_samples, wf_ms), "wavefront_ms": wf_ms,
            "speedup": plain_ms / wf_ms,
            "target": "wavefront >= 5x the plain GPU path (fused renderer)",
            "target_met": plain_ms / wf_ms >= 5.0,
            "plain_reference_loop": {"samples": "[0, %d) of %d" % (loop_samples, spp),
                                     "samples_per_s": _render_rate(n_scenes * size * size * loop_samples, loop_ms),
                                     "ms": loop_ms, "launches": n_scenes * loop_samples *
                                     (2 + (size * size + tile - 1) // tile)},
            "speedup_vs_reference_loop": _render_rate(n_samples, wf_ms) /
                                         _render_rate(n_scenes * size * size * loop_samples, loop_ms),
            "frames_identical": bool(same),
            "rmse": {"scene": rmse_scene, "reference": "%dx%d at %d spp (seed 1, wavefront, %.1f s)"
                     % (size, size, ref_spp, ref_s), "spp": spp, "plain": rmse_plain, "wavefront": rmse_wf},
            "rmse_16384": small,
            "wavefront_graph_launches": 1, "wavefront_iterations": iters,
            "wavefront_rays": {"closest": ext, "shadow": shadow,
                               "mrays_per_s": (ext + shadow) / (wf_ms * 1e-3) / 1e6},
            "tuning": {k: int(tuning[k]) for k in tuning.dtype.names}, "autotune_s": tune_s}


def bench_cornell(ctx, checks, cpu=True, textured=False):
    """Cornell workload: 34 triangles, 256x256, 16 spp, depth 4, seed 0, path
    mode: plain GPU render vs the oracle on all host cores. textured: the
    floor, back wall and short box use textured shaders (two RGBA8 images,
    bilinear wrapping fetch)."""
    import torch
    from aurora_gb300 import api, scenes, types as T
    sd = scenes.cornell_textured() if textured else scenes.cornell()
    sc = api.Scene(ctx, sd)
    if textured:
        sc.set_textures(sd.texcoords, sd.textures)
    p = T.render_params(256, 256, 16, 4, seed=0, mode=T.MODE_PATH)
    sc.render(p)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    e0.record(stream)
    for _ in range(reps):
        img = sc.render(p)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    out = {"workload": "Cornell box (34 triangles%s), 256x256, 16 spp, depth 4, path mode"
                       % (", 3 textured shaders" if textured else ""),
           "gpu_samples_per_s": 256 * 256 * 16 / (ms * 1e-3), "gpu_ms": ms}
    if cpu:
        import oracle
        ns = oracle.NmhScene(sd)
        t0 = time.perf_counter()
        if textured:
            ref, _ = oracle.render(ns, p, nthreads=os.cpu_count() or 1)
        else:
            ref, fetches, shaded = oracle.render_counted(ns, p, nthreads=os.cpu_count() or 1)
        dt = time.perf_counter() - t0
        out["cpu_samples_per_s"] = 256 * 256 * 16 / dt
        out["cpu_cores"] = os.cpu_count()
        g = img.cpu().numpy()
        out["matches_oracle"] = checks.add("Cornell%s frame within 1e-4 of the oracle" % (" textured" if textured else ""),
                                           np.all(np.abs(g - ref) <= 1e-4 * np.abs(ref) + 1e-7))
        out["bit_exact"] = checks.add("Cornell%s frame bit-exact with the oracle" % (" textured" if textured else ""),
                                      np.array_equal(g, ref))
        if not textured:
            # path-sampling roofline: per sample, 72 B per node fetch of the
            # reference algorithm (closest and any hit), 36 B of normals and an
            # 80-byte shader per shading point, 16 B of accumulation (counted
            # by the oracle on the same render); the 34-triangle scene itself
            # is 2 KB, so these bytes come from L1 and L2
            n = 256 * 256 * 16
            per_sample = (72.0 * fetches + (36.0 + 80.0) * shaded + 16.0 * n) / n
            peak, _ = load_peaks()
            gbs = per_sample * out["gpu_samples_per_s"] / 1e9
            out["roofline"] = {"algorithmic_bytes_per_sample": per_sample,
                               "node_fetches_per_sample": fetches / n, "shading_points_per_sample": shaded / n,
                               "achieved_GBps": gbs, "frac_of_hbm_peak": gbs / peak}
    return out


def bench_mis(ctx, size=256, spp=16, depth=3, ref_renders=256):
    """AUR_MODE_PATH_MIS on the Cornell box lit by emissive geometry (a
    ceiling lamp, a glowing block, a small wall emitter): samples/s of MIS at
    depth d and of path mode at depth d + 1 (the same set of paths), the RMSE
    of one spp-sample render of each against the mean of `ref_renders`
    independent MIS renders of the same sub-pixel grid, and the efficiency
    gain (rmse_path^2 * t_path) / (rmse_mis^2 * t_mis): how much less time
    MIS needs for the same error."""
    import torch
    from aurora_gb300 import api, scenes, types as T
    sc = api.Scene(ctx, scenes.cornell_emissive())
    acc = None
    for s in range(ref_renders):
        acc = sc.render(T.render_params(size, size, spp, depth, seed=1000 + s, mode=T.MODE_PATH_MIS), accum=acc)
    ref = (acc / ref_renders).cpu().numpy()[..., :3].astype(np.float64)
    stream = torch.cuda.current_stream()
    out = {"workload": "Cornell box lit by 15 emissive triangles, %dx%d, %d spp; MIS at depth %d vs path mode "
                       "at depth %d" % (size, size, spp, depth, depth + 1)}
    for name, mode, d in (("mis", T.MODE_PATH_MIS, depth), ("path", T.MODE_PATH, depth + 1)):
        p = T.render_params(size, size, spp, d, seed=0, mode=mode)
        sc.render(p)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5
        e0.record(stream)
        for _ in range(reps):
            img = sc.render(p)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        err = img.cpu().numpy()[..., :3].astype(np.float64) - ref
        out[name + "_ms"] = ms
        out[name + "_samples_per_s"] = size * size * spp / (ms * 1e-3)
        out[name + "_rmse"] = float(np.sqrt(np.mean(err * err)))
    out["efficiency_vs_path"] = (out["path_rmse"] ** 2 * out["path_ms"]) / (out["mis_rmse"] ** 2 * out["mis_ms"])
    return out


def bench_filter(ctx, width=3840, height=2160, reps=20):
    """aur_filter_pixels on a 3840x2160 float4 frame (133 MB in, 133 MB out,
    both larger than L2): algorithmic bytes 16 B read + 16 B written per pixel
    against the measured HBM peak."""
    import torch
    from aurora_gb300 import api
    src = torch.rand((height, width, 4), device="cuda")
    out = torch.empty_like(src)
    api.filter_pixels(ctx, width, height, src, out)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        api.filter_pixels(ctx, width, height, src, out)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    peak, _ = load_peaks()
    gbs = width * height * 32 / (ms * 1e-3) / 1e9
    return {"workload": "3x3 binomial filter, %dx%d float4" % (width, height), "ms": ms, "GBps": gbs,
            "frac_of_hbm_peak": gbs / peak}


def bench_adjoint(ctx, checks, size=256, spp=64, depth=4):
    """Differentiable workload: Cornell box + 4096-triangle sphere, one shader
    per triangle (albedo U[0.2, 0.8]), 256x256, 64 spp, depth 4; L2 loss
    against the frame rendered at albedo + N(0, 0.05). grad/fwd = adjoint
    time / forward render time; two gradients are checked against central
    differences (h = 1e-3, common random numbers)."""
    import torch
    from aurora_gb300 import api, scenes, types as T
    sd = scenes.cornell_sphere(seed=0)
    sc = api.Scene(ctx, sd)
    p = T.render_params(size, size, spp, depth, seed=0, mode=T.MODE_PATH)
    rng = np.random.default_rng(0)
    tsh = sd.shaders.copy()
    tsh["diffuse_color"] = np.clip(tsh["diffuse_color"] + rng.normal(0, 0.05, (sd.count, 3)), 0, 1)
    sc.set_shaders(tsh)
    target = sc.render(p)
    sc.set_shaders(sd.shaders)
    stream = torch.cuda.current_stream()
    img = sc.render(p)
    torch.cuda.synchronize()
    e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
    e0.record(stream)
    img = sc.render(p)
    e1.record(stream)
    d_image = (2.0 * (img - target)).contiguous()
    d_image[..., 3] = 0
    gs, gl = sc.adjoint(p, d_image)
    torch.cuda.synchronize()
    gs.zero_(); gl.zero_()
    e2.record(stream)
    sc.adjoint(p, d_image, gs, gl)
    e3.record(stream)
    torch.cuda.synchronize()
    fwd_ms, adj_ms = e0.elapsed_time(e1), e2.elapsed_time(e3)
    g = gs.cpu().numpy()

    def loss():
        d = sc.render(p).double() - target.double()
        return float((d[..., :3] ** 2).sum())

    fd_checks = []
    for k in list(np.argsort(-np.abs(g).ravel())[:2]):
        i, c = int(k // 3), int(k % 3)
        vals = []
        for sgn in (1, -1):
            sh = sd.shaders.copy()
            sh["diffuse_color"][i, c] += sgn * 1e-3
            sc.set_shaders(sh)
            vals.append(loss())
        sc.set_shaders(sd.shaders)
        fd = (vals[0] - vals[1]) / 2e-3
        fd_checks.append({"shader": i, "channel": c, "adjoint": float(g[i, c]), "fd": fd,
                          "rel_err": abs(float(g[i, c]) - fd) / abs(fd)})
        checks.add("adjoint d/d(albedo[%d][%d]) within 1e-3 of central differences" % (i, c),
                   abs(float(g[i, c]) - fd) <= 1e-3 * abs(fd) + 1e-6)
    return {"workload": "Cornell box + 4096-triangle sphere (4130 per-triangle shaders), %dx%d, %d spp, depth %d, "
                        "path mode, L2 loss" % (size, size, spp, depth),
            "forward_ms": fwd_ms, "adjoint_ms": adj_ms, "grad_over_fwd": adj_ms / fwd_ms, "fd_checks": fd_checks}


def bench_terrain(ctx, checks, res=2048, samples=16, ref_seed=1, crop=(64, 36), cpu=True):
    """Large workload: 2048x2048-vertex fBm heightfield (8,380,418 triangles),
    16 area lights, 1920x1080, 256 spp, depth 8, path mode, full frame.
      * NMH build of the terrain (warm, CUDA events);
      * plain GPU path (fused renderer) and wavefront on samples [0, `samples`)
        of the 256, timed; the frames must be identical;
      * the wavefront renders all 256 samples of the frame with seed
        `ref_seed` (independent of the timed seed 0), timed: the workload at
        its full sample count, and the reference image for the RMSE of the
        timed frames;
      * the reference-structured loop (65,536-ray megakernel tiles) on sample 0;
      * CPU baseline: the oracle renders a `crop` of the same camera at 1 spp
        on all host cores (a bounded sample of the workload), and the GPU's
        render of that crop must equal it bit for bit."""
    import torch
    from aurora_gb300 import api, scenes, types as T
    t0 = time.perf_counter()
    sd = scenes.terrain(res=res, seed=0)
    gen_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sc = api.Scene(ctx, sd)
    torch.cuda.synchronize()
    scene_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    Vd = torch.from_numpy(sd.vertices.reshape(-1)).cuda()
    build = []
    for _ in range(3):                                 # the third build replays the recorded graph
        e0.record(stream)
        api.Nmh(ctx, Vd, count=sd.count).close()
        e1.record(stream)
        torch.cuda.synchronize()
        build.append(e0.elapsed_time(e1))
    del Vd
    W, H, spp, depth = 1920, 1080, 256, 8
    p = T.render_params(W, H, spp, depth, seed=0, mode=T.MODE_PATH, sample_end=samples)
    sc.render(T.render_params(W, H, spp, depth, seed=0, mode=T.MODE_PATH, sample_end=1))     # warm-up
    torch.cuda.synchronize()
    e0.record(stream)
    plain = sc.render(p)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    # the plain path as the reference structures it, sample 0: generate,
    # 65,536-ray megakernel tiles, draw (render/monteCarloRaytracer.cpp:81-120)
    tile = 65536
    rays_b = torch.empty((W * H * 9,), dtype=torch.float32, device="cuda")
    hits_b = torch.empty((W * H * 12,), dtype=torch.float32, device="cuda")
    loop_img = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    e0.record(stream)
    api.generate_rays(ctx, W, H, 0, spp, sd.camera, rays_b, hits_b)
    for off in range(0, W * H, tile):
        api.raytrace_monte_carlo(ctx, sc, p, 0, off, min(tile, W * H - off), rays_b, hits_b)
    api.draw_pixels(ctx, W, H, 1.0 / spp, hits_b, loop_img)
    e1.record(stream)
    torch.cuda.synchronize()
    loop_ms = e0.elapsed_time(e1)
    p1 = T.render_params(W, H, spp, depth, seed=0, mode=T.MODE_PATH, sample_end=1)
    checks.add("terrain: the reference-structured loop's frame equals the fused renderer's",
               torch.equal(loop_img, sc.render(p1)))
    del rays_b, hits_b, loop_img
    t0 = time.perf_counter()
    tuning, _ = api.autotune(ctx, [sc], [p])
    tune_s = time.perf_counter() - t0
    batch = api.Batch(ctx, [sc], [p], tuning=tuning)
    batch.render()
    batch.status()
    e0.record(stream)
    wf = batch.render()[0]
    e1.record(stream)
    batch.status()
    wf_ms = e0.elapsed_time(e1)
    ext, shadow, iters = batch.counters()
    batch.close()
    same = checks.add("terrain: wavefront frame equals the fused renderer's (1920x1080, %d spp)" % samples,
                      torch.equal(wf, plain))
    # all 256 samples, seed ref_seed: the full workload, and the RMSE reference
    pf = T.render_params(W, H, spp, depth, seed=ref_seed, mode=T.MODE_PATH)
    fb = api.Batch(ctx, [sc], [pf], tuning=tuning)
    e0.record(stream)
    ref = fb.render()[0]
    e1.record(stream)
    fb.status()
    full_ms = e0.elapsed_time(e1)
    full_rays = fb.counters()
    fb.close()
    rmse_plain, rmse_wf = _rmse(plain, ref), _rmse(wf, ref)
    checks.add("terrain: equal RMSE of plain and wavefront", rmse_plain == rmse_wf)
    small = _rmse_16384(ctx, sc, T.render_params(64, 36, spp, depth, seed=0, mode=T.MODE_PATH), tuning)
    checks.add("terrain: equal RMSE against the 16384-spp view", small["plain"] == small["wavefront"])
    n_samples = W * H * samples
    out = {"workload": "fBm terrain %dx%d vertices (%d triangles), 16 area lights, %dx%d, %d spp, depth %d, path mode, "
                       "full frame; plain and wavefront timed on samples [0, %d), the wavefront also on all %d"
                       % (res, res, sd.count, W, H, spp, depth, samples, spp),
           "generate_s": gen_s, "scene_upload_and_build_s": scene_s, "nmh_build_ms": build[-1],
           "nmh_build_mtris_per_s": sd.count / (build[-1] * 1e-3) / 1e6,
           "plain_samples_per_s": _render_rate(n_samples, plain_ms), "plain_ms": plain_ms,
           "wavefront_samples_per_s": _render_rate(n_samples, wf_ms), "wavefront_ms": wf_ms,
           "speedup": plain_ms / wf_ms, "target": "wavefront >= 5x the plain GPU path (fused renderer)",
           "target_met": plain_ms / wf_ms >= 5.0,
           "wavefront_full_spp": {"spp": spp, "ms": full_ms, "samples_per_s": _render_rate(W * H * spp, full_ms),
                                  "closest_rays": full_rays[0], "shadow_rays": full_rays[1]},
           "plain_reference_loop": {"samples": "[0, 1) of %d" % spp, "ms": loop_ms,
                                    "samples_per_s": _render_rate(W * H, loop_ms)},
           "speedup_vs_reference_loop": _render_rate(n_samples, wf_ms) / _render_rate(W * H, loop_ms),
           "frames_identical": same,
           "tuning": {k: int(tuning[k]) for k in tuning.dtype.names}, "autotune_s": tune_s,
           "wavefront_rays": {"closest": ext, "shadow": shadow, "iterations": iters,
                              "mrays_per_s": (ext + shadow) / (wf_ms * 1e-3) / 1e6},
           "rmse": {"reference": "the full %dx%d frame at %d spp, seed %d (wavefront)" % (W, H, spp, ref_seed),
                    "spp": samples, "plain": rmse_plain, "wavefront": rmse_wf},
           "rmse_16384": small}
    if cpu:
        import oracle
        sw, sh = crop
        cam = sd.camera
        ns = oracle.NmhScene(sd, perm=sc.nmh.export(with_vertices=False)[0])
        pc = T.render_params(sw, sh, 1, depth, seed=0, mode=T.MODE_PATH)
        nth = os.cpu_count() or 1
        t0 = time.perf_counter()
        cimg, _ = oracle.render(ns, pc, camera=cam, nthreads=nth)
        cpu_s = time.perf_counter() - t0
        exact = checks.add("terrain: GPU crop bit-exact with the oracle",
                           np.array_equal(sc.render(pc, camera=cam).cpu().numpy(), cimg))
        out["cpu_baseline"] = {"samples_per_s": sw * sh / cpu_s, "cores": nth, "kind": "port",
                               "sample": "%dx%d frame of the same camera, 1 spp, depth 8, oracle C++ restatement "
                                         "(the GPU's NMH permutation, equal to the oracle's build)" % (sw, sh),
                               "gpu_bit_exact": exact}
    return out


def run_reference(args):
    """--impl reference: the reference traversal restated in C++ (the oracle;
    the reference's own sources do not travel to this machine) on the host
    cores, on bounded samples of the same workload."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    import oracle
    from aurora_gb300 import scenes  # noqa: F401
    V, rays = workload()
    perm, _ = oracle.nmh_build(V)
    verts = oracle.gather9(V, perm)
    nth = os.cpu_count() or 1
    rng = np.random.default_rng(11)
    per_step = 1 << 17
    times = []
    for s in range(args.warmup + args.steps):
        idx = rng.choice(rays.shape[0], size=per_step, replace=False)
        sub = np.ascontiguousarray(rays[np.sort(idx)])
        t0 = time.perf_counter()
        oracle.trace_closest(verts, perm, sub, nthreads=nth)
        if s >= args.warmup:
            times.append(time.perf_counter() - t0)
    T = sum(times)
    value = args.steps * per_step / T / 1e6
    out = {"metric": METRIC, "value": value, "unit": "Mrays/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * T / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded)", "config": {"workload": WORKLOAD, "triangles": N_TRIS, "rays": N_RAYS,
                                                    "step_sample_rays": per_step},
           "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": nth, "kind": "port",
                            "sample": "%d random rays of the 2^24 per step, oracle C++ restatement of intersect() "
                                      "(the reference's traversal), %d host threads" % (per_step, nth)},
           "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args)
    if args.terrain:
        from aurora_gb300 import api, build as abuild
        abuild.build()
        checks = Checks()
        print(json.dumps({"terrain": bench_terrain(api.Context(0), checks), "parity": checks.summary()}), flush=True)
        sys.exit(1 if checks.failures else 0)
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from aurora_gb300 import api, build as abuild
    abuild.build()
    ctx = api.Context(local)
    V, rays = workload()
    Vd = torch.from_numpy(V.reshape(-1)).cuda()
    for _ in range(2):                              # warm-up: the second build of a size records its graph
        api.Nmh(ctx, Vd, count=V.shape[0]).close()
    builds = []
    for _ in range(5):                              # host wall time of the whole call, median of 5
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nmh = api.Nmh(ctx, Vd, count=V.shape[0])
        torch.cuda.synchronize()
        builds.append(1e3 * (time.perf_counter() - t0))
        if len(builds) < 5:
            nmh.close()
    build_ms = float(np.median(builds))
    rays_d = api.rays_tensor(rays)
    hits_d = torch.empty((N_RAYS, 4), dtype=torch.float32, device="cuda")
    occ_d = torch.empty((N_RAYS,), dtype=torch.int32, device="cuda")
    visits_closest, visits_any = api.count_visits(ctx, nmh, rays_d)
    work = api.trace_stats(ctx, nmh, rays_d)
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        api.trace_closest(ctx, nmh, rays_d, hits_d)
    barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clk:
        ev[0].record(stream)
        for s in range(args.steps):
            api.trace_closest(ctx, nmh, rays_d, hits_d)
            ev[s + 1].record(stream)
        barrier()
    launch_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    total_ms = max_over_ranks(ev[0].elapsed_time(ev[-1]), world, "cuda")
    ms_per_step = total_ms / args.steps
    value = replica_throughput(N_RAYS * args.steps, world, total_ms * 1e-3) / 1e6

    # any hit, same rays (reported beside the headline)
    for _ in range(2):
        api.trace_any(ctx, nmh, rays_d, occ_d)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        api.trace_any(ctx, nmh, rays_d, occ_d)
    e1.record(stream)
    barrier()
    any_ms = e0.elapsed_time(e1) / args.steps

    # end to end through the host-buffer C-ABI call
    rays_h = torch.empty((N_RAYS, 8), dtype=torch.float32, pin_memory=True)
    rays_h.numpy()[:] = rays.view(np.float32).reshape(-1, 8)
    hits_h = torch.empty((N_RAYS, 4), dtype=torch.float32, pin_memory=True)
    rh, hh = rays_h.numpy(), hits_h.numpy().view(np.uint8).view(
        np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4")])).reshape(-1)
    e2e_steps = max(3, min(args.steps, 10))
    api.trace_closest_host(ctx, nmh, rh.view(np.uint8).view(rays.dtype).reshape(-1), hh)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        api.trace_closest_host(ctx, nmh, rh.view(np.uint8).view(rays.dtype).reshape(-1), hh)
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_value = world * N_RAYS / e2e_s / 1e6
    same = np.array_equal(hits_h.numpy().view(np.uint32), hits_d.cpu().numpy().view(np.uint32))

    peak, peak_kind = load_peaks()
    wc = work["closest"]
    own_bytes = (N_RAYS * (RAY_IN_BYTES + HIT_OUT_BYTES) + SLAB_BYTES * wc["node_fetches"] +
                 TRI_BYTES * wc["slab_crossings"] + BOX_BYTES * wc["box_loads"])
    ref_bytes = N_RAYS * (REF_RAY_IN_BYTES + HIT_OUT_BYTES) + NODE_BYTES * visits_closest
    avg_launch_s = statistics.mean(launch_ms) * 1e-3
    achieved = ref_bytes / avg_launch_s / 1e9
    traffic, traffic_source = load_traffic()
    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "triangles": N_TRIS, "rays": N_RAYS, "nmh_levels": nmh.info()[1],
                   "l2": "inputs larger than L2: 512 MiB of rays streamed per step; the 64 MB of node records "
                         "stay L2-resident as in any traversal",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_source,
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "definition": "reference algorithm bytes per trace: 24 B ray in + 16 B hit out + 72 B per node "
                                   "the reference's intersect() visits (counted by this traversal without box "
                                   "pruning), divided by the average CUDA-event time of a trace call (its two "
                                   "launches: the warp-packet pass and the one-ray-per-thread pass over the "
                                   "chunks it deferred)",
                     "algorithmic_bytes_per_launch": ref_bytes,
                     "reference_node_visits_per_ray": visits_closest / N_RAYS,
                     "dram_GBps": traffic / avg_launch_s / 1e9 if traffic else None,
                     "dram_frac": traffic / avg_launch_s / 1e9 / peak if traffic else None,
                     "limiter": "instruction issue and the L1 data pipe, not DRAM (see the ncu summary): the 64 MB "
                                "of node records stay in the 129 MB L2, so the algorithmic bytes are served by "
                                "L1/L2 and their rate can exceed the HBM copy peak",
                     "traversal_reads_bytes_per_launch": own_bytes,
                     "traversal_reads_GBps": own_bytes / avg_launch_s / 1e9,
                     "node_fetches_per_ray": wc["node_fetches"] / N_RAYS,
                     "slab_crossings_per_ray": wc["slab_crossings"] / N_RAYS},
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": N_RAYS * 32,
                "d2h_bytes_per_step": N_RAYS * 16, "matches_device_result": bool(same)},
        "gpu_launches": 2 * args.steps,    # k_trace_packets + k_trace per step
        "clocks": clocks,
        "any_hit": {"value": world * N_RAYS / (any_ms * 1e-3) / 1e6, "unit": "Mrays/s", "ms_per_step": any_ms,
                    "node_fetches_per_ray": work["any"]["node_fetches"] / N_RAYS,
                    "reference_node_visits_per_ray": visits_any / N_RAYS},
    }
    checks = Checks()
    checks.add("e2e hits equal the device-resident hits", same)
    levels = nmh.info()[1]
    build_bytes = NMH_LEVEL_BYTES * V.shape[0] * levels
    out["nmh_build"] = {
        "workload": "NMH build of the same 1M-triangle soup (%d levels), warm (graph replay), host wall time of "
                    "the whole aur_nmh_build call, median of 5" % levels,
        "ms": build_ms, "mtris_per_s": N_TRIS / (build_ms * 1e-3) / 1e6,
        "roofline": {"bound": "hbm", "achieved": build_bytes / (build_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": build_bytes / (build_ms * 1e-3) / 1e9 / peak, "algorithmic_bytes_per_build": build_bytes,
                     "definition": "16 B read + 16 B written per triangle per level (key, id, node, permutation)"}}
    if rank == 0 and not args.no_cpu_baseline:
        perm, verts = nmh.export()
        out["cpu_baseline"] = cpu_baseline(verts, perm, rays, args.cpu_sample)
        out["nmh_build"]["cpu_baseline"] = cpu_build_baseline(V, perm)
        checks.add("NMH build of the 1M soup equals the oracle's", out["nmh_build"]["cpu_baseline"].pop("equal"))
    if not args.skip_extras:
        del rays_d, hits_d, occ_d
        cpu = rank == 0 and not args.no_cpu_baseline
        out["cornell_plain"] = bench_cornell(ctx, checks, cpu=cpu)
        out["cornell_textured"] = bench_cornell(ctx, checks, cpu=cpu, textured=True)
        out["filter_pixels"] = bench_filter(ctx)
        out["mis"] = bench_mis(ctx)
        out["batched_wavefront"] = bench_batched(ctx, checks)
        out["adjoint"] = bench_adjoint(ctx, checks)
        out["terrain"] = bench_terrain(ctx, checks, cpu=cpu)
    out["parity"] = checks.summary()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    if checks.failures:
        sys.exit(1)


if __name__ == "__main__":
    main()
