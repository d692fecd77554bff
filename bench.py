"""Ray-query benchmark: closest-hit Mrays/s on the 1M-triangle kd-tree.

Workload (one step): closest hit for 4,194,304 rays (origins uniform in the
scene box, directions uniform on S^2, float32) against a 1,048,576-triangle
displaced sphere (radius 1, gradient-noise amplitude 0.05, seeded) plus
50,000 random triangles of edge ~0.01 in the unit cube -- seeded synthetic
inputs with the shapes of the ray-query microbenchmark configuration.

* value      : rays / kernel time, inputs resident in HBM, L2 flushed (a
               256 MiB write) before every timed step, CUDA events on the
               launching stream.
* e2e        : the same metric through the C ABI host-buffer entry point
               (skw_intersect_host): pinned host rays in, hits out, the
               transfers inside the timed region (on a coherent CPU-GPU
               link the traversal reads the rays from and writes the hits
               to the pinned host buffers itself).
* roofline   : algorithmic bytes per launch (32 + 16 + 32*N_nodes +
               36*N_tris per ray, N from the instrumented oracle on a sample
               of the same rays) / kernel time, against the measured HBM
               copy bandwidth.
* cpu_baseline: the reference's own TriangleAccelerator::Intersect (built
               from its sources) on the host cores over a ray sample.

Multi-GPU: rays are independent, so each rank traces its own 4M-ray batch
(weak scaling, no data-path collective; a max-reduce of the timings only).

--impl reference runs the reference's CPU path instead (rank 0 only).
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "closest-hit Mrays/s (1M-triangle kd-tree, 4M uniform rays)"
UNIT = "Mrays/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--rays", type=int, default=4 * 1024 * 1024)
    p.add_argument("--subdiv", type=int, default=9)
    p.add_argument("--nrandom", type=int, default=50_000)
    p.add_argument("--cpu-sample", type=int, default=1_000_000, help="rays in one CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-render", action="store_true", help="skip the direct-lighting render measurement")
    p.add_argument("--no-batch", action="store_true", help="skip the batched multi-view render measurement")
    p.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement")
    p.add_argument("--no-photon", action="store_true", help="skip the photon-mapping measurement")
    p.add_argument("--knn-sample", type=int, default=0,
                   help="time the k-NN on a uniform random sample of this many of the primary hits (0: all)")
    return p.parse_args()


def config(args, world):
    return {"workload": f"ray-query: displaced sphere 4*4^{args.subdiv} tris + {args.nrandom} random tris, "
                        f"{args.rays} uniform rays per GPU, closest hit",
            "triangles": 4 * 4 ** args.subdiv + args.nrandom, "rays_per_step_per_gpu": args.rays,
            "l2": "flushed before every timed step (256 MiB write)", "parallelism": f"replicas x{world}"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.stop = threading.Event()
        self.t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


_T0 = time.perf_counter()


def log(msg: str) -> None:
    """Progress on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)


def reduce_max(value: float, world: int, device="cpu") -> float:
    """The maximum of a per-rank scalar over all ranks (the slowest rank's
    time); the identity with one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_ray_seed(rank: int) -> int:
    """Each rank traces its own ray batch (weak scaling: rays are independent
    units, no data-path collective)."""
    return 7 + 1000 * rank


def load_traffic(kind: str, rays: int):
    """DRAM bytes per launch from the committed ncu summary, scaled to `rays`."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text()).get(kind)
    if not d:
        return None
    return d.get("dram_bytes_per_launch", 0.0) + d["dram_bytes_per_ray"] * rays


def host_transfer_mode(ctx) -> str:
    """How skw_intersect_host moves pinned host buffers on this device."""
    from skwarka_gb300 import _lib
    if _lib.load().skw_ctx_host_buffers_in_place(ctx.handle) == 1:
        return ("in place: the traversal reads the rays from and writes the hits to the pinned host buffers over "
                "the coherent CPU-GPU link")
    return "staged: 2M-ray chunks copied in and out on two streams, overlapped with the traversals"


def load_l2(kind: str, rays: int, seconds: float):
    """The L2 side of the roofline: L2 bytes per ray (lts__t_sectors of the
    committed ncu capture) at this run's rays per second, against the L2
    peak of the same capture (its bytes over its duration over its
    lts__throughput fraction)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text()).get(kind) or {}
    if "l2_bytes_per_ray" not in d:
        return None
    achieved = d["l2_bytes_per_ray"] * rays / seconds / 1e9
    return {"achieved": achieved, "peak": d["l2_peak_gbs"], "unit": "GB/s", "frac": achieved / d["l2_peak_gbs"],
            "bytes_per_ray": d["l2_bytes_per_ray"],
            "source": "lts__t_sectors per ray and the L2 peak from the committed ncu capture, at this run's rays/s"}


def hit_parity(gpu_hits: np.ndarray, ref: dict) -> dict:
    """Agreement of the GPU's closest hits (int32 (n, 4): t bits, prim, tri,
    flags) with the reference's on the same rays: hit-id agreement over
    (primitive, mesh triangle), the largest relative t difference on agreeing
    hits, and how many GPU hits were decided or refined in double precision
    or flagged as near ties."""
    g = np.asarray(gpu_hits)
    prim, tri, flags = g[:, 1], g[:, 2], g[:, 3].astype(np.uint32)
    t = g[:, 0].copy().view(np.float32).astype(np.float64)
    same = (prim == ref["prim"]) & (tri == ref["tri"])
    hit = same & (ref["prim"] >= 0)
    rel = np.abs(t[hit] - ref["t"][hit]) / np.maximum(np.abs(ref["t"][hit]), 1e-300)
    diff = np.nonzero(~same)[0]
    return {"rays": int(len(g)), "hit_id_agree": float(same.mean()), "mismatches": int(len(diff)),
            "mismatch_near_tie": int(((flags[diff] & 2) != 0).sum()),
            "max_t_rel": float(rel.max()) if len(rel) else 0.0,
            "fp64_decided": int(((flags & 1) != 0).sum()), "near_ties": int(((flags & 2) != 0).sum()),
            "t_refined": int(((flags & 4) != 0).sum()), "hits": int((ref["prim"] >= 0).sum())}


def cpu_model() -> str:
    """The host CPU's model name (from /proc/cpuinfo or lscpu)."""
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            k = line.split(":")[0].strip().lower()
            if k in ("model name", "cpu model", "hardware"):
                return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_baseline(meshes, rays, sample, rank, gpu_hits=None):
    """The reference's own Intersect over `sample` rays on all host cores, plus
    the instrumented oracle's node / triangle counts on the same rays.  With
    the GPU's hits for those rays, the reference's answers are kept and
    compared with them (parity on the timed workload)."""
    from oracle.api import Oracle, Reference
    cores = os.cpu_count() or 1
    sub = rays[:sample]
    oa = Oracle().accel(meshes)
    cnt = oa.intersect(sub[:200_000], counters=True)
    n_nodes, n_tris = float(cnt["nodes"].mean()), float(cnt["tris"].mean())
    if Reference.available():
        ra = Reference().accel(meshes)
        ra.intersect(sub[:10_000])
        t0 = time.perf_counter()
        res = ra.intersect(sub, threads=cores)
        dt = time.perf_counter() - t0
        kind = "reference"
    else:
        t0 = time.perf_counter()
        res = oa.intersect(sub, threads=cores)
        dt = time.perf_counter() - t0
        kind = "port"
    out = {"value": sample / dt / 1e6, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": kind,
           "sample": f"{sample} of the step's rays, TriangleAccelerator::Intersect incl. differential geometry"
           if kind == "reference" else f"{sample} of the step's rays, oracle restatement"}
    parity = hit_parity(gpu_hits[:sample], res) if gpu_hits is not None else None
    return out, (n_nodes, n_tris), parity


def ray_bytes(prims, cams, spp_x, spp_y, light_quads, sample=20_000, seed=11):
    """Algorithmic bytes per ray query of a direct-lighting sample in this
    scene: 32 (ray in) + 16 (hit out) + 32 N_nodes + 36 N_tris, with N the
    mean nodes visited and triangles tested by the instrumented oracle walk
    (the reference's traversal) on a sample of the frame's camera rays, of
    shadow rays from their hits to a uniform point of a quad light (or to a
    point light: light_quads of shape (n, 3)), and of
    cosine-hemisphere BSDF rays from the hits.  Returns the per-kind figures,
    the camera hit fraction and the mean over the rays of one sample (one
    camera ray, one shadow and one BSDF ray per camera hit)."""
    from oracle.api import Oracle
    rng = np.random.default_rng(seed)
    meshes = [(np.asarray(p.mesh.vertices, np.float32), np.asarray(p.mesh.triangles, np.int32)) for p in prims]
    cam_rays = np.concatenate([scenes_camera_rays(c, spp_x, spp_y, seed) for c in cams])
    cam_rays = cam_rays[rng.choice(len(cam_rays), size=min(sample, len(cam_rays)), replace=False)]
    oa = Oracle().accel(meshes)
    ch = oa.intersect(cam_rays, counters=True)
    hit = ch["prim"] >= 0
    p = cam_rays[hit, :3].astype(np.float64) + ch["t"][hit, None] * cam_rays[hit, 3:6].astype(np.float64)
    if light_quads.ndim == 2:  # point lights
        lp = light_quads[rng.integers(len(light_quads), size=len(p))]
    else:
        quad = light_quads[rng.integers(len(light_quads), size=len(p))]
        u, v = rng.uniform(size=(2, len(p), 1))
        lp = quad[:, 0] + u * (quad[:, 1] - quad[:, 0]) + v * (quad[:, 3] - quad[:, 0])
    to = lp - p
    dist = np.linalg.norm(to, axis=1)
    sray = np.zeros((len(p), 8), np.float32)
    sray[:, :3], sray[:, 3:6] = p, to / dist[:, None]
    sray[:, 6], sray[:, 7] = 1e-4, dist - 1e-4
    _, sn, st = oa.intersect_test(sray, counters=True)
    d = rng.normal(size=(len(p), 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d *= np.sign((d * -cam_rays[hit, 3:6]).sum(1))[:, None]  # the hemisphere facing the camera
    bray = np.zeros((len(p), 8), np.float32)
    bray[:, :3], bray[:, 3:6], bray[:, 6], bray[:, 7] = p, d, 1e-4, np.inf
    bh = oa.intersect(bray, counters=True)

    def b(nodes, tris):
        return 48.0 + 32.0 * float(np.mean(nodes)) + 36.0 * float(np.mean(tris))
    f = float(hit.mean())
    cb, sb, bb = b(ch["nodes"], ch["tris"]), b(sn, st), b(bh["nodes"], bh["tris"])
    return {"camera_ray_bytes": cb, "shadow_ray_bytes": sb, "bsdf_ray_bytes": bb, "camera_hit_fraction": f,
            "mean_ray_bytes": (cb + f * (sb + bb)) / (1.0 + 2.0 * f)}


def scenes_camera_rays(cam, spp_x, spp_y, seed):
    from skwarka_gb300 import scenes
    return scenes.camera_rays(cam, spp_x, spp_y, seed=seed)


def render_roofline(msamples_per_s, rays_per_sample, rb, what, extra_per_ray=0.0):
    """HBM roofline of a render line: bytes per sample = rays traced per
    sample (counted on the device over the timed frames) x the mean
    algorithmic bytes per ray (+ extra_per_ray) + 24 bytes of film + 68 bytes
    of shading reads (triangle attributes and material) per camera hit."""
    peak, kind = peaks()
    bps = rays_per_sample * (rb["mean_ray_bytes"] + extra_per_ray) + 24.0 + 68.0 * rb["camera_hit_fraction"]
    achieved = msamples_per_s * 1e6 * bps / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "bytes_per_sample": bps, "rays_per_sample": rays_per_sample, "peak_source": kind, "what": what, **rb}


def photon_ray_bytes(prims, light_pos, sample=20_000, seed=12):
    """Algorithmic bytes per ray query of photon shooting on this scene
    (32 + 16 + 32 N_nodes + 36 N_tris, N from the instrumented oracle walk):
    rays leaving the point light in uniform directions, and cosine bounce
    rays from their hits.  Returns (emitted, bounce) bytes per ray."""
    from oracle.api import Oracle
    rng = np.random.default_rng(seed)
    meshes = [(np.asarray(p.mesh.vertices, np.float32), np.asarray(p.mesh.triangles, np.int32)) for p in prims]
    oa = Oracle().accel(meshes)
    d = rng.normal(size=(sample, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    er = np.zeros((sample, 8), np.float32)
    er[:, :3], er[:, 3:6], er[:, 6], er[:, 7] = np.asarray(light_pos), d, 0.0, np.inf
    eh = oa.intersect(er, counters=True)
    hit = eh["prim"] >= 0
    p = er[hit, :3].astype(np.float64) + eh["t"][hit, None] * er[hit, 3:6].astype(np.float64)
    bd = rng.normal(size=(len(p), 3))
    bd /= np.linalg.norm(bd, axis=1, keepdims=True)
    bd *= np.sign((bd * -er[hit, 3:6]).sum(1))[:, None]
    br = np.zeros((len(p), 8), np.float32)
    br[:, :3], br[:, 3:6], br[:, 6], br[:, 7] = p, bd, 1e-4, np.inf
    bh = oa.intersect(br, counters=True)

    def b(h):
        return 48.0 + 32.0 * float(np.mean(h["nodes"])) + 36.0 * float(np.mean(h["tris"]))
    return b(eh), b(bh)


def light_quads(prims):
    return np.stack([np.asarray(p.mesh.vertices, np.float64)[:4] for p in prims if any(p.emission)])


def knn_parity(gpu: dict, gpu_perm: np.ndarray, ref: dict, ref_perm: np.ndarray) -> dict:
    """Agreement of the GPU's k-NN answers with the reference's on the same
    queries and photons: found counts, index sets, heap order and squared
    distances (indices mapped through each tree's permutation to input
    order, so that the comparison does not rest on the two trees' orders)."""
    def ids(idx, perm):
        out = np.where(idx >= 0, perm[np.maximum(idx, 0)], -1)
        return out
    gi, ri = ids(gpu["idx"], gpu_perm), ids(ref["idx"], ref_perm)
    sets = np.array_equal(np.sort(gi, axis=1), np.sort(ri, axis=1))
    return {"queries": int(len(gi)), "counts_equal": bool(np.array_equal(gpu["count"], ref["count"])),
            "sets_equal": bool(sets), "order_equal": bool(np.array_equal(gi, ri)),
            "d2_equal": bool(np.array_equal(gpu["d2"].view(np.uint64), ref["d2"].view(np.uint64))),
            "rows_differing": int((gi != ri).any(axis=1).sum())}


def render_bench(args, dev, ctx, measure_cpu):
    """Plain direct lighting (256 x 256, 2x2 stratified samples, one light
    sample per hit, the 12-triangle box + 20,480-triangle spheres + quad
    light): samples/s of the GPU wavefront renderer on the device and end to
    end (film copied to pinned host memory), next to the reference's
    SamplerBasedRenderer on the host cores."""
    import torch
    from skwarka_gb300 import scenes
    from skwarka_gb300.render import RenderScene
    prims, mats, camf = scenes.direct_lighting_box()
    cam = camf(256, 256)
    spp = 4
    samples = cam.width * cam.height * spp
    sc = RenderScene(prims, mats, ctx=ctx)
    film = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device=dev)
    hfilm = torch.empty((cam.height, cam.width, 3), dtype=torch.float32).pin_memory()
    stream = torch.cuda.current_stream(dev)
    for i in range(max(3, args.warmup)):
        sc.render_direct(cam, 2, 2, seed=i, out=film)
    torch.cuda.synchronize()
    steps = max(5, args.steps)
    l0 = ctx.launch_count()
    r0 = sc.accelerator().rays_traced()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for i in range(steps):
        sc.render_direct(cam, 2, 2, seed=100 + i, out=film)
    e.record(stream)
    torch.cuda.synchronize()
    dev_ms = s.elapsed_time(e) / steps
    launches = (ctx.launch_count() - l0) / steps
    rays_per_sample = (sc.accelerator().rays_traced() - r0) / (steps * samples)
    t0 = time.perf_counter()
    for i in range(steps):
        sc.render_direct(cam, 2, 2, seed=200 + i, out=film)
        hfilm.copy_(film, non_blocking=True)
        stream.synchronize()
    e2e_ms = (time.perf_counter() - t0) / steps * 1e3
    # the same frame with the LDSampler (4 samples per pixel)
    from skwarka_gb300.render import LD
    for i in range(3):
        sc.render_direct(cam, 2, 2, seed=i, out=film, sampler=LD)
    s.record(stream)
    for i in range(steps):
        sc.render_direct(cam, 2, 2, seed=300 + i, out=film, sampler=LD)
    e.record(stream)
    torch.cuda.synchronize()
    ld_ms = s.elapsed_time(e) / steps
    out = {"workload": "direct lighting, 256x256, 2x2 spp, 1 light sample, box + 20,480-tri spheres + quad light",
           "unit": "Msamples/s", "value": samples / dev_ms / 1e3, "ms_per_frame": dev_ms,
           "e2e": {"value": samples / e2e_ms / 1e3, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": hfilm.numel() * 4},
           "gpu_launches_per_frame": launches,
           "ld_sampler": {"value": samples / ld_ms / 1e3, "unit": "Msamples/s", "ms_per_frame": ld_ms}}
    out["roofline"] = render_roofline(out["value"], rays_per_sample, ray_bytes(prims, [cam], 2, 2, light_quads(prims)),
                                      "rays traced per sample x algorithmic bytes per ray (the oracle's visit "
                                      "counts on the frame's camera, shadow and BSDF rays) + film + shading reads")
    if measure_cpu:
        from oracle.api import Reference
        if Reference.available():
            log("reference render")
            ref = Reference()
            ref.render_direct(prims, mats, [], camf(64, 64), 2, 2)
            _, sec = ref.render_direct(prims, mats, [], cam, 2, 2)
            out["cpu_baseline"] = {"value": samples / sec / 1e6, "unit": "Msamples/s", "cores": os.cpu_count() or 1, "cpu": cpu_model(),
                                   "kind": "reference", "sample": "one full 256x256 4-spp frame, SamplerBasedRenderer"}
    return out


def specular_bench(args, dev, ctx, measure_cpu):
    """Direct lighting with specular recursion (maximum depth 6): a glass
    sphere (1,024 triangles, index 1.5) above a matte floor under a quad
    light, 256 x 256, 2x2 spp; GPU samples/s beside the reference's
    SamplerBasedRenderer on the host cores."""
    import torch
    from skwarka_gb300 import scenes
    from skwarka_gb300.render import TRANSPARENT, Material, RenderScene
    glass = Material(kind=TRANSPARENT, kd=(1.0, 1.0, 1.0), ks=(1.0, 1.0, 1.0), refractive_index=1.5)
    prims, mats, lights, cam = scenes.glass_sphere_scene(glass, "area", (256, 256))
    samples = cam.width * cam.height * 4
    sc = RenderScene(prims, mats, lights, ctx=ctx)
    sc.set_max_specular_depth(6)
    film = torch.empty((cam.height, cam.width, 3), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for i in range(3):
        sc.render_direct(cam, 2, 2, seed=i, out=film)
    torch.cuda.synchronize()
    steps = max(5, args.steps)
    l0 = ctx.launch_count()
    r0 = sc.accelerator().rays_traced()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for i in range(steps):
        sc.render_direct(cam, 2, 2, seed=100 + i, out=film)
    e.record(stream)
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / steps
    rays_per_sample = (sc.accelerator().rays_traced() - r0) / (steps * samples)
    out = {"workload": "direct lighting + specular recursion (depth 6), glass sphere over a floor, 256x256, 2x2 spp",
           "unit": "Msamples/s", "value": samples / ms / 1e3, "ms_per_frame": ms,
           "gpu_launches_per_frame": (ctx.launch_count() - l0) / steps,
           "mrays_per_s": samples * rays_per_sample / ms / 1e3}
    out["roofline"] = render_roofline(out["value"], rays_per_sample, ray_bytes(prims, [cam], 2, 2, light_quads(prims)),
                                      "rays traced per sample (the specular trees included) x algorithmic bytes per "
                                      "ray (the oracle's visit counts on the frame's camera, shadow and BSDF rays) + "
                                      "film + shading reads")
    if measure_cpu:
        from oracle.api import Reference
        if Reference.available():
            log("reference specular render")
            _, sec = Reference().render_direct(prims, mats, lights, cam, 2, 2)
            out["cpu_baseline"] = {"value": samples / sec / 1e6, "unit": "Msamples/s", "cores": os.cpu_count() or 1, "cpu": cpu_model(),
                                   "kind": "reference",
                                   "sample": "one full 256x256 4-spp frame, SamplerBasedRenderer, max specular depth 6"}
    return out


def batch_bench(args, dev, ctx):
    """64 views of the 200k-triangle scene (square films, side log-uniform in
    [64, 1024]), 8 samples per pixel (4x2), one light sample: 64 sequential
    single-camera renders against one autotuned batch (one CUDA graph launch
    per run).  Both produce bit-identical images (same per-view seeds), so
    their image error is equal by construction."""
    import torch
    from skwarka_gb300 import scenes
    from skwarka_gb300.render import RenderBatch, RenderScene
    prims, mats = scenes.batching_scene()
    cams = scenes.batching_views(64)
    sc = RenderScene(prims, mats, ctx=ctx)
    b = RenderBatch(sc, cams, 4, 2, seed=1)
    samples = sum(c.width * c.height for c in cams) * 8
    films = b.new_films()
    stream = torch.cuda.current_stream(dev)
    views = [b.view(films, v) for v in range(len(cams))]

    def plain():
        for v, c in enumerate(cams):
            sc.render_direct(c, 4, 2, seed=1 + v, out=views[v])

    def timed(fn, reps):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(reps):
            fn()
        e.record(stream)
        torch.cuda.synchronize()
        return s.elapsed_time(e) / reps

    reps = 3
    plain()
    torch.cuda.synchronize()
    plain_ms = timed(plain, reps)
    ref_img = films.clone()
    default_cfg = b.config()
    b.run(films)
    default_ms = timed(lambda: b.run(films), reps)
    t0 = time.perf_counter()
    cfg, tuned_ms, n_cand = b.autotune()
    tune_s = time.perf_counter() - t0
    b.run(films)
    l0 = ctx.launch_count()
    r0 = sc.accelerator().rays_traced()
    batch_ms = timed(lambda: b.run(films), reps)
    launches = (ctx.launch_count() - l0) / reps
    rays_per_sample = (sc.accelerator().rays_traced() - r0) / (reps * samples)
    identical = bool(torch.equal(films, ref_img))
    roof = render_roofline(samples / batch_ms / 1e3, rays_per_sample,
                           ray_bytes(prims, cams[::8], 4, 2, light_quads(prims)),
                           "batched run: rays traced per sample x algorithmic bytes per ray (the oracle's visit "
                           "counts on camera, shadow and BSDF rays of 8 of the views) + film + shading reads")
    return {"workload": "64 views of the 201,742-tri scene, films 64^2..1024^2 log-uniform, 8 spp, 1 light sample",
            "roofline": roof,
            "samples_per_run": samples, "unit": "Msamples/s",
            "plain_value": samples / plain_ms / 1e3, "batched_value": samples / batch_ms / 1e3,
            "speedup": plain_ms / batch_ms, "plain_ms": plain_ms, "batched_ms": batch_ms,
            "batched_default_config_ms": default_ms, "default_config": default_cfg, "tuned_config": cfg,
            "autotune_s": tune_s, "autotune_candidates": n_cand, "images_bit_identical": identical,
            "kernel_launches_per_run": launches, "graph_launches_per_run": 1}


def adjoint_bench(args, dev, ctx):
    """Direct-lighting adjoint on the 200k-triangle scene at 512x512, 16 spp
    (4x4), one light sample: forward render time against adjoint time (the
    adjoint replays the forward's rays and accumulates per-triangle albedo
    and emission-scale gradients), CUDA events on the launching stream."""
    import numpy as np
    import torch
    from skwarka_gb300 import scenes
    from skwarka_gb300.adjoint import DirectLighting
    from skwarka_gb300.render import Camera, RenderScene
    prims, mats = scenes.batching_scene()
    sc = RenderScene(prims, mats, ctx=ctx)
    cam = Camera.look_at((0.0, 0.3, -0.9), (0.0, -0.4, 0.6), (0, 1, 0), np.radians(70), 512, 512)
    r = DirectLighting(sc, cam, 4, 4, 1, seed=3)
    rng = np.random.default_rng(6)
    albedo = torch.tensor(rng.uniform(0.1, 0.9, size=(sc.n_triangles, 3)), dtype=torch.float32, device=dev)
    target = r.forward_image((albedo + torch.tensor(rng.normal(0, 0.05, size=albedo.shape), dtype=torch.float32,
                                                    device=dev)).clamp(0, 1), 1.0)
    img = r.forward_image(albedo, 1.0)
    d_img = 2.0 * (img - target)
    stream = torch.cuda.current_stream(dev)

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(reps):
            fn()
        e.record(stream)
        torch.cuda.synchronize()
        return s.elapsed_time(e) / reps

    acc = sc.accelerator()
    fwd_ms = timed(lambda: r.forward_image(albedo, 1.0))
    r0 = acc.rays_traced()
    adj_ms = timed(lambda: r.adjoint(albedo, 1.0, d_img))
    samples = 512 * 512 * 16
    rays_per_sample = (acc.rays_traced() - r0) / (6 * samples)  # timed() runs the adjoint 1 + 5 times
    out = {"workload": "adjoint of direct lighting, 201,742-tri scene, 512x512, 16 spp, per-triangle albedo + "
                       "emission scale", "forward_ms": fwd_ms, "adjoint_ms": adj_ms, "adjoint_over_forward": adj_ms / fwd_ms,
           "forward_msamples_s": samples / fwd_ms / 1e3, "adjoint_msamples_s": samples / adj_ms / 1e3}
    out["roofline"] = render_roofline(samples / adj_ms / 1e3, rays_per_sample,
                                      ray_bytes(prims, [cam], 4, 4, light_quads(prims)),
                                      "adjoint: rays traced per sample x (algorithmic bytes per ray + 12 bytes of "
                                      "gradient atomics per ray) + film + shading reads", extra_per_ray=12.0)
    # the same with the configuration's homogeneous medium in the box
    from skwarka_gb300.render import Medium
    sc.set_medium(Medium(sigma_a=(0.05,) * 3, sigma_s=(0.2,) * 3, g=0.3, step=0.05))
    img = r.forward_image(albedo, 1.0)
    d_img = 2.0 * (img - target)
    fwd_m = timed(lambda: r.forward_image(albedo, 1.0), 3)
    adj_m = timed(lambda: r.adjoint(albedo, 1.0, d_img), 3)
    out["with_medium"] = {"medium": "sigma_a 0.05, sigma_s 0.2, HG g 0.3, march step 0.05, box [-1,1]^3",
                          "forward_ms": fwd_m, "adjoint_ms": adj_m, "adjoint_over_forward": adj_m / fwd_m}
    sc.set_medium(None)
    return out


def photon_bench(args, dev, ctx, measure_cpu):
    """Photon mapping on the 1M-triangle scene (matte 0.6, point light of
    intensity 50): 2M photon paths of at most 8 bounces with Russian roulette
    p = 0.7 shot on the GPU (paths/s), the maps' host kd-trees and GPU
    irradiance map (build time), k = 100 filtered nearest photons within 0.05
    of the 512x512x16 primary hits in the direct map (queries/s), and the
    photon-mapping render (16 gather samples) at 512x512 with 4 spp
    (samples/s).  Next to it: the reference's ShootPhotons(2M) (its own
    bounce and Russian-roulette rules) and its KDTree lookups on a sample of
    the same queries, on the host cores."""
    import torch
    from skwarka_gb300 import scenes
    from skwarka_gb300.accel import Primitive, TriangleAccelerator
    from skwarka_gb300.kdtree import PhotonKDTree, direction_table
    from skwarka_gb300.photon import PhotonMap, render_photon
    from skwarka_gb300.render import RenderScene
    prims, mats, lights, camf = scenes.photon_scene(args.subdiv, args.nrandom)
    sc = RenderScene(prims, mats, lights, ctx=ctx)
    paths = 2_000_000
    PhotonMap.shoot(sc, 100_000, max_bounces=8, rr_probability=0.7, seed=1)  # warm-up
    torch.cuda.synchronize()
    sacc = sc.accelerator()
    r0 = sacc.rays_traced()
    t0 = time.perf_counter()
    pm = PhotonMap.shoot(sc, paths, max_bounces=8, rr_probability=0.7, seed=2)
    wall = time.perf_counter() - t0
    shoot_rays = sacc.rays_traced() - r0
    info = pm.info()
    out = {"workload": "2M photon paths (<= 8 bounces, RR p=0.7) on the 1,098,576-tri scene, matte 0.6, "
                       "point light I=50; k=100 r=0.05 lookups at 512x512x16 primary hits; render 512x512x4 spp",
           "paths": paths, "shoot_paths_per_s": paths / (info["shoot_ms"] / 1e3), "shoot_ms": info["shoot_ms"],
           "maps_build_ms": info["build_ms"], "shoot_and_build_wall_s": wall,
           "trees_on_gpu": {k: bool(info["trees_on_gpu"] & (1 << i)) for i, k in
                            enumerate(("caustic", "direct", "indirect"))},
           "photons": {k: info["n_" + k] for k in ("caustic", "direct", "indirect", "irradiance")}}
    # shooting roofline: rays traced (emitted + bounces, counted on the device)
    # at the oracle's bytes per emitted / bounce ray, plus 28 bytes per stored
    # photon (position, normal and direction ids, weight)
    eb, bb = photon_ray_bytes(prims, lights[0].position)
    stored = sum(info["n_" + k] for k in ("caustic", "direct", "indirect"))
    shoot_bytes = paths * eb + max(shoot_rays - paths, 0) * bb + 28.0 * stored
    peak, peak_kind = peaks()
    ach = shoot_bytes / (info["shoot_ms"] / 1e3) / 1e9
    out["shoot_roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                             "rays_per_path": shoot_rays / paths, "emitted_ray_bytes": eb, "bounce_ray_bytes": bb,
                             "peak_source": peak_kind,
                             "what": "rays traced (device count) x the oracle's bytes per emitted / bounce ray + 28 B "
                                     "per stored photon, over the shooting time"}
    # the same shoot with the reference's own rules (luminance Russian
    # roulette, no bounce cap within the 1,024 the GPU allows): the figure to
    # set beside the reference's ShootPhotons
    PhotonMap.shoot(sc, 100_000, max_bounces=1024, rr_probability=0.0, seed=1)
    torch.cuda.synchronize()
    pm_ref_rules = PhotonMap.shoot(sc, paths, max_bounces=1024, rr_probability=0.0, seed=2)
    ir = pm_ref_rules.info()
    out["shoot_reference_rules"] = {
        "rules": "luminance Russian roulette (the reference's), bounce cap 1024", "paths_per_s":
        paths / (ir["shoot_ms"] / 1e3), "shoot_ms": ir["shoot_ms"], "maps_build_ms": ir["build_ms"],
        "photons": {k: ir["n_" + k] for k in ("caustic", "direct", "indirect", "irradiance")}}
    del pm_ref_rules
    # k-NN at the primary hits
    cam = camf(512, 512)
    rays = torch.from_numpy(scenes.camera_rays(cam, 4, 4, seed=3)).to(dev)
    acc = TriangleAccelerator([Primitive(p.mesh) for p in prims], ctx)
    hits = acc.intersect(rays)
    torch.cuda.synchronize()
    t = hits[:, 0].view(torch.float32)
    ok = hits[:, 1] >= 0
    r, tt = rays[ok], t[ok].double()
    q = (r[:, :3].double() + tt[:, None] * r[:, 3:6].double()).contiguous()
    prim, tri = hits[ok, 1].long(), hits[ok, 2].long()
    nrm = torch.zeros_like(q)
    for pi, p in enumerate(prims):
        sel = prim == pi
        if not bool(sel.any()):
            continue
        v = torch.from_numpy(np.asarray(p.mesh.vertices, np.float64)).to(dev)
        tr = torch.from_numpy(np.asarray(p.mesh.triangles, np.int64)).to(dev)[tri[sel]]
        n = torch.linalg.cross(v[tr[:, 1]] - v[tr[:, 0]], v[tr[:, 2]] - v[tr[:, 0]])
        nrm[sel] = n / n.norm(dim=1, keepdim=True)
    qn = nrm.contiguous()
    if 0 < args.knn_sample < q.shape[0]:
        keep = torch.from_numpy(np.sort(np.random.default_rng(6).choice(q.shape[0], size=args.knn_sample,
                                                                         replace=False))).to(dev)
        q, qn = q[keep].contiguous(), qn[keep].contiguous()
    direct = pm.export("direct")
    kd = PhotonKDTree(direct["position"], direct["normal"], ctx=ctx)
    # warm-up at the full size, so that the timed call reuses its output buffers
    kd.get_nearest_points(q, qn, 100, 0.05, 0.87)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # three timed lookups, the median reported (each writes 12 bytes per
    # neighbour slot, 3.6 GB at full size: far past L2 between them)
    runs = []
    for _ in range(3):
        res = None  # its buffers back to the cache: the next call reuses them, no allocation inside the timing
        s.record()
        res = kd.get_nearest_points(q, qn, 100, 0.05, 0.87)
        e.record()
        torch.cuda.synchronize()
        runs.append(s.elapsed_time(e))
    knn_ms = float(np.median(runs))
    nq = q.shape[0]
    out["knn"] = {"queries": nq, "ms": knn_ms, "queries_per_s": nq / (knn_ms / 1e3), "ms_runs": runs,
                  "mean_found": float(res["count"].float().mean())}
    # photon-mapping render
    cam4 = camf(512, 512)
    render_photon(sc, pm, camf(64, 64), 2, 2, gather_samples=16)
    torch.cuda.synchronize()
    r0 = sacc.rays_traced()
    s.record()
    render_photon(sc, pm, cam4, 2, 2, gather_samples=16, seed=4)
    e.record()
    torch.cuda.synchronize()
    rms = s.elapsed_time(e)
    rsamples = 512 * 512 * 4
    rrays = (sacc.rays_traced() - r0) / rsamples
    out["render"] = {"samples": rsamples, "ms": rms, "msamples_per_s": rsamples / rms / 1e3,
                     "roofline": render_roofline(rsamples / rms / 1e3, rrays,
                                                 ray_bytes(prims, [cam4], 2, 2,
                                                           np.asarray([l.position for l in lights], np.float64)),
                                                 "rays traced per sample (camera, shadow and gather rays) x "
                                                 "algorithmic bytes per ray (the oracle's visit counts on the frame's "
                                                 "camera, shadow and cosine rays) + film + shading reads; the "
                                                 "irradiance-photon lookups of the gather hits are not counted")}
    if measure_cpu:
        from oracle.api import Reference
        if Reference.available():
            log("reference photon shooting and lookups")
            ref = Reference()
            from skwarka_gb300.render import Camera
            nocam = Camera(np.eye(4), 1.0, 0, 0)
            _, rinfo = ref.render_photon(prims, mats, lights, nocam, 1, 1, paths, gather_samples=16)
            # a uniform random sample of the queries: they are in image order, and
            # a prefix (the top rows) sees far fewer photons than the average query
            ns = 200_000
            rkd = ref.kdtree(direct["position"], direct["normal"], direct["incident"])
            pick = np.sort(np.random.default_rng(5).choice(q.shape[0], size=min(ns, q.shape[0]), replace=False))
            qs, qns = q.cpu().numpy()[pick], qn.cpu().numpy()[pick]
            ns = len(pick)
            t0 = time.perf_counter()
            rres = rkd.knn(qs, qns, 100, 0.05, 0.87, threads=os.cpu_count() or 1)
            kdt = time.perf_counter() - t0
            out["knn"]["parity"] = knn_parity({k: v.cpu().numpy()[pick] for k, v in res.items()}, kd.perm, rres,
                                              rkd.perm)
            # the k-NN roofline: algorithmic bytes per query 32 + 36 N_visited + 8 k
            # (query in; node and photon per visited point; results out), N_visited
            # from the instrumented oracle walk (the reference's order) on the sample
            from oracle.api import Oracle
            ok_ = Oracle().kdtree(direct["position"], direct["normal"])
            cnt = ok_.knn(qs, qns, 100, 0.05, 0.87, counters=True, threads=os.cpu_count() or 1)
            n_vis = float(cnt["visited"].mean())
            bpq = 32 + 36 * n_vis + 8 * 100
            achieved = bpq * nq / (knn_ms / 1e3) / 1e9
            peak, peak_kind = peaks()
            out["knn"]["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                      "frac": achieved / peak, "bytes_per_query": bpq,
                                      "visited_per_query": n_vis, "peak_source": peak_kind}
            out["cpu_baseline"] = {
                "kind": "reference", "cores": os.cpu_count() or 1, "cpu": cpu_model(),
                "shoot_paths_per_s": paths / rinfo["shoot_s"], "shoot_s_incl_maps": rinfo["shoot_s"],
                "photons": {k: rinfo[k] for k in ("caustic", "direct", "indirect", "irradiance")},
                "knn_queries_per_s": ns / kdt,
                "sample": f"ShootPhotons({paths}) with the reference's own rules (no bounce cap, luminance Russian "
                          f"roulette), incl. its kd-trees and irradiance map; KDTree::GetNearestPoints on {ns} of "
                          "the GPU's queries (uniform random sample, kept in image order) against the same direct "
                          "photons"}
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    from skwarka_gb300 import scenes
    from oracle.api import Oracle, Reference
    meshes = scenes.ray_query_scene(args.subdiv, args.nrandom, seed=3)
    lo, hi = scenes.scene_bounds(meshes)
    # the same rays as rank 0 of the GPU arm traces, all of them every step
    rays = scenes.uniform_rays(args.rays, lo, hi, seed=rank_ray_seed(0))
    cores = os.cpu_count() or 1
    if Reference.available():
        acc, kind = Reference().accel(meshes), "reference"
    else:
        acc, kind = Oracle().accel(meshes), "port"
    for _ in range(args.warmup):
        acc.intersect(rays[:100_000], threads=cores)  # warm-up on a slice of the rays
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        acc.intersect(rays, threads=cores)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.rays * args.steps / total / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args, world),
            "note": "host CPU (no L2 flush); TriangleAccelerator::Intersect includes the differential geometry "
                    "of each hit",
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": kind,
                             "sample": f"all {args.rays} rays of the step, every step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from skwarka_gb300 import scenes
    from skwarka_gb300.accel import Context, Primitive, TriangleAccelerator, TriangleMesh

    log("building the ray-query scene")
    meshes = scenes.ray_query_scene(args.subdiv, args.nrandom, seed=3)
    lo, hi = scenes.scene_bounds(meshes)
    rays_np = scenes.uniform_rays(args.rays, lo, hi, seed=rank_ray_seed(rank))
    ctx = Context(local)
    acc = TriangleAccelerator([Primitive(TriangleMesh(v, t)) for v, t in meshes], ctx)
    rays = torch.from_numpy(rays_np).to(dev)
    hits = torch.empty((args.rays, 4), dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    from skwarka_gb300 import _lib
    lib = _lib.load()

    def step():
        _lib.check(lib.skw_intersect(acc.handle, rays.data_ptr(), args.rays, hits.data_ptr(), stream.cuda_stream),
                   ctx.handle)

    log("accelerator built; warm-up")
    for _ in range(args.warmup):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    launches0 = ctx.launch_count()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for s, e in evs:
            flush.fill_(float(len(evs)))
            s.record(stream)
            step()
            e.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    launches = ctx.launch_count() - launches0
    kern_ms = [s.elapsed_time(e) for s, e in evs]
    total_s = reduce_max(sum(kern_ms), world, dev) / 1e3
    value = args.rays * args.steps * world / total_s / 1e6

    log("closest-hit timed; end-to-end")
    # End to end through the host-buffer entry point (copies included).
    hrays = torch.from_numpy(rays_np).pin_memory()
    hhits = torch.empty((args.rays, 4), dtype=torch.int32).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        _lib.check(lib.skw_intersect_host(acc.handle, hrays.data_ptr(), args.rays, hhits.data_ptr()), ctx.handle)
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        _lib.check(lib.skw_intersect_host(acc.handle, hrays.data_ptr(), args.rays, hhits.data_ptr()), ctx.handle)
    e2e_s = reduce_max(time.perf_counter() - t0, world, dev)
    e2e = args.rays * e2e_steps * world / e2e_s / 1e6

    log("any-hit")
    # Any-hit throughput (shadow rays, tmax ~ U[0, 2]) for the record.
    srays = torch.from_numpy(scenes.uniform_rays(args.rays, lo, hi, seed=8 + 1000 * rank, tmax_range=(0, 2))).to(dev)
    occ = torch.empty(args.rays, dtype=torch.uint8, device=dev)
    a_ms = []
    for i in range(args.warmup + 5):
        flush.fill_(3.0)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        _lib.check(lib.skw_intersect_test(acc.handle, srays.data_ptr(), args.rays, occ.data_ptr(), stream.cuda_stream),
                   ctx.handle)
        e.record(stream)
        torch.cuda.synchronize()
        if i >= args.warmup:
            a_ms.append(s.elapsed_time(e))
    anyhit = args.rays / (sum(a_ms) / len(a_ms) / 1e3) / 1e6

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return 0

    cpu = None
    parity = None
    n_nodes, n_tris = None, None
    if not args.no_cpu_baseline and world == 1:
        log("CPU baseline (reference Intersect)")
        cpu, (n_nodes, n_tris), parity = cpu_baseline(meshes, rays_np, min(args.cpu_sample, args.rays), rank,
                                                      gpu_hits=hits.cpu().numpy())
    render = None
    if not args.no_render:
        log("direct-lighting render")
        render = render_bench(args, dev, ctx, measure_cpu=not args.no_cpu_baseline and world == 1)
    specular = None
    if not args.no_render:
        log("specular render")
        specular = specular_bench(args, dev, ctx, measure_cpu=not args.no_cpu_baseline and world == 1)
    batch = None
    if not args.no_batch:
        log("batched multi-view render")
        batch = batch_bench(args, dev, ctx)
    adjoint = None
    if not args.no_adjoint:
        log("adjoint")
        adjoint = adjoint_bench(args, dev, ctx)
    photon = None
    if not args.no_photon:
        log("photon mapping")
        photon = photon_bench(args, dev, ctx, measure_cpu=not args.no_cpu_baseline and world == 1)
    peak, peak_kind = peaks()
    per_launch_s = sum(kern_ms) / len(kern_ms) / 1e3
    roofline = None
    if n_nodes is not None:
        bytes_per_ray = 32 + 16 + 32 * n_nodes + 36 * n_tris
        achieved = bytes_per_ray * args.rays / per_launch_s / 1e9
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": load_traffic("closest", args.rays),
                    "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                    else "fallback 6.8 TB/s",
                    "bytes_per_ray": bytes_per_ray, "nodes_per_ray": n_nodes, "tris_per_ray": n_tris,
                    "l2": load_l2("closest", args.rays, per_launch_s)}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sum(kern_ms) / len(kern_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(args, world),
            "e2e": {"value": e2e, "unit": UNIT, "transfer": host_transfer_mode(ctx),
                    "h2d_bytes_per_step": args.rays * 32,
                    "d2h_bytes_per_step": args.rays * 16},
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "clocks": clk.summary(), "gpu_launches": launches,
            "wall_s_timed_region": wall, "anyhit_mrays_s": anyhit, "render": render, "specular": specular, "batch": batch, "adjoint": adjoint, "photon": photon,
            "accel": {k: acc.info[k] for k in ("n_nodes", "max_depth", "build_ms", "built_on_device", "device_bytes")}}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
