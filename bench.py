"""Benchmark of the raw development path on GB300.

Workload (one step = one develop of one image): the 24 MP darkroom graph,
6000x4000 RGGB uint16 holding 14-bit values (black 512, white 16383), the
seeded synthetic scene with Poisson-Gaussian noise a=8, b=1.6 (DN) and 2% of
the pixels clipped, white balance (2, 1, 1.6), llap at 6 pyramid levels,
denoise -> hilite -> demosaic -> colour -> filmcurv -> llap with the module
defaults and the darkroom .cfg values. Output rgba f16.

value: MP/s of input mosaic with the inputs resident in HBM (a ring of 4
distinct mosaics, 192 MB > 129 MB L2, each with its own captured CUDA graph).
e2e:   the same metric through the public C-ABI call with host buffers: the
pinned host mosaic is uploaded, developed and the rgba f16 result read back
inside the timed region of every step.

--impl reference: the CPU implementation of the path (the oracle, a C++
restatement of the reference shaders, or the reference shaders compiled for
the CPU when that build is present), all host threads, on a bounded sample.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "develop MP/s batched+served vs per-image on 1 GB300 at stated err; p50/p99 latency"
WD, HT = 6000, 4000
BLACK, WHITE = 512.0, 16383.0
NOISE_A, NOISE_B = 8.0, 1.6
LEVELS = 6
RING = 4
DENOISE = 0.0


def img_param(v, wd, ht):
    rng = WHITE - BLACK
    return v.default_img_param(black=BLACK, white=WHITE, wd=wd, ht=ht,
                               noise_a=NOISE_A / rng ** 2, noise_b=NOISE_B / rng)


def config():
    return {"workload": "%d MP darkroom graph, one image per step%s" % (round(WD * HT / 1e6),
                                                                       ", wavelet denoise" if DENOISE > 0 else ""),
            "wd": WD, "ht": HT, "cfa": "rggb", "denoise_strength": DENOISE,
            "bits": 14, "black": BLACK, "white": WHITE, "noise_a_dn": NOISE_A, "noise_b_dn": NOISE_B,
            "llap_levels": LEVELS,
            "graph": "denoise(%s)->hilite->demosaic->colour->filmcurv->llap" % ("wavelet" if DENOISE > 0 else "noop"),
            "l2": "ring of %d distinct resident mosaics (%d MB > 129 MB L2)" % (RING, RING * WD * HT * 2 // 2 ** 20)}


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p:
            time.sleep(0.15)
            self.p.terminate()
            out, _ = self.p.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except (ValueError, IndexError):
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(seconds=10.0, ref=False):
    """The CPU path on a bounded sample of the workload (same recipe, 2000x1332)."""
    import vkdt_gb300 as v
    import oracle
    wd, ht = 2000, 1332
    m = v.scene_host(v.make_scene(wd, ht, seed=1, a=NOISE_A, b=NOISE_B))
    ip = oracle.img_param(img_param(v, wd, ht))
    p = oracle.default_params()
    p.ll_levels = LEVELS
    p.dn_strength = DENOISE
    kind = "port"
    run = lambda: oracle.develop(m, ip, params=p, stages=("llap",))
    if ref:
        try:
            from oracle import glsl_ref
            if glsl_ref.available():
                run = lambda: glsl_ref.develop(m, ip, params=p)
                kind = "reference"
        except ImportError:
            pass
    run()  # warm
    t0 = time.perf_counter()
    n = 0
    while True:
        run()
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    mps = n * wd * ht / 1e6 / dt
    return {"value": mps, "unit": "MP/s", "cores": os.cpu_count(), "kind": kind,
            "sample": "%d develops of a %dx%d mosaic of the same recipe (%.1f s)" % (n, wd, ht, dt)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cb = cpu_baseline(seconds=max(5.0, 2.0 * args.steps), ref=True)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "MP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(),
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "MP/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    global WD, HT, RING, LEVELS, DENOISE
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="cuda")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--size", default="%dx%d" % (WD, HT), help="WxH of the mosaic (profiling of smaller cases)")
    ap.add_argument("--ring", type=int, default=RING, help="number of resident inputs")
    ap.add_argument("--levels", type=int, default=LEVELS, help="llap pyramid depth (0 = automatic)")
    ap.add_argument("--denoise", type=float, default=DENOISE,
                    help="denoise strength (0 = the darkroom default, denoise/noop; > 0 the wavelet path)")
    args = ap.parse_args()
    WD, HT = [int(x) for x in args.size.lower().split("x")]
    RING, LEVELS, DENOISE = args.ring, args.levels, args.denoise
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import vkdt_gb300 as v

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    v.init(local)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    # ring of resident inputs, one graph (and CUDA graph) per slot
    graphs = []
    for i in range(RING):
        g = v.Graph()
        g.set_input(WD, HT, img_param(v, WD, HT))
        if LEVELS:
            g.set_llap_levels(LEVELS)
        if DENOISE > 0:
            g.set_param("denoise", "strength", DENOISE)
        g.alloc()
        src, _ = g.device_buffers()
        v.scene_device(v.make_scene(WD, HT, seed=1000 * rank + i, image_id=i, a=NOISE_A, b=NOISE_B), src, sp)
        graphs.append(g)
    torch.cuda.synchronize()

    def step(i):
        graphs[i % RING].run(flags=0, stream=sp)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- value: device resident
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier()
        ev0.record(stream)
        for i in range(args.steps):
            step(i)
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    mp_step = WD * HT / 1e6
    value = world * args.steps * mp_step / (ms / 1e3)

    # ---- per kernel durations (events around every launch, one sync per step)
    gt = v.Graph()
    gt.set_input(WD, HT, img_param(v, WD, HT))
    if LEVELS:
        gt.set_llap_levels(LEVELS)
    if DENOISE > 0:
        gt.set_param("denoise", "strength", DENOISE)
    gt.set_timing(True)
    gt.alloc()
    src, _ = gt.device_buffers()
    v.scene_device(v.make_scene(WD, HT, seed=1000 * rank + 7, a=NOISE_A, b=NOISE_B), src, sp)
    acc = None
    nt = max(3, min(args.steps, 20))
    for i in range(args.warmup + nt):
        gt.run(flags=0, stream=sp)
        gt.wait()
        t = gt.times()
        if i >= args.warmup:
            vals = np.array([x[1] for x in t])
            acc = vals if acc is None else acc + vals
    names = [x[0] for x in t]
    kms = acc / nt
    launches_per_step = len(names)
    dev_idx = names.index("demosaic:fix")
    dev_ms = float(kms[dev_idx])
    # algorithmic bytes of the fused develop kernel per launch: mosaic in (2 B/px),
    # the hilite coarse level (8 B per (W/4 x H/4) px), filmcurv rgba f16 out (8 B/px),
    # 11 llap level 1 planes out (11 * 2 B per (W/2 x H/2) px)
    npx = WD * HT
    alg = npx * 2 + (WD // 4) * (HT // 4) * 8 + npx * 8 + 11 * 2 * (WD // 2) * (HT // 2)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = alg / (dev_ms / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get("k_develop_bytes_per_launch")
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": "k_develop (hilite doub + demosaic + colour + filmcurv + llap curve/reduce)",
                "kernel_ms": dev_ms, "alg_bytes_per_launch": alg,
                "peak_source": "measured" if peaks else "fallback",
                "per_launch_ms": [[n, round(float(x), 5)] for n, x in zip(names, kms)],
                "per_kernel_ms": {n: round(float(sum(x for m, x in zip(names, kms) if m == n)), 5) for n in names}}
    gt.close()

    # ---- e2e: host mosaic in, host rgba f16 out, through the C-ABI run call
    ge = graphs[0]
    host_in = [v.scene_host(v.make_scene(WD, HT, seed=50 + i, a=NOISE_A, b=NOISE_B)) for i in range(2)] if rank == 0 else None
    if host_in is None:
        host_in = [v.scene_host(v.make_scene(WD, HT, seed=50 + i + 100 * rank, a=NOISE_A, b=NOISE_B)) for i in range(2)]
    lat = []
    ne = max(3, min(args.steps, 20))
    for i in range(args.warmup):
        ge.run(host_in[i % 2], flags=v.RUN_ALL, stream=sp)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(ne):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        ge.source()[...] = host_in[i % 2]
        a.record(stream)
        ge.run(flags=v.RUN_UPLOAD_SOURCE | v.RUN_DOWNLOAD_SINK, stream=sp)
        b.record(stream)
        b.synchronize()
        lat.append(a.elapsed_time(b))
    e1.record(stream)
    barrier()
    lat = np.array(lat)
    e2e_ms = float(lat.mean())
    if world > 1:
        t = torch.tensor([e2e_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e = {"value": world * mp_step / (e2e_ms / 1e3), "unit": "MP/s", "h2d_bytes_per_step": WD * HT * 2,
           "d2h_bytes_per_step": WD * HT * 8, "latency_ms": {"p50": float(np.percentile(lat, 50)),
                                                            "p99": float(np.percentile(lat, 99))}}

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cb = cpu_baseline(seconds=10.0)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "MP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(),
                "roofline": roofline, "cpu_baseline": cb, "e2e": e2e,
                "gpu_launches": launches_per_step * args.steps, "clocks": clk.summary(),
                "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}}
        print(json.dumps(line))
    for g in graphs:
        g.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
