"""Benchmark of the raw development path on GB300.

Workload (one step = one develop of one image): the 24 MP full darkroom
graph, 6000x4000 RGGB uint16 holding 14-bit values (black 512, white 16383),
the seeded synthetic scene with Poisson-Gaussian noise a=8, b=1.6 (DN) and 2%
of the pixels clipped, white balance (2, 1, 1.6), llap at 6 pyramid levels,
the chain of bin/default-darkroom.i-raw: denoise -> hilite -> demosaic -> crop
-> colour -> filmcurv -> llap -> grade with the module defaults and the .cfg's
values (crop at its defaults: the exif rotation, none here, and a 3 px margin,
so the output is 5993x3994). --graph chain drops crop and grade (the 6000x4000
output of the plain chain). Output rgba f16.

value: MP/s of input mosaic with the inputs resident in HBM (a ring of 4
distinct mosaics, 192 MB > 129 MB L2, each with its own captured CUDA graph).
e2e:   the same metric through the public C-ABI call with host buffers: the
pinned host mosaic is uploaded, developed and the rgba f16 result read back
inside the timed region of every step.

err:   the benchmarked image's llap output against the FP32 oracle and the
FP64 build of the same restatement (full image), computed after the timed
region in a child process, so the timed process never maps the oracle.
batch: the mixed-size batch (64 mosaics of 4000x3000 .. 9504x6336) through the
develop server beside the plain per-image path, with p50/p99 latency.

--impl reference: the reference's own shaders compiled for the CPU (or, where
that build is missing, the oracle, a C++ restatement of them), all host
threads, one develop of the full 6000x4000 mosaic per step. That process loads
no library of this package: its mosaic comes from the oracle's copy of the
scene recipe.
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
DEMOSAIC = 0          # demosaic method: 0 gaussian splats (the raw photo default), 1 rcd, 2 half size
FILTERS = 0x94949494  # bayer rggb; 9: x-trans
DEMOSAIC_NAMES = {0: "gaussian splats (method 0)", 1: "rcd (method 1)", 2: "half size (method 2)"}
GRAPH = "darkroom"    # darkroom: bin/default-darkroom.i-raw's chain (crop, grade); chain: without them
# grade/params defaults (the llap output graded as the darkroom cfg leaves it)
GRADE_DEFAULTS = ((0, 0, 0, 0), (1, 1, 1, 0), (1, 1, 1, 0), (0, 0, 0, 0), 0, 0.3, 0.4)
# the synthetic camera's matrix to rec2020 (rows sum to one), as the package's default image parameters
CAM_TO_REC2020 = (1.20, -0.15, -0.05, -0.10, 1.25, -0.15, 0.02, -0.22, 1.20)
# the sources of the fused develop kernel: the DRAM traffic of an ncu capture is reported only
# while they are the ones that capture measured (profiles/traffic.json holds their hash)
K_DEVELOP_SOURCES = ["k_develop.cu", "common.cuh", "hilite.cuh", "pixel.cuh", "develop_px.cuh", "gauss.cuh", "kernels.h"]


def source_hash(files):
    import hashlib
    h = hashlib.sha256()
    for f in files:
        with open(os.path.join(ROOT, "vkdt_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def over_ranks(x, op="max"):
    """x reduced over the ranks of the job (a no-op without torch.distributed): the slowest
    rank's time ("max") or the sum of the ranks' work ("sum"). The tensor lives where the
    backend wants it (nccl: the rank's GPU, gloo: the host)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def replica_rate(units, seconds):
    """whole-job throughput of independent replicas: every rank's units over the slowest rank's time"""
    return over_ranks(units, "sum") / over_ranks(seconds, "max")


def img_param(v, wd, ht):
    rng = WHITE - BLACK
    return v.default_img_param(black=BLACK, white=WHITE, wd=wd, ht=ht, filters=FILTERS,
                               noise_a=NOISE_A / rng ** 2, noise_b=NOISE_B / rng)


def graph_cfg(v):
    return v.DARKROOM_FULL_CFG if GRAPH == "darkroom" else v.DARKROOM_CFG


def graph_name():
    dn = "denoise(%s)" % ("wavelet" if DENOISE > 0 else "noop")
    if GRAPH == "darkroom":
        return dn + "->hilite->demosaic->crop->colour->filmcurv->llap->grade (bin/default-darkroom.i-raw)"
    return dn + "->hilite->demosaic->colour->filmcurv->llap"


def config():
    mp = WD * HT / 1e6
    return {"workload": "%s MP %s graph, one image per step%s" % ("%d" % round(mp) if mp >= 10 else "%.2g" % mp,
                                                               "full darkroom" if GRAPH == "darkroom" else "plain chain",
                                                               ", wavelet denoise" if DENOISE > 0 else ""),
            "wd": WD, "ht": HT, "cfa": "x-trans" if FILTERS == 9 else "rggb", "denoise_strength": DENOISE,
            "bits": 14, "black": BLACK, "white": WHITE, "noise_a_dn": NOISE_A, "noise_b_dn": NOISE_B,
            "llap_levels": LEVELS,
            "graph": graph_name(),
            "demosaic": DEMOSAIC_NAMES[DEMOSAIC],
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


def oracle_img_param(oracle, wd, ht):
    """the workload's image parameters as the oracle's struct (no package import)"""
    ip = oracle.ImgParam()
    rng = WHITE - BLACK
    for k in range(4):
        ip.black[k], ip.white[k] = BLACK, WHITE
    for k, w in enumerate((2.0, 1.0, 1.6, 1.0)):
        ip.whitebalance[k] = w
    ip.filters = FILTERS
    ip.crop_aabb[0], ip.crop_aabb[1], ip.crop_aabb[2], ip.crop_aabb[3] = 0, 0, wd, ht
    for i in range(9):
        ip.cam_to_rec2020[i] = CAM_TO_REC2020[i]
    ip.noise_a, ip.noise_b = NOISE_A / rng ** 2, NOISE_B / rng
    return ip


def oracle_params(oracle, wd=None, ht=None):
    p = oracle.default_params()
    p.ll_levels = LEVELS
    p.dn_strength = DENOISE
    p.dm_method = DEMOSAIC
    if GRAPH == "darkroom":   # crop/main.c's commit at its defaults for the demosaic output
        blk, cw, ch = oracle.crop_commit(wd or WD, ht or HT)
        oracle.set_crop(p, blk, cw, ch)
    return p


def oracle_sink(oracle, m, ip, p, double=False, force=None):
    """the graph's output on the oracle: the llap output, graded with grade's defaults
    (stored as f16) on the full darkroom graph; force: decisions taken in place of its own"""
    out = oracle.develop(m, ip, params=p, double=double, stages=("llap",), force=force)["llap"]
    if GRAPH == "darkroom":
        out = oracle.grade(out, *GRADE_DEFAULTS).astype(np.float16).astype(np.float32)
    return out


def reference_sink(glsl_ref, m, ip, p):
    """the same on the reference's shaders compiled for the CPU (grade/main.comp for the grade)"""
    out = glsl_ref.develop(m, ip, params=p)["llap"]
    if GRAPH == "darkroom":
        lift, gamma, gain, off, mode, sp, hp = GRADE_DEFAULTS
        h, w = out.shape[:2]
        src, dst = glsl_ref.Img(w, h, 4), glsl_ref.Img(w, h, 4)
        src.a[...] = out
        glsl_ref.run("grade_main", w, h, {0: src, 1: dst},
                     uniform=glsl_ref.f32(*lift, *gamma, *gain, *off) + glsl_ref.i32(mode) + glsl_ref.f32(sp, hp))
        out = dst.a
    return out


def cpu_leg(args):
    """Child process of the GPU arm (after its timed region): the error of the benchmarked image
    against the oracle (FP32) and the FP64 build, and the oracle's own throughput on the same
    workload (cpu_baseline). Reads the mosaic and the GPU result from args.cpu_leg."""
    import oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from metrics import delta_e2000
    m = np.load(os.path.join(args.cpu_leg, "mosaic.npy"))
    out = np.load(os.path.join(args.cpu_leg, "out.npy")).astype(np.float32)
    ht, wd = m.shape
    ip = oracle_img_param(oracle, wd, ht)
    p = oracle_params(oracle, wd, ht)
    res = {}

    def err(ref):
        e = np.abs(out[..., :3].astype(np.float64) - ref[..., :3]) / np.maximum(1.0, np.abs(ref[..., :3]))
        e = e.max(axis=-1)
        de = delta_e2000(out, ref)
        return {"max": float(e.max()), "mean": float(e.mean()), "px_over_2e-3": int((e > 2e-3).sum()),
                "de2000_max": float(de.max()), "px_de_over_0.5": int((de >= 0.5).sum())}
    dec = {}
    for kind in oracle.DECISION_KINDS:
        f = os.path.join(args.cpu_leg, "dec_%s.npy" % kind)
        if os.path.exists(f):
            dec[kind] = np.load(f)
    res["err"] = {"stage": "the graph's output (%s), rgb, |a-b|/max(1,|b|)" % ("grade" if GRAPH == "darkroom" else "llap"),
                  "window": "full %dx%d" % (out.shape[1], out.shape[0]),
                  "vs_oracle_fp32": err(oracle_sink(oracle, m, ip, p)),
                  "vs_fp64": err(oracle_sink(oracle, m, ip, p, double=True)),
                  "tolerance": {"max": 2e-3, "mean": 1e-4, "de2000": 0.5,
                                "note": "pixels over 2e-3 are where a branch of the reference was a near tie "
                                        "(tests/parity.py shows each such decision explained)"}}
    if dec:
        own = oracle.develop(m, ip, params=p, stages=("llap",), record=True)
        res["err"]["decisions_differing"] = {k: int((dec[k] != own["dec_" + k]).sum()) for k in dec}
        res["err"]["vs_oracle_fp32_same_decisions"] = err(oracle_sink(oracle, m, ip, p, force=dec))
    if not args.no_cpu:
        run = lambda: oracle_sink(oracle, m, ip, p)
        run()
        t0 = time.perf_counter()
        n = 0
        while n < 1 or time.perf_counter() - t0 < args.cpu_seconds:
            run()
            n += 1
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": n * wd * ht / 1e6 / dt, "unit": "MP/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": "%d develops of the %dx%d workload mosaic (%.1f s), "
                               "the FP32 oracle on all host threads" % (n, wd, ht, dt)}
    print(json.dumps(res))


def run_reference(args):
    """The reference's CPU implementation of the path on the GPU arm's workload: one develop of
    the full mosaic per step, all host threads; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    kind, run = "port", None
    m = oracle.scene(WD, HT, seed=0, image_id=0, filters=FILTERS, black=BLACK, white=WHITE, a=NOISE_A, b=NOISE_B)
    ip = oracle_img_param(oracle, WD, HT)
    p = oracle_params(oracle)
    try:
        from oracle import glsl_ref
        if glsl_ref.build():
            run = lambda: reference_sink(glsl_ref, m, ip, p)
            kind = "reference"
    except Exception:
        run = None
    if run is None:
        run = lambda: oracle_sink(oracle, m, ip, p)
    t0 = time.perf_counter()
    run()                                   # first warm-up step: also sizes the run
    t_one = time.perf_counter() - t0
    for _ in range(max(0, min(args.warmup, 2) - 1)):
        run()
    steps = args.steps
    # each step develops the full mosaic; where K of them would take more than about three
    # minutes, each step develops fewer of its rows (a band of the same workload) and says so
    rows = HT
    if steps * t_one > 180.0:
        rows = max(64, int(HT * 180.0 / (steps * t_one)) // 2 * 2)
        mb = np.ascontiguousarray(m[:rows])
        ipb = oracle_img_param(oracle, WD, rows)
        pb = oracle_params(oracle, WD, rows)
        run = (lambda: reference_sink(glsl_ref, mb, ipb, pb)) if kind == "reference" else \
              (lambda: oracle_sink(oracle, mb, ipb, pb))
        run()
    t0 = time.perf_counter()
    for _ in range(steps):
        run()
    dt = time.perf_counter() - t0
    value = steps * WD * rows / 1e6 / dt
    sample = "%d develops of the %dx%d workload mosaic (%.1f s)" % (steps, WD, rows, dt)
    cfg = config()
    if rows != HT:
        cfg["workload"] += "; reference arm: each step a %dx%d band of the mosaic" % (WD, rows)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "MP/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": dt / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "MP/s", "cores": os.cpu_count(), "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "MP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------- served / batched workloads
# The mixed-size batch, the Poisson request stream and the video + x-trans mix
# run through the develop server (vkdt_cuda_server_*): jobs admitted as slots
# and device memory free up, overlapping on the device. Each reports the
# server's MP/s beside the plain per-image path (one develop at a time, same
# jobs) and p50/p99 latency. Inputs are seeded synthetic mosaics generated
# on the device; outputs stay on the device (value) unless stated.

MIX_SIZES = [(4000, 3000), (6000, 4000), (8256, 5504), (9504, 6336)]


def _mixed_images(v, torch, n, seed, sp, rank=0):
    """n mosaics of the mixed sizes with per image noise and white balance (seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        wd, ht = MIX_SIZES[int(rng.integers(len(MIX_SIZES)))]
        a, b = float(rng.uniform(1, 16)), float(rng.uniform(0.2, 3))
        wb = (float(rng.uniform(1.5, 2.5)), 1.0, float(rng.uniform(1.2, 2.0)))
        src = torch.empty(wd * ht, dtype=torch.int16, device="cuda")
        v.scene_device(v.make_scene(wd, ht, seed=seed * 1000 + i + 100000 * rank, image_id=i, a=a, b=b, wb=wb),
                       src.data_ptr(), sp)
        rng_dn = WHITE - BLACK
        ip = v.default_img_param(black=BLACK, white=WHITE, wb=wb, wd=wd, ht=ht, noise_a=a / rng_dn ** 2,
                                 noise_b=b / rng_dn)
        out.append((wd, ht, ip, src))
    return out


def _per_image(v, torch, imgs, dsts, graphs, outsz=None):
    """The plain per-image path: one develop at a time on a graph of the image's shape."""
    for k, (wd, ht, ip, src) in enumerate(imgs):
        ow, oh = outsz[k] if outsz else (0, 0)
        key = (wd, ht, ow, oh, ip.filters)
        g = graphs.get(key)
        if g is None:
            g = v.Graph()
            g.set_input(wd, ht, ip)
            if LEVELS:
                g.set_llap_levels(LEVELS)
            if ow:
                g.set_output_size(ow, oh)
            if DEMOSAIC:
                g.set_param("demosaic", "method", np.int32(DEMOSAIC))
            g.alloc()
            graphs[key] = g
        g.set_input(wd, ht, ip)
        g.develop(src.data_ptr(), dsts[k].data_ptr())
        g.wait()


def _server(v, slots, method=None):
    """A develop server on the darkroom graph with the given demosaic method."""
    method = DEMOSAIC if method is None else method
    cfg = v.DARKROOM_CFG + ("param:demosaic:01:method:%d\n" % method if method else "")
    return v.Server(slots=slots, llap_levels=LEVELS, hbm_cap=int(120e9), cfg=cfg)


def _served(v, s, imgs, dsts, outsz=None):
    ids = []
    for k, (wd, ht, ip, src) in enumerate(imgs):
        ow, oh = outsz[k] if outsz else (0, 0)
        ids.append(s.submit(src.data_ptr(), dsts[k].data_ptr(), wd, ht, ip, ow, oh))
    s.drain()
    return ids


def _timed(torch, fn):
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1), time.perf_counter() - t0, r


def workload_batch(args, v, torch, sp, clk):
    """64 mixed-size mosaics (4000x3000 .. 9504x6336), per image noise and white balance."""
    n = args.images
    imgs = _mixed_images(v, torch, n, 2, sp)
    torch.cuda.synchronize()
    dsts = [torch.empty(wd * ht * 4, dtype=torch.float16, device="cuda") for wd, ht, _, _ in imgs]
    mp = sum(wd * ht for wd, ht, _, _ in imgs) / 1e6
    # plain per-image path: a warm pass (graphs per shape), then timed
    graphs = {}
    _per_image(v, torch, imgs, dsts, graphs)
    ms_pi, _, _ = _timed(torch, lambda: _per_image(v, torch, imgs, dsts, graphs))
    for g in graphs.values():
        g.close()
    # served: the autotuner times the whole batch at each slot count (after a warm
    # pass that fills the pool of graphs) and keeps the fastest
    tune = {}
    best, best_mps = None, 0.0
    for slots in (1, 2, 3, 4, 6):
        s = _server(v, slots)
        _served(v, s, imgs, dsts)
        ms, _, _ = _timed(torch, lambda: _served(v, s, imgs, dsts))
        mps = mp / (ms / 1e3)
        tune[slots] = round(mps, 1)
        s.close()
        if mps > best_mps:
            best, best_mps = slots, mps
    s = _server(v, best)
    _served(v, s, imgs, dsts)
    s.reset_stats()
    with clk:
        ms_b, _, _ = _timed(torch, lambda: _served(v, s, imgs, dsts))
    st = s.stats()
    # e2e: the first 16 images with pinned host buffers in and out, through the same server
    hin = [torch.empty(wd * ht, dtype=torch.int16, pin_memory=True) for wd, ht, _, _ in imgs[:16]]
    hout = [torch.empty(wd * ht * 4, dtype=torch.float16, pin_memory=True) for wd, ht, _, _ in imgs[:16]]
    for h, (_, _, _, src) in zip(hin, imgs[:16]):
        h.copy_(src.cpu())

    def e2e_run():
        ids = [s.submit(hin[k].data_ptr(), hout[k].data_ptr(), wd, ht, ip, src_on_device=False, dst_on_device=False)
               for k, (wd, ht, ip, _) in enumerate(imgs[:16])]
        s.drain()
        return ids
    ms_e, _, _ = _timed(torch, e2e_run)
    mp16 = sum(wd * ht for wd, ht, _, _ in imgs[:16]) / 1e6
    s.close()
    value = mp / (ms_b / 1e3)
    return {"workload": "64 mixed-size mosaics (4000x3000, 6000x4000, 8256x5504, 9504x6336), per image noise "
                        "a~U[1,16] b~U[0.2,3] and white balance, one batch per step", "images": n, "mpix": round(mp, 1)}, \
        value, ms_b, {
            "per_image": {"value": mp / (ms_pi / 1e3), "unit": "MP/s", "ms": ms_pi},
            "served_over_per_image": value / (mp / (ms_pi / 1e3)),
            "autotune": {"slots": best, "candidates_mps": tune},
            "latency_ms": {"p50": st["latency_p50_ms"], "p99": st["latency_p99_ms"],
                           "note": "submit to done; all 64 jobs are submitted at once"},
            "peak_device_bytes": st["peak_device_bytes"],
            "e2e": {"value": mp16 / (ms_e / 1e3), "unit": "MP/s", "h2d_bytes_per_step": int(mp16 * 2e6),
                    "d2h_bytes_per_step": int(mp16 * 8e6), "images": 16}}


def _request_trace(duration, rate, seed):
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            return out
        size = int(rng.integers(len(MIX_SIZES)))
        thumb = bool(rng.uniform() < 0.3)
        out.append((t, size, thumb))


def _replay(v, s, trace, pool, outs):
    """submit each request at its arrival time; returns (first submit, last done) host times"""
    nxt = {}
    t0 = time.perf_counter()
    for t, size, thumb in trace:
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        wd, ht, ip, src = pool[size][len(nxt) % len(pool[size])]
        key = (size, thumb)
        ring = outs[key]
        k = nxt.get(key, 0)
        nxt[key] = k + 1
        ow, oh = (wd // 8, ht // 8) if thumb else (0, 0)
        s.submit(src.data_ptr(), ring[k % len(ring)].data_ptr(), wd, ht, ip, ow, oh)
    s.drain(timeout_ms=600000)
    return t0, time.perf_counter()


def workload_serve(args, v, torch, sp, clk):
    """Poisson arrivals (200 requests/s, the configuration's rate, or --rate): 70% full size, 30% 1/8
    thumbnails, admission capped at 120 GB. Above one GPU's capacity (about 1 000/s) both forms fall
    behind and their MP/s is what they develop, not the offered rate."""
    trace = _request_trace(args.duration, args.rate, 3)
    pool = {}
    for i, (wd, ht) in enumerate(MIX_SIZES):
        # two resident mosaics per size, each with its own noise and white balance
        rng = np.random.default_rng(20 + i)
        pool[i] = []
        for k in range(2):
            a, b = float(rng.uniform(1, 16)), float(rng.uniform(0.2, 3))
            wb = (float(rng.uniform(1.5, 2.5)), 1.0, float(rng.uniform(1.2, 2.0)))
            src = torch.empty(wd * ht, dtype=torch.int16, device="cuda")
            v.scene_device(v.make_scene(wd, ht, seed=500 + 10 * i + k, a=a, b=b, wb=wb), src.data_ptr(), sp)
            ip = v.default_img_param(black=BLACK, white=WHITE, wb=wb, wd=wd, ht=ht,
                                     noise_a=a / (WHITE - BLACK) ** 2, noise_b=b / (WHITE - BLACK))
            pool[i].append((wd, ht, ip, src))
    outs = {}
    for i, (wd, ht) in enumerate(MIX_SIZES):
        outs[(i, False)] = [torch.empty(wd * ht * 4, dtype=torch.float16, device="cuda") for _ in range(32)]
        outs[(i, True)] = [torch.empty((wd // 8) * (ht // 8) * 4, dtype=torch.float16, device="cuda") for _ in range(32)]
    torch.cuda.synchronize()
    mp = sum(MIX_SIZES[sz][0] * MIX_SIZES[sz][1] for _, sz, _ in trace) / 1e6
    res = {}
    for name, slots in (("per_image", 1), ("served", args.slots)):
        s = _server(v, slots)
        _replay(v, s, _request_trace(2.0, 50.0, 4), pool, outs)      # warm the pool of graphs
        s.reset_stats()
        if name == "served":
            with clk:
                t0, t1 = _replay(v, s, trace, pool, outs)
        else:
            t0, t1 = _replay(v, s, trace, pool, outs)
        st = s.stats()
        res[name] = {"value": mp / (t1 - t0), "unit": "MP/s", "wall_s": t1 - t0, "completed": st["completed"],
                     "failed": st["failed"], "p50_ms": st["latency_p50_ms"], "p99_ms": st["latency_p99_ms"],
                     "peak_device_bytes": st["peak_device_bytes"], "slots": slots}
        s.close()
    return {"workload": "served request stream: Poisson arrivals %g/s for %g s (%d requests), 70%% full size "
                        "(sizes of the mixed batch), 30%% 1/8 thumbnails, HBM admission cap 120 GB"
                        % (args.rate, args.duration, len(trace)),
            "requests": len(trace), "offered_mpix_per_s": mp / args.duration}, \
        res["served"]["value"], res["served"]["wall_s"] * 1e3, {
            "per_image": res["per_image"], "served": res["served"],
            "latency_ms": {"p50": res["served"]["p50_ms"], "p99": res["served"]["p99_ms"]}}


def _video_host_e2e(v, torch, W, H, ip, method, packed, frames=96):
    """Four video streams from host memory to host memory: each frame crosses to the device as u16
    samples (uploaded from the graph's pinned source) or as the packed 12-bit magic lantern frame
    (copied from pinned memory, unpacked on the device into the graph's source), is developed and
    read back as rgba f16. One graph and stream per video stream, frames pipelined across streams.
    The samples are random 12-bit values (the same distribution both ways)."""
    R = 4
    g = torch.Generator(device="cpu")
    g.manual_seed(3)
    nb = W * H * 12 // 8
    graphs, streams, hp, dp = [], [], [], []
    for k in range(R):
        gr = v.Graph()
        gr.set_input(W, H, ip)
        if LEVELS:
            gr.set_llap_levels(LEVELS)
        if method:
            gr.set_param("demosaic", "method", np.int32(method))
        gr.alloc()
        graphs.append(gr)
        streams.append(torch.cuda.Stream())
        if packed:
            hp.append(torch.randint(0, 256, (nb,), dtype=torch.uint8, generator=g).pin_memory())
            dp.append(torch.empty(nb, dtype=torch.uint8, device="cuda"))
        else:
            gr.source()[...] = torch.randint(0, 4096, (H, W), dtype=torch.int16, generator=g).numpy()

    def frame(k):
        gr, st = graphs[k % R], streams[k % R]
        if packed:
            src, _ = gr.device_buffers()
            with torch.cuda.stream(st):
                dp[k % R].copy_(hp[k % R], non_blocking=True)
            v.unpack_mlv(dp[k % R].data_ptr(), nb, 12, W, H, src, st.cuda_stream)
            gr.run(flags=v.RUN_DOWNLOAD_SINK, stream=st.cuda_stream)
        else:
            gr.run(flags=v.RUN_UPLOAD_SOURCE | v.RUN_DOWNLOAD_SINK, stream=st.cuda_stream)
    for k in range(2 * R):
        if k >= R:
            graphs[k % R].wait()
        frame(k)
    for gr in graphs:
        gr.wait()
    t0 = time.perf_counter()
    for k in range(frames):
        if k >= R:
            graphs[k % R].wait()
        frame(k)
    for gr in graphs:
        gr.wait()
    wall = time.perf_counter() - t0
    for gr in graphs:
        gr.close()
    return {"value": frames * W * H / 1e6 / wall, "unit": "MP/s", "frames": frames,
            "h2d_bytes_per_frame": nb if packed else 2 * W * H, "d2h_bytes_per_frame": 8 * W * H}


def workload_video(args, v, torch, sp, clk):
    """4 raw video streams 4096x2160 RGGB 12-bit, 120 panned frames each, and x-trans 6240x4160 stills at 5/s."""
    VW, VH, XW, XH = 4096, 2160, 6240, 4160
    frames = []
    for st_i in range(4):
        fr = []
        for f in range(120):
            src = torch.empty(VW * VH, dtype=torch.int16, device="cuda")
            v.scene_device(v.make_scene(VW, VH, seed=900 + st_i, image_id=f, black=256.0, white=4095.0, a=4.0, b=0.8,
                                        pan=(3.0 * f, 0.0)), src.data_ptr(), sp)
            fr.append(src)
        frames.append(fr)
    vip = v.default_img_param(black=256.0, white=4095.0, wd=VW, ht=VH, noise_a=4.0 / (4095 - 256) ** 2,
                              noise_b=0.8 / (4095 - 256))
    stills = []
    for k in range(2):
        src = torch.empty(XW * XH, dtype=torch.int16, device="cuda")
        v.scene_device(v.make_scene(XW, XH, seed=950 + k, filters=9, a=8.0, b=1.6), src.data_ptr(), sp)
        stills.append(src)
    xip = v.default_img_param(wd=XW, ht=XH, filters=9, noise_a=8.0 / (16383 - 512) ** 2, noise_b=1.6 / (16383 - 512))
    vout = [[torch.empty(VW * VH * 4, dtype=torch.float16, device="cuda") for _ in range(4)] for _ in range(4)]
    xout = [torch.empty(XW * XH * 4, dtype=torch.float16, device="cuda") for _ in range(4)]
    torch.cuda.synchronize()
    # the raw video graphs' demosaic is rcd (bin/default-darkroom.i-mcraw: param:demosaic:01:method:1),
    # the stills' the raw photo default; one server per graph configuration
    vmethod = args.demosaic if args.demosaic >= 0 else 1
    s = _server(v, args.slots, vmethod)
    sx = _server(v, args.slots, 0) if vmethod else s

    def run(paced):
        vid, xid = [], []
        t0 = time.perf_counter()
        nst = 0
        for f in range(120):
            if paced:
                now = time.perf_counter() - t0
                if f / 24.0 > now:
                    time.sleep(f / 24.0 - now)
            while nst < 25 and nst / 5.0 <= (time.perf_counter() - t0 if paced else f / 24.0):
                xid.append(sx.submit(stills[nst % 2].data_ptr(), xout[nst % 4].data_ptr(), XW, XH, xip))
                nst += 1
            ids = [s.submit(frames[k][f].data_ptr(), vout[k][f % 4].data_ptr(), VW, VH, vip) for k in range(4)]
            vid += ids
            if not paced:                 # back to back: the next frame of each stream after this one
                for j in ids:
                    s.wait(j)
        while nst < 25:
            xid.append(sx.submit(stills[nst % 2].data_ptr(), xout[nst % 4].data_ptr(), XW, XH, xip))
            nst += 1
        s.drain()
        sx.drain()
        t1 = time.perf_counter()
        lv = sorted(s.job_times(j)[1] for j in vid)
        lx = sorted(sx.job_times(j)[1] for j in xid)
        mp = (len(vid) * VW * VH + len(xid) * XW * XH) / 1e6
        pct = lambda l, q: l[min(len(l) - 1, max(0, int(np.ceil(q * len(l))) - 1))]
        return {"value": mp / (t1 - t0), "unit": "MP/s", "wall_s": t1 - t0,
                "frame_latency_ms": {"p50": pct(lv, 0.5), "p99": pct(lv, 0.99)},
                "still_latency_ms": {"p50": pct(lx, 0.5), "p99": pct(lx, 0.99)}}
    run(False)                               # warm the pool
    s.reset_stats()
    sx.reset_stats()
    with clk:
        b2b = run(False)
    paced = run(True)
    s.close()
    if sx is not s:
        sx.close()
    del frames, stills, vout, xout
    torch.cuda.synchronize()
    host = {"u16": _video_host_e2e(v, torch, VW, VH, vip, vmethod, packed=False),
            "mlv_12bit": _video_host_e2e(v, torch, VW, VH, vip, vmethod, packed=True)}
    return {"workload": "4 raw video streams 4096x2160 RGGB 12-bit (black 256, white 4095, a=4, b=0.8, panned 3 px/frame, "
                        "120 frames each) and 25 x-trans 6240x4160 14-bit stills at 5/s",
            "demosaic": "video: %s, stills: %s" % (DEMOSAIC_NAMES[vmethod], DEMOSAIC_NAMES[0]),
            "modes": "back-to-back (each stream's next frame after its last) and paced at 24 fps"}, \
        b2b["value"], b2b["wall_s"] * 1e3, {"back_to_back": b2b, "paced_24fps": paced, "e2e_from_host": host,
                                             "latency_ms": {"p99_frame": b2b["frame_latency_ms"]["p99"]}}


def workload_ingest(args, v, torch, sp, clk):
    """Device ingestion of packed raw video, 4096x2160 frames: the magic lantern unpack at
    12 and 14 bits and the motioncam block decode (bit counts 5..8 per block, as 12-bit video
    noise gives them), each over a ring of frames larger than L2."""
    W, H, N, K = 4096, 2160, 16, 64
    npx = W * H
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    outs = [torch.empty(npx, dtype=torch.int16, device="cuda") for _ in range(N)]
    res = {}

    def timed(launch, nbytes):
        for i in range(4):
            launch(i % N)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(K):
            launch(i % N)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / K
        gbs = nbytes / (ms / 1e3) / 1e9
        return {"ms_per_frame": ms, "mpix_per_s": npx / 1e6 / (ms / 1e3), "gbs": gbs, "hbm_frac": gbs / peak,
                "bytes_per_frame": nbytes}
    with clk:
        for bpp in (12, 14):
            nb = npx * bpp // 8
            ins = [torch.randint(0, 256, (nb,), dtype=torch.uint8, device="cuda", generator=g) for _ in range(N)]
            res["mlv_%dbit" % bpp] = timed(lambda i: v.unpack_mlv(ins[i].data_ptr(), nb, bpp, W, H, outs[i].data_ptr(), sp),
                                           nb + 2 * npx)
            del ins
        blocks = npx // 64
        rng = np.random.default_rng(5)
        streams = []
        for i in range(N):
            nib = rng.integers(5, 9, blocks).astype(np.uint8)
            bc = (nib[0::2] | (nib[1::2] << 4)).astype(np.uint8)
            size = int(np.where(nib <= 6, 8 * nib.astype(np.int64), 64).sum())
            streams.append((torch.from_numpy(bc).cuda(), torch.randint(0, 2000, (blocks,), dtype=torch.int16, device="cuda",
                                                                        generator=g),
                            torch.randint(0, 256, (size,), dtype=torch.uint8, device="cuda", generator=g), size))
        scratch = torch.empty(max(8, v._lib.lib().vkdt_cuda_mcraw_scratch_bytes(W, H)), dtype=torch.uint8, device="cuda")
        mean_bytes = sum(st[3] for st in streams) / N + blocks // 2 + 2 * blocks
        res["mcraw"] = timed(lambda i: v.mcraw_decode(streams[i][0].data_ptr(), streams[i][1].data_ptr(),
                                                      streams[i][2].data_ptr(), streams[i][3], W, H, outs[i].data_ptr(),
                                                      d_scratch=scratch.data_ptr(), stream=sp),
                             mean_bytes + 2 * npx)
        del streams
        # the output side at the same size: colenc of an rgba f16 frame to sRGB u8, BC1 of the u8 frame
        f16 = [torch.rand(npx * 4, device="cuda", generator=g).half() for _ in range(N // 2)]
        u8 = [torch.randint(0, 1 << 30, (npx,), dtype=torch.int32, device="cuda", generator=g) for _ in range(N // 2)]
        bc = [torch.empty(npx // 2, dtype=torch.uint8, device="cuda") for _ in range(N // 2)]
        res["colenc_u8"] = timed(lambda i: v.colenc(f16[i % (N // 2)].data_ptr(), W, H, 2, 2, 0, u8[i % (N // 2)].data_ptr(), sp),
                                 npx * (8 + 4))
        res["bc1"] = timed(lambda i: v.bc1_encode(u8[i % (N // 2)].data_ptr(), W, H, bc[i % (N // 2)].data_ptr(), sp),
                           npx * 4 + npx // 2)
    return {"workload": "device ingestion of packed raw video frames, 4096x2160: magic lantern 12/14-bit unpack, "
                        "motioncam block decode (bit counts 5..8); and the output encode of such a frame: colenc "
                        "to sRGB u8, BC1", "frames_in_ring": N,
            "roofline_note": "gbs counts the packed bytes read and the u16 mosaic written once per frame"}, \
        res["mcraw"]["mpix_per_s"], res["mcraw"]["ms_per_frame"], {"ingest": res, "gpu_launches": 5 * K}


def run_workload(args):
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
    sp = torch.cuda.current_stream().cuda_stream
    clk = Clocks(local)
    fn = {"batch": workload_batch, "serve": workload_serve, "video": workload_video,
          "ingest": workload_ingest}[args.workload]
    cfg, value, ms, extra = fn(args, v, torch, sp, clk)
    value = over_ranks(value, "sum")   # replicas: whole-job MP/s
    if rank == 0:
        cfg.update({"llap_levels": LEVELS, "graph": "denoise(noop)->hilite->demosaic->colour->filmcurv->llap",
                    "l2": "inputs of 12 MP and more per image (> 129 MB L2 in flight)"})
        line = {"metric": METRIC, "value": value, "unit": "MP/s", "n_gpus": world, "steps": 1, "warmup": 1,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": cfg, "clocks": clk.summary()}
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()

def main():
    global WD, HT, RING, LEVELS, DENOISE, DEMOSAIC, FILTERS, GRAPH
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="cuda")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-err", action="store_true", help="skip the error against the oracle and FP64 build")
    ap.add_argument("--no-batch", action="store_true", help="skip the mixed-size batch sub-object")
    ap.add_argument("--cpu-leg", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help=argparse.SUPPRESS)
    ap.add_argument("--size", default="%dx%d" % (WD, HT), help="WxH of the mosaic (profiling of smaller cases)")
    ap.add_argument("--ring", type=int, default=RING, help="number of resident inputs")
    ap.add_argument("--levels", type=int, default=LEVELS, help="llap pyramid depth (0 = automatic)")
    ap.add_argument("--denoise", type=float, default=DENOISE,
                    help="denoise strength (0 = the darkroom default, denoise/noop; > 0 the wavelet path)")
    ap.add_argument("--workload", default="single", choices=("single", "batch", "serve", "video", "ingest"),
                    help="single: the 24 MP develop (default); batch: 64 mixed-size mosaics; "
                         "serve: Poisson request stream; video: 4 raw video streams + x-trans stills; "
                         "ingest: device unpack/decode of packed raw video frames")
    ap.add_argument("--images", type=int, default=64, help="batch: mosaics in the batch")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: requests per second (Poisson)")
    ap.add_argument("--slots", type=int, default=4, help="serve/video: jobs in flight")
    ap.add_argument("--cfa", default="rggb", choices=("rggb", "xtrans"), help="single: the mosaic's colour filter array")
    ap.add_argument("--graph", default=GRAPH, choices=("darkroom", "chain"),
                    help="single: darkroom (bin/default-darkroom.i-raw's chain with crop and grade) or chain "
                         "(denoise .. llap only)")
    ap.add_argument("--demosaic", type=int, default=-1, choices=(-1, 0, 1, 2),
                    help="demosaic method (-1: the workload's default: 0 for photos, 1 for the video streams)")
    args = ap.parse_args()
    WD, HT = [int(x) for x in args.size.lower().split("x")]
    RING, LEVELS, DENOISE = args.ring, args.levels, args.denoise
    DEMOSAIC = max(0, args.demosaic)
    FILTERS = 9 if args.cfa == "xtrans" else 0x94949494
    GRAPH = args.graph
    if args.cpu_leg:
        return cpu_leg(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "single":
        return run_workload(args)

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
        g = v.Graph(graph_cfg(v))
        g.set_input(WD, HT, img_param(v, WD, HT))
        if LEVELS:
            g.set_llap_levels(LEVELS)
        if DENOISE > 0:
            g.set_param("denoise", "strength", DENOISE)
        if DEMOSAIC:
            g.set_param("demosaic", "method", np.int32(DEMOSAIC))
        g.alloc()
        src, _ = g.device_buffers()
        v.scene_device(v.make_scene(WD, HT, seed=1000 * rank + i, image_id=i, a=NOISE_A, b=NOISE_B, filters=FILTERS), src, sp)
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
    ms_rank = ev0.elapsed_time(ev1)
    mp_step = WD * HT / 1e6
    value = replica_rate(args.steps * mp_step, ms_rank / 1e3)   # every rank's megapixels over the slowest rank
    ms = over_ranks(ms_rank, "max")

    # ---- per kernel durations (events around every launch, one sync per step)
    gt = v.Graph(graph_cfg(v))
    gt.set_input(WD, HT, img_param(v, WD, HT))
    if LEVELS:
        gt.set_llap_levels(LEVELS)
    if DENOISE > 0:
        gt.set_param("denoise", "strength", DENOISE)
    if DEMOSAIC:
        gt.set_param("demosaic", "method", np.int32(DEMOSAIC))
    gt.set_timing(True)
    gt.alloc()
    src, _ = gt.device_buffers()
    v.scene_device(v.make_scene(WD, HT, seed=1000 * rank + 7, a=NOISE_A, b=NOISE_B, filters=FILTERS), src, sp)
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
    # one timed entry per fused launch; the develop entry is two kernels (interior tiles, border ring)
    launches_per_step = len(names) + (1 if "demosaic:fix" in names and FILTERS != 9 and not DEMOSAIC else 0)
    # the dominant kernel: the fused develop kernel where the graph runs it, else the longest launch
    fused = "demosaic:fix" in names and FILTERS != 9 and not DEMOSAIC
    dev_idx = names.index("demosaic:fix") if fused else int(np.argmax(kms))
    dev_ms = float(kms[dev_idx])
    npx, qpx = WD * HT, (WD // 2) * (HT // 2)
    ow, oh = gt.out_wd, gt.out_ht                       # the output size (the crop window)
    opx, oqpx = ow * oh, ((ow + 1) // 2) * ((oh + 1) // 2)
    crop_fused = fused and (ow, oh) != (WD, HT)         # the develop kernel ends at filmcurv
    # algorithmic bytes per launch (each buffer the launch must read or write, once):
    alg_bytes = {
        # fused develop: mosaic in (2 B/px), the hilite coarse level (8 B per (W/4 x H/4) px),
        # filmcurv rgba f16 out (8 B per output px), 11 llap level 1 planes out (11 * 2 B per
        # level 1 px) unless a crop follows demosaic (then the next launch makes them)
        "demosaic:fix": npx * 2 + (WD // 4) * (HT // 4) * 8 + opx * 8 + (0 if crop_fused else 11 * 2 * oqpx),
        # rcd_fill: mosaic, vh, pq + lp (half width) in, rgba f16 out
        "demosaic:rcd_fill": npx * (2 + 2 + 2 + 8),
        # rcd_conv: mosaic in, vh, pq + lp out
        "demosaic:rcd_conv": npx * (2 + 2 + 2),
        # colour .. llap curve + level 1 reduce of the per-node chain: rgba in, rgba out, 11 planes out;
        # after the fused develop kernel with a crop: filmcurv rgba in, 11 planes out
        "llap:curve": (opx * 8 if crop_fused else opx * (8 + 8)) + 11 * 2 * oqpx,
        # llap level 0 assemble + colour (+ grade): rgba, 11 level 1 planes, level 1 assembled in, rgba out
        "llap:colour": opx * (8 + 8) + 11 * 2 * oqpx + 2 * oqpx,
    }
    if not fused:
        alg_bytes.pop("demosaic:fix")
        # the x-trans per-node kernels: fix reads the mosaic, the splat green and the covariance
        # (1/9 size), writes rgba f16; splat reads the mosaic and the covariance, writes the green
        alg_bytes.update({"demosaic:fix": npx * (2 + 2 + 8) + (WD // 3) * (HT // 3) * 8,
                          "demosaic:splat": npx * (2 + 2) + (WD // 3) * (HT // 3) * 8})
    alg = alg_bytes.get(names[dev_idx])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = alg / (dev_ms / 1e3) / 1e9 if alg else None
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    issue = None
    traffic_note = None
    if os.path.exists(tp) and fused:
        try:
            tj = json.load(open(tp))
            if tj.get("k_develop_source_sha") == source_hash(K_DEVELOP_SOURCES) and (WD, HT) == (6000, 4000) \
                    and DENOISE == 0 and tj.get("graph", "chain") == GRAPH:
                traffic = tj.get("k_develop_bytes_per_launch")
                traffic_note = "ncu capture of this kernel source at this size (" + tj.get("source", "") + ")"
                # the kernel is bound by instruction issue, not by HBM: the same capture's issue
                # utilisation and instructions per pixel are reported beside the HBM fraction
                issue = {"issue_active": tj.get("k_develop_issue_active"),
                         "thread_inst_per_px": tj.get("k_develop_thread_inst_per_px"), "source": "ncu capture, profiles/"}
            else:
                traffic_note = "no ncu capture of this kernel source, size and graph"
        except Exception:
            traffic = None
    kname = {"demosaic:fix": ("k_develop (hilite doub + demosaic + crop + colour + filmcurv)" if crop_fused else
                              "k_develop (hilite doub + demosaic + colour + filmcurv + llap curve/reduce)") if fused
             else "k_nd_fix_xt",
             "demosaic:splat": "k_nd_splat_xt",
             "demosaic:rcd_fill": "k_rcd_fill", "demosaic:rcd_conv": "k_rcd_conv",
             "llap:curve": "k_post (colour + filmcurv + llap curve/reduce)",
             "llap:colour": "k_llap_final (llap assemble level 0 + colour)"}.get(names[dev_idx], names[dev_idx])
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None,
                "traffic": traffic, "traffic_source": traffic_note, "kernel": kname, "compute": issue,
                "kernel_ms": dev_ms, "alg_bytes_per_launch": alg,
                "peak_source": "measured" if peaks else "fallback",
                "per_launch_ms": [[n, round(float(x), 5)] for n, x in zip(names, kms)],
                "per_kernel_ms": {n: round(float(sum(x for m, x in zip(names, kms) if m == n)), 5) for n in names}}
    gt.close()

    # ---- e2e: host mosaic in, host rgba f16 out, through the C-ABI run call
    ge = graphs[0]
    host_in = [v.scene_host(v.make_scene(WD, HT, seed=50 + i, a=NOISE_A, b=NOISE_B, filters=FILTERS)) for i in range(2)] if rank == 0 else None
    if host_in is None:
        host_in = [v.scene_host(v.make_scene(WD, HT, seed=50 + i + 100 * rank, a=NOISE_A, b=NOISE_B, filters=FILTERS)) for i in range(2)]
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
    e2e_ms = over_ranks(float(lat.mean()), "max")
    # pipelined: a ring of graphs on their own streams, each holding its image in its pinned source
    # (where a decoder writes it); every step uploads its mosaic, develops and reads the result back,
    # while the next step's copies overlap this one's kernels
    ring = graphs[:min(3, len(graphs))]
    streams = [torch.cuda.Stream() for _ in ring]
    for k, g in enumerate(ring):
        g.source()[...] = host_in[k % 2]
    for k in range(2 * len(ring)):
        ring[k % len(ring)].run(flags=v.RUN_UPLOAD_SOURCE | v.RUN_DOWNLOAD_SINK, stream=streams[k % len(ring)].cuda_stream)
    for g in ring:
        g.wait()
    barrier()
    def pipelined(n):
        barrier()
        t0 = time.perf_counter()
        for k in range(n):
            g = ring[k % len(ring)]
            if k >= len(ring):
                g.wait()
            g.run(flags=v.RUN_UPLOAD_SOURCE | v.RUN_DOWNLOAD_SINK, stream=streams[k % len(ring)].cuda_stream)
        for g in ring:
            g.wait()
        return time.perf_counter() - t0
    # steps per repeat for about 1.2 s of work, then 3 timed repeats; their median
    probe = max(3 * len(ring), 12)
    np_ = max(probe, int(probe * 1.2 / max(pipelined(probe), 1e-3)))
    reps = sorted(replica_rate(np_ * mp_step, pipelined(np_)) for _ in range(3))
    pipe_value = reps[1]
    e2e = {"value": pipe_value, "unit": "MP/s", "h2d_bytes_per_step": WD * HT * 2,
           "d2h_bytes_per_step": ow * oh * 8, "steps": np_, "repeats_mps": [round(x, 1) for x in reps],
           "timing": "median of 3 repeats of %d pipelined steps each (host clock, >= 1 s each)" % np_,
           "graphs_in_flight": len(ring),
           "one_at_a_time": {"value": world * mp_step / (e2e_ms / 1e3), "unit": "MP/s"},
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}}

    # the mixed-size batch (served vs per image) on this GPU
    batch = None
    if not args.no_batch and (WD, HT) == (6000, 4000):
        for g in graphs[1:]:
            g.close()
        graphs = graphs[:1]
        torch.cuda.synchronize()
        bclk = Clocks(local)
        args.images = 64
        bcfg, bvalue, bms, bextra = workload_batch(args, v, torch, sp, bclk)
        batch = {"workload": bcfg["workload"], "mpix": bcfg["mpix"], "value": bvalue, "unit": "MP/s", "ms": bms,
                 "per_image": bextra["per_image"], "served_over_per_image": bextra["served_over_per_image"],
                 "latency_ms": bextra["latency_ms"], "autotune": bextra["autotune"], "clocks": bclk.summary()}

    # the error of the benchmarked image and the CPU baseline, in a child process (the oracle)
    cb, err = None, None
    if rank == 0 and world == 1 and not (args.no_cpu and args.no_err):
        import tempfile
        # graph 0 holds host_in[0] in its pinned source (the e2e runs uploaded it): develop it again
        # and read the result back
        g0 = graphs[0]
        g0.source()[...] = host_in[0]
        out = g0.run(flags=v.RUN_UPLOAD_SOURCE | v.RUN_DOWNLOAD_SINK | v.RUN_WAIT_DONE, stream=sp)
        host_m = np.array(host_in[0], copy=True)
        # the discrete decisions this image's develop took (a graph with the debug stages, whose
        # results equal the plain graph's): the error against the oracle is also reported with the
        # oracle taking the same decisions, which isolates the arithmetic from near-tie branches
        dec = {}
        gd = v.Graph(graph_cfg(v))
        try:
            gd.set_input(WD, HT, img_param(v, WD, HT))
            if LEVELS:
                gd.set_llap_levels(LEVELS)
            if DENOISE > 0:
                gd.set_param("denoise", "strength", DENOISE)
            if DEMOSAIC:
                gd.set_param("demosaic", "method", np.int32(DEMOSAIC))
            gd.set_debug(True)
            gd.alloc()
            gd.run(host_m)
            for kind in ("gauss", "dn_cov", "dn_thr"):
                try:
                    dec[kind] = gd.debug_decisions(kind)
                except v._lib.VkdtError:
                    pass
        finally:
            gd.close()
        with tempfile.TemporaryDirectory() as td:
            np.save(os.path.join(td, "mosaic.npy"), host_m)
            np.save(os.path.join(td, "out.npy"), np.asarray(out))
            for kind, d in dec.items():
                np.save(os.path.join(td, "dec_%s.npy" % kind), d)
            cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-leg", td, "--size", "%dx%d" % (WD, HT),
                   "--graph", GRAPH,
                   "--levels", str(LEVELS), "--denoise", str(DENOISE), "--cfa", "xtrans" if FILTERS == 9 else "rggb",
                   "--demosaic", str(DEMOSAIC)] + (["--no-cpu"] if args.no_cpu else [])
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
            if r.returncode == 0:
                leg = json.loads(r.stdout.strip().splitlines()[-1])
                cb, err = leg.get("cpu_baseline"), leg.get("err")
            else:
                err = {"unavailable": "cpu leg failed: " + r.stderr.strip().splitlines()[-1] if r.stderr.strip() else "?"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "MP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(),
                "roofline": roofline, "cpu_baseline": cb, "e2e": e2e, "err": err, "batch": batch,
                "gpu_launches": launches_per_step * args.steps, "clocks": clk.summary(),
                "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}}
        print(json.dumps(line))
    for g in graphs:
        g.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
