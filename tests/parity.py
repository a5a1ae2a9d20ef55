"""Parity of the CUDA path against the oracle, at the stated tolerance.

The path computes in FP32 and stores f16 where the reference stores an image.
The error of a stage is, per pixel, the largest over r, g, b of
|a - b| / max(1, |b|): the absolute error below 1; above 1 relative, because
f16 storage resolves values relatively (one f16 step of a value above 4 is
more than 2e-3). The tolerance is max 2e-3, mean 1e-4 and CIEDE2000 < 0.5.

1. Discrete decisions. The reference has branches whose inputs come out of
   continuous arithmetic (demosaic/gauss.comp:65,72 the structure tensor form
   and the snapped direction; denoise/cov.glsl:84,130 the form and the hot
   pixel skip; denoise/assemble.comp:144-153 the coarse threshold switch).
   Every decision the CUDA path took that differs from the oracle's own is
   explained: gauss decisions equal the oracle's gauss on the CUDA path's own
   hilite output bit for bit (exact IEEE arithmetic in both); the structure
   tensor choices equal the oracle's (exact arithmetic on the bit identical
   half image); a differing threshold switch is a near tie (| |d| - 10 | / 10
   below DN_THR_TIE in the oracle). The oracle is then run with the CUDA
   path's decisions; the pixels that changes are the flipped pixels.
2. Node-wise, strict: every stage (hilite, demosaic, colour, filmcurv, llap,
   and each node of the wavelet denoise) evaluated by the oracle on the CUDA
   path's own input of that stage meets max 2e-3 and mean 1e-4 at every pixel
   against the CUDA path's output of it. This is the check of the kernels.
3. End to end against the oracle with the same decisions: mean <= 1e-4 at
   every stage. Every pixel meets max 2e-3 (and CIEDE2000 < 0.5 after filmcurv
   and at the llap output), except where the reference's own arithmetic
   amplifies in-tolerance differences of its input:
   - the colour transform is linear: its output can move by the colour
     matrix's gain times the demosaic output's difference plus one f16 step;
     each colour pixel over 2e-3 is checked to be within that bound;
   - after colour (filmcurv, llap) a pixel over the tolerance must come from
     the colour input: the oracle run from colour on to the end on the CUDA
     path's own colour input (each pixel of which meets the tolerance against
     the reference's) meets the tolerance there;
   - on the wavelet denoise path (its detail mask raises the slope of the
     coarse levels to the 16th power) and through rcd (its gradient weights
     are 1 / (1e-5 + |difference|)), the pixels over the tolerance are fewer
     than those by which the same restatement in FP64 differs from FP32: the
     CUDA path is at least as close to the FP32 reference as the reference's
     arithmetic carried in double precision is.
   Against the FP64 build (double=True) the same rules hold, except on those
   ill-conditioned paths: there the FP64 build's own decisions follow values
   the FP32 arithmetic does not reproduce, and the CUDA path is held to be no
   farther from the FP64 result than the FP32 reference is (pixels over the
   tolerance and the mean within 25%).
"""
import json
import os

import numpy as np

import oracle
from metrics import delta_e2000

TOL = 2e-3
MEAN = 1e-4
DE = 0.5
DN_THR_TIE = 0.05   # a differing coarse threshold switch: |d| within 5% of 10 in the oracle


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.ndim == 2:
        a, b = a[..., None], b[..., None]
    e = np.abs(a[..., :3] - b[..., :3]) / np.maximum(1.0, np.abs(b[..., :3]))
    e = np.where(np.isnan(e), np.inf, e)
    return e.max(axis=-1)


def log(name, rec):
    """Print a parity record and append it to $VKDT_PARITY_LOG (json lines)."""
    rec = dict(rec, case=name)
    print("parity", json.dumps(rec, sort_keys=True))
    path = os.environ.get("VKDT_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(rec, sort_keys=True) + "\n")


def develop_gpu(v, m, ip, setup=None, hist=False, cfg=None):
    """Develop through the C-ABI with the debug stages: every stage image and the decisions."""
    g = v.Graph(cfg) if cfg else v.Graph()
    try:
        g.set_input(m.shape[1], m.shape[0], ip)
        if setup:
            setup(g)
        g.set_debug(True)
        g.set_hist(hist)
        g.alloc()
        out = g.run(m).astype(np.float32)
        st = {"llap": out, "denoise": g.debug_stage(0), "hilite": g.debug_stage(1), "filmcurv": g.debug_stage(2),
              "demosaic": g.debug_stage(3), "colour": g.debug_stage(4)}
        if hist:
            st["hist"] = g.hist()
        try:
            st["crop"] = g.debug_stage(11)
        except v._lib.VkdtError:
            pass
        try:
            st["dn_nodes"] = {n: g.debug_stage(5 + i) for i, n in enumerate(oracle.DENOISE_NODES)}
        except v._lib.VkdtError:
            pass
        dec = {}
        for kind in ("gauss", "dn_cov", "dn_thr"):
            try:
                dec[kind] = g.debug_decisions(kind)
            except v._lib.VkdtError:
                pass
        st["dec"] = dec
    finally:
        g.close()
    return st


def colour_gain(m, ip, op, shape):
    """max over output channels of the sum of |colour matrix| entries: the colour
    stage of the oracle applied to unit inputs (it is linear below its clamp)"""
    h, w = shape[:2]
    unit = np.zeros((h, w, 4), np.float32)
    unit[..., 3] = 1.0
    for k in range(3):
        unit[k // w if k // w < h else 0, k % w, k] = 1.0
    q = oracle.develop(m, oracle.img_param(ip), params=op, stages=("colour",), start="colour", input=unit)["colour"]
    cols = [q[k // w if k // w < h else 0, k % w, :3] for k in range(3)]
    return float(np.abs(np.stack(cols, 1)).sum(1).max()) * 1.01


def crop_reach(op, dm_shape, out_shape, radius=2):
    """per output pixel of the crop stage, the largest |difference| of the demosaic
    output `d` (a 2-d map at the demosaic's size) within `radius` texels of the
    position the pixel samples (crop/main.comp, in double precision): the
    demosaic texels its filter can reach. Returns a function of d."""
    b = np.array([op.cr_block[k] for k in range(20)], np.float64)
    dh, dw = dm_shape[:2]
    ch, cw = out_shape[:2]
    y, x = np.mgrid[0:ch, 0:cw].astype(np.float64)
    px, py = x + 0.5 + b[16] * dw, y + 0.5 + b[18] * dh
    vx, vy = px - dw * 0.5, py - dh * 0.5
    qx, qy = b[12] * vx + b[14] * vy + dw * 0.5, b[13] * vx + b[15] * vy + dh * 0.5
    hz = b[2] * qx + b[6] * qy + b[10]
    with np.errstate(divide="ignore", invalid="ignore"):
        sx = (b[0] * qx + b[4] * qy + b[8]) / hz
        sy = (b[1] * qx + b[5] * qy + b[9]) / hz
    inside = (sx >= 0) & (sy >= 0) & (sx < dw) & (sy < dh)
    ix = np.clip(np.nan_to_num(sx), 0, dw - 1).astype(np.int64)
    iy = np.clip(np.nan_to_num(sy), 0, dh - 1).astype(np.int64)

    def reach(d):
        from numpy.lib.stride_tricks import sliding_window_view
        pad = np.pad(d, radius, mode="edge")
        mx = sliding_window_view(pad, (2 * radius + 1, 2 * radius + 1)).max(axis=(-1, -2))
        return np.where(inside, mx[iy, ix], 0.0)
    return reach


def check(name, v, m, ip, op, gpu, stages=("denoise", "hilite", "demosaic", "crop", "colour", "filmcurv", "llap"),
          tol=TOL, mean=MEAN, de=DE, double=False):
    """The CUDA path's stage images `gpu` (develop_gpu) against the oracle on the same
    mosaic and parameters; asserts the rules above and returns the record."""
    stages = tuple(s for s in stages if s in gpu)
    want = stages + (("hist",) if "hist" in gpu else ())
    own = oracle.develop(m, oracle.img_param(ip), params=op, stages=want, record=True, double=double)
    rec = {"size": [int(m.shape[1]), int(m.shape[0])], "levels": int(own["llap_levels"]), "fp64": bool(double)}
    dec = gpu["dec"]
    problems = []
    # ---- 1. decisions
    forced = own
    differ = {}
    for kind, d in dec.items():
        mine = own["dec_" + kind]
        assert d.shape == mine.shape, (kind, d.shape, mine.shape)
        diff = d != mine
        differ[kind] = int(diff.sum())
        rec["dec_" + kind + "_differ"] = differ[kind]
        if kind == "gauss" and diff.any():
            on_gpu_input, _ = oracle.gauss_decisions(gpu["hilite"], ip.filters)
            if not np.array_equal(on_gpu_input, d):
                problems.append(("gauss decisions not explained by the hilite input", int((on_gpu_input != d).sum())))
            rec["gauss_margin_max_differing"] = float(own["margin_gauss"][diff].max())
        elif kind == "dn_cov" and diff.any() and not double:
            problems.append(("denoise structure tensor decisions differ", differ[kind]))
        elif kind == "dn_thr" and diff.any() and not double:
            bits = (d ^ mine)
            mar = own["margin_dn_thr"]
            worst = 0.0
            for l in range(4):
                sel = ((bits >> l) & 1) == 1
                if sel.any():
                    worst = max(worst, float(mar[..., l][sel].max()))
            rec["dn_thr_margin_max_differing"] = worst
            if not worst < DN_THR_TIE:
                problems.append(("denoise threshold switch differs away from a tie", worst))
    if any(differ.values()):
        forced = oracle.develop(m, oracle.img_param(ip), params=op, stages=want, double=double,
                                force={k: dec[k] for k in differ})
    # ---- 2. node-wise (FP32, the CUDA path's own inputs, its decisions)
    node = {}
    order = ("denoise", "hilite", "demosaic", "crop", "colour", "filmcurv", "llap")
    prev = None
    for s in order:
        if s in stages and prev is not None:
            node[s] = oracle.develop(m, oracle.img_param(ip), params=op, stages=(s,), start=s, input=gpu[prev],
                                     force=dec)[s]
        if s in gpu:
            prev = s
    if "dn_nodes" in gpu:
        q = oracle.denoise_nodes(m, oracle.img_param(ip), op, gpu["dn_nodes"], force=dec)
        for n in oracle.DENOISE_NODES:
            node["dn_" + n] = (gpu["dn_nodes"][n], q[n])
        node["dn_doub"] = (gpu["denoise"], q["doub"])
    for s, nv in node.items():
        a, b = (gpu[s], nv) if not isinstance(nv, tuple) else nv
        e = rel_err(a, b)
        r = {"max": float(e.max()), "mean": float(e.mean())}
        rec.setdefault("node", {})[s] = r
        if not (r["max"] <= tol and r["mean"] <= mean):
            problems.append(("node", s, r, np.unravel_index(int(np.argmax(e)), e.shape)))
    # ---- 3. end to end against the oracle with the same decisions
    ill = op.dn_strength > 0 or op.dm_method == 1
    f64 = f32 = None
    if ill and not double:
        f64 = oracle.develop(m, oracle.img_param(ip), params=op, stages=stages, double=True,
                             force={k: dec[k] for k in dec})
    if ill and double:
        # against the FP64 build of an ill-conditioned path, the yardstick is the FP32
        # reference itself: the CUDA path is to be no farther from the FP64 result than
        # the FP32 arithmetic of the reference (with the same decisions) is
        f32 = oracle.develop(m, oracle.img_param(ip), params=op, stages=stages, force={k: dec[k] for k in dec})
    gain = None
    chain = None   # the oracle from colour on, on the CUDA path's own colour input
    for s in stages:
        a, b = gpu[s], forced[s]
        assert a.shape[:2] == b.shape[:2], (name, s, a.shape, b.shape)
        e = rel_err(a, b)
        over = e > tol
        r = {"max": float(e.max()), "mean": float(e.mean()), "over": int(over.sum()),
             "max_vs_own": float(rel_err(a, own[s]).max())}
        if forced is not own:
            r["flipped"] = int((rel_err(forced[s], own[s]) > tol).sum())
        if s in ("filmcurv", "llap"):
            dE = delta_e2000(a, b)
            r["de_max"] = float(dE.max())
            r["de_over"] = int((dE >= de).sum())
        if f64 is not None:
            e64 = rel_err(f64[s], b)
            r["fp64_over"] = int((e64 > tol).sum())
            r["fp64_max"] = float(e64.max())
            if s in ("filmcurv", "llap"):
                r["fp64_de_over"] = int((delta_e2000(f64[s], b) >= de).sum())
        if f32 is not None:
            e32 = rel_err(f32[s], b)
            r["fp32_over"], r["fp32_mean"] = int((e32 > tol).sum()), float(e32.mean())
            if s in ("filmcurv", "llap"):
                r["fp32_de_over"] = int((delta_e2000(f32[s], b) >= de).sum())
            if not (r["over"] <= 1.25 * r["fp32_over"] + 16 and r["mean"] <= 1.25 * r["fp32_mean"] + 1e-5
                    and r.get("de_over", 0) <= 1.25 * r.get("fp32_de_over", 0) + 16):
                problems.append(("farther from the FP64 build than the FP32 reference", s, r))
            rec[s] = r
            continue
        if not (r["mean"] <= mean):
            problems.append(("e2e mean", s, r["mean"]))
        if over.any() or r.get("de_over", 0):
            if ill and f64 is not None:
                if not (r["over"] <= r["fp64_over"] and r.get("de_over", 0) <= r.get("fp64_de_over", 0)):
                    problems.append(("e2e over the tolerance beyond the FP64 build's", s, r))
            elif s == "crop" and "demosaic" in gpu:
                # a resampler with weights of absolute sum below 1.3 (Catmull-Rom, or one texel):
                # |dcrop| <= node error + 1.3 max |ddemosaic| over the texels it reaches + one f16 step
                dcr = np.abs(a[..., :3].astype(np.float64) - b[..., :3]).max(-1)
                ddm = np.abs(gpu["demosaic"][..., :3].astype(np.float64) - forced["demosaic"][..., :3]).max(-1)
                dnode = np.abs(a[..., :3].astype(np.float64) - node["crop"][..., :3]).max(-1)
                step = np.abs(np.spacing(np.abs(b[..., :3]).astype(np.float16)).astype(np.float64)).max(-1)
                bound = dnode + 1.3 * crop_reach(op, ddm.shape, b.shape)(ddm) + step
                bad = over & (dcr > bound * 1.0001)
                r["over_beyond_reach_bound"] = int(bad.sum())
                if bad.any():
                    problems.append(("crop over the tolerance beyond the propagated bound", r))
            elif s == "colour" and "demosaic" in gpu:
                # linear colour transform: |dcol| <= node error + gain |dinput| + one f16 step
                if gain is None:
                    gain = colour_gain(m, ip, op, b.shape)
                    rec["colour_gain"] = gain
                dcol = np.abs(a[..., :3].astype(np.float64) - b[..., :3]).max(-1)
                src = "crop" if "crop" in gpu else "demosaic"
                ddm = np.abs(gpu[src][..., :3].astype(np.float64) - forced[src][..., :3]).max(-1)
                dnode = np.abs(a[..., :3].astype(np.float64) - node["colour"][..., :3]).max(-1)
                step = np.abs(np.spacing(np.abs(b[..., :3]).astype(np.float16)).astype(np.float64)).max(-1)
                bound = dnode + gain * ddm + step
                bad = over & (dcol > bound * 1.0001)
                r["over_beyond_gain_bound"] = int(bad.sum())
                if bad.any():
                    problems.append(("colour over the tolerance beyond the propagated bound", r))
            elif s in ("filmcurv", "llap") and ("crop" in gpu or "demosaic" in gpu):
                if chain is None:
                    src = "crop" if "crop" in gpu else "demosaic"
                    chain = oracle.develop(m, oracle.img_param(ip), params=op, stages=("filmcurv", "llap"),
                                           start="colour", input=gpu[src], force=dec)
                bad = over & (rel_err(a, chain[s]) > tol)
                bad |= (delta_e2000(a, b) >= de) & (delta_e2000(a, chain[s]) >= de)
                r["over_beyond_input_chain"] = int(bad.sum())
                if bad.any():
                    problems.append(("%s over the tolerance not explained by the colour input" % s, r))
            else:
                problems.append(("e2e", s, r, np.unravel_index(int(np.argmax(e)), e.shape)))
        rec[s] = r
    if "hist" in gpu:
        h = oracle.hist(gpu["colour"])
        rec["hist_equal_on_gpu_colour"] = bool(np.array_equal(h, gpu["hist"]))
        if not rec["hist_equal_on_gpu_colour"]:
            problems.append(("hist", int(np.abs(h.astype(np.int64) - gpu["hist"]).sum())))
    rec["ok"] = not problems
    log(name, rec)
    assert not problems, (name, problems, rec)
    return rec
