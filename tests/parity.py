"""Parity of the CUDA path against the oracle, at the stated tolerance.

The path computes in FP32 and stores f16 where the reference stores an image.
Every pixel of every checked stage is held to:
 - |a - b| / max(1, |b|) <= 2e-3, per pixel the largest over r, g, b: the
   absolute error below 1; above 1 relative, because f16 storage resolves
   values relatively (one f16 step of a value above 4 is more than 2e-3);
 - mean of that error <= 1e-4 over the image;
 - CIEDE2000 < 0.5 at every pixel after filmcurv and at the llap output,
against the oracle run with the CUDA path's own discrete decisions. The
reference has branches whose inputs come out of continuous arithmetic
(demosaic/gauss.comp:65,72 the structure tensor form and the snapped
direction; denoise/cov.glsl:84,130 the form and the hot pixel skip;
denoise/assemble.comp:144-153 the coarse threshold switch). Where such an
input is a near tie, an f16 step upstream can take the other branch, and
that pixel's neighbourhood then legitimately differs by far more than the
tolerance. So every decision the CUDA path took that differs from the
oracle's own is checked to be explained:
 - gauss: the CUDA path's decisions equal the oracle's gauss evaluated on the
   CUDA path's own hilite output, bit for bit (the gauss arithmetic is exact
   IEEE in both; a differing decision then follows from hilite values that
   are themselves within the tolerance);
 - dn_cov: equal to the oracle's own, bit for bit (exact IEEE arithmetic on
   the bit identical half size image);
 - dn_thr: a near tie: the oracle's own | |d_l| - 10 | / 10 < DN_THR_TIE.
The pixels where the oracle's own and the forced results differ beyond the
tolerance are the flipped pixels; they are counted and reported, and every
pixel (flipped or not) meets the tolerance against the forced oracle.
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


def develop_gpu(v, m, ip, setup=None, hist=False):
    """Develop through the C-ABI with the debug stages: every stage image and the decisions."""
    g = v.Graph()
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


def check(name, v, m, ip, op, gpu, stages=("denoise", "hilite", "demosaic", "colour", "filmcurv", "llap"),
          tol=TOL, mean=MEAN, de=DE, double=False):
    """The CUDA path's stage images `gpu` (develop_gpu) against the oracle on the same
    mosaic and parameters; asserts the tolerance above and returns the record."""
    stages = tuple(s for s in stages if s in gpu)
    want = stages + (("hist",) if "hist" in gpu else ())
    own = oracle.develop(m, oracle.img_param(ip), params=op, stages=want, record=True, double=double)
    rec = {"size": [int(m.shape[1]), int(m.shape[0])], "levels": int(own["llap_levels"]), "fp64": bool(double)}
    dec = gpu["dec"]
    forced = own
    differ = {}
    for kind, d in dec.items():
        mine = own["dec_" + kind]
        assert d.shape == mine.shape, (kind, d.shape, mine.shape)
        diff = d != mine
        differ[kind] = int(diff.sum())
        rec["dec_" + kind + "_differ"] = differ[kind]
        if kind == "gauss" and diff.any():
            # the exact gauss on the CUDA path's own hilite output takes the CUDA path's decisions
            on_gpu_input, _ = oracle.gauss_decisions(gpu["hilite"], ip.filters)
            assert np.array_equal(on_gpu_input, d), (name, "gauss decisions not explained by the hilite input",
                                                     int((on_gpu_input != d).sum()))
            rec["gauss_margin_max_differing"] = float(own["margin_gauss"][diff].max())
        elif kind == "dn_cov" and not double:
            assert not diff.any(), (name, "denoise structure tensor decisions differ", differ[kind])
        elif kind == "dn_thr" and diff.any():
            # the bits that differ: each one a near tie of |d_l| and 10 in the oracle
            bits = (d ^ mine)
            mar = own["margin_dn_thr"]
            worst = 0.0
            for l in range(4):
                sel = ((bits >> l) & 1) == 1
                if sel.any():
                    worst = max(worst, float(mar[..., l][sel].max()))
            rec["dn_thr_margin_max_differing"] = worst
            assert worst < DN_THR_TIE, (name, "denoise threshold switch differs away from a tie", worst)
    if any(differ.values()):
        forced = oracle.develop(m, oracle.img_param(ip), params=op, stages=want, double=double,
                                force={k: dec[k] for k in differ})
    worst = []
    for s in stages:
        a, b = gpu[s], forced[s]
        assert a.shape[:2] == b.shape[:2], (name, s, a.shape, b.shape)
        e = rel_err(a, b)
        r = {"max": float(e.max()), "mean": float(e.mean()),
             "max_vs_own": float(rel_err(a, own[s]).max())}
        if forced is not own:
            r["flipped"] = int((rel_err(forced[s], own[s]) > tol).sum())
        if s in ("filmcurv", "llap"):
            dE = delta_e2000(a, b)
            r["de_max"] = float(dE.max())
            if not (r["de_max"] < de):
                worst.append((s, "de", r["de_max"]))
        if not (r["max"] <= tol):
            worst.append((s, "max", r["max"], np.unravel_index(int(np.argmax(e)), e.shape)))
        if not (r["mean"] <= mean):
            worst.append((s, "mean", r["mean"]))
        rec[s] = r
    if "hist" in gpu:
        # the bins of the CUDA path's own colour output, bit exact
        h = oracle.hist(gpu["colour"])
        rec["hist_equal_on_gpu_colour"] = bool(np.array_equal(h, gpu["hist"]))
        if not rec["hist_equal_on_gpu_colour"]:
            worst.append(("hist", int(np.abs(h.astype(np.int64) - gpu["hist"]).sum())))
    log(name, rec)
    assert not worst, (name, worst, rec)
    return rec
