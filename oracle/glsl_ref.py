"""Run the reference's own shaders, compiled for the CPU (oracle/_ref), as the
node graph the modules' create_nodes build (test infrastructure only).

The shader sources are translated and compiled by oracle/glsl/translate.py
from the vkdt tree. This module packs push constants and uniform blocks the
way each module's create_nodes / commit_params do (cited per node) and
dispatches the nodes in the scheduler's order.
"""
import ctypes as C
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
SO = os.path.join(REF, "libvkdt_ref.so")
# the vkdt source tree (VKDT_REFERENCE, default: where this build found it)
MODULES = os.path.join(os.environ.get("VKDT_REFERENCE", "/root/reference"), "src", "pipe", "modules")

F16, F32, UNORM16 = 0, 1, 2


class ImageT(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_float)), ("w", C.c_int), ("h", C.c_int), ("c", C.c_int), ("fmt", C.c_int)]


class Dispatch(C.Structure):
    _fields_ = [("wd", C.c_int), ("ht", C.c_int), ("dp", C.c_int), ("uniform", C.c_void_p), ("push", C.c_void_p),
                ("glob", C.c_void_p), ("bind", (C.POINTER(ImageT) * 32) * 8), ("buf", C.c_void_p * 8)]


def build():
    """Translate and compile when the vkdt sources are present, else compile
    the translation units already in oracle/_ref (as on a machine without them)."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "glsl"))
    import translate
    if os.path.isdir(MODULES):
        translate.build(MODULES)
    elif os.path.isdir(REF) and any(f.endswith(".cpp") for f in os.listdir(REF)):
        translate.compile_ref()
    return available()


def available():
    return os.path.exists(SO)


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(SO)
    return _lib


class Img:
    def __init__(self, w, h, c, fmt=F16):
        self.a = np.zeros((h, w, c), np.float32)
        self.t = ImageT(self.a.ctypes.data_as(C.POINTER(C.c_float)), w, h, c, fmt)
        self.w, self.h, self.c = w, h, c


def run(name, wd, ht, binds, push=None, uniform=None, dp=1, buffers=None):
    """buffers: {binding: numpy array} for storage buffers"""
    d = Dispatch()
    for b, a in (buffers or {}).items():
        d.buf[b] = a.ctypes.data
    d.wd, d.ht, d.dp = wd, ht, dp
    keep = []
    for k, v in (("push", push), ("uniform", uniform)):
        if v is not None:
            buf = C.create_string_buffer(bytes(v) + b"\0" * 4096)
            keep.append(buf)
            setattr(d, k, C.cast(buf, C.c_void_p))
    glob = C.create_string_buffer(4096)
    keep.append(glob)
    d.glob = C.cast(glob, C.c_void_p)
    for b, im in binds.items():
        ims = im if isinstance(im, (list, tuple)) else [im]
        for e, x in enumerate(ims):
            d.bind[b][e] = C.pointer(x.t)
    getattr(lib(), "ref_" + name)(C.byref(d))


def f32(*v):
    return struct.pack("<%df" % len(v), *v)


def i32(*v):
    return struct.pack("<%di" % len(v), *v)


def u32(*v):
    return struct.pack("<%dI" % len(v), *v)


def develop(mosaic, ip, params=None, stages=("llap",)):
    """The development path on the reference shaders. ip: an oracle ImgParam,
    params: an oracle Params (module parameters). Returns a dict of stages
    (denoise, hilite: W*H, demosaic/colour/filmcurv/llap: H*W*4)."""
    import oracle
    p = params or oracle.default_params()
    mosaic = np.ascontiguousarray(mosaic, np.uint16)
    fh, fw = mosaic.shape
    raw = Img(fw, fh, 1, UNORM16)
    raw.a[..., 0] = mosaic.astype(np.float32) / np.float32(65535.0)
    filters = ip.filters
    block = 3 if filters == 9 else 2
    crop = [int(ip.crop_aabb[k]) for k in range(4)]
    W, H = crop[2] - crop[0], crop[3] - crop[1]
    black = [np.float32(ip.black[k]) / np.float32(65535.0) for k in range(4)]   # denoise/main.c:165-168
    white = [np.float32(ip.white[k]) / np.float32(65535.0) for k in range(4)]
    wb = [float(ip.whitebalance[k]) for k in range(4)]
    out = {}
    dn_par = f32(p.dn_strength, p.dn_luma, p.dn_detail, p.dn_pad, *list(p.dn_edges)) + i32(p.dn_gainmap)

    # ---- denoise (denoise/main.c:133-333)
    if p.dn_strength <= 0.0:
        dn = Img(W, H, 4)
        run("denoise_noop", W, H, {0: raw, 1: dn, 2: raw},
            push=i32(*crop) + f32(*black) + f32(*white) + f32(0, 0, 0, 0) + u32(filters, 0), uniform=dn_par)
    else:
        hw, hh = W // block, H // block
        half = Img(hw, hh, 4)
        run("denoise_half", hw, hh, {0: raw, 1: half},
            push=f32(*wb) + f32(*black) + f32(*white) + i32(*crop) + u32(filters), uniform=dn_par)
        downs = []
        src = half
        for i in range(4):
            o = Img(hw, hh, 4)
            cov = Img(hw, hh, 4)
            pc = f32(*wb) + f32(*black) + f32(*white) + i32(0, 0, 0, 0) + f32(ip.noise_a, ip.noise_b) + i32(i) + u32(block)
            if i == 0:
                run("denoise_downcov", hw, hh, {0: src, 1: o, 2: cov}, push=pc, uniform=dn_par)
            else:
                run("denoise_down", hw, hh, {0: src, 1: o}, push=pc, uniform=dn_par)
            downs.append(o)
            src = o
        asm = Img(hw, hh, 4)
        run("denoise_assemble", hw, hh, {0: half, 1: downs[0], 2: downs[1], 3: downs[2], 4: downs[3], 5: asm},
            push=f32(*wb) + f32(*black) + f32(*white) + i32(0, 0, 0, 0) + f32(ip.noise_a, ip.noise_b) + u32(filters),
            uniform=dn_par)
        dn = Img(W, H, 1)
        run("denoise_doub", W, H, {0: raw, 1: asm, 2: half, 3: dn, 4: half},
            push=f32(*wb) + f32(*black) + f32(*white) + i32(*crop) + u32(filters) + f32(ip.noise_a, ip.noise_b)
            + i32(0) + f32(0, 0, 0, 0), uniform=dn_par)
    if "denoise" in stages:
        out["denoise"] = dn.a[..., 0].copy()

    # ---- hilite (hilite/main.c:5-90)
    hl_par = f32(p.hl_white, p.hl_desat, p.hl_soft)
    hpc = f32(*wb) + u32(filters)
    hw, hh = W // block, H // block
    h0 = Img(hw, hh, 4)
    run("hilite_half", hw, hh, {0: dn, 1: h0}, push=hpc, uniform=hl_par)
    reds = []
    rcw, rch = (hw - 1) // 2 + 1, (hh - 1) // 2 + 1
    fine = h0
    for l in range(1, 15):
        r = Img(rcw, rch, 4)
        run("hilite_reduce", rcw, rch, {0: fine, 1: r}, push=hpc, uniform=hl_par)
        reds.append(r)
        fine = r
        rcw, rch = (rcw - 1) // 2 + 1, (rch - 1) // 2 + 1
        if rcw <= 1 or rch <= 1 or l + 1 == 15:
            break
    up = reds[-1]
    for l in range(len(reds) - 1, -1, -1):
        f = h0 if l == 0 else reds[l - 1]
        a = Img(f.w, f.h, 4)
        run("hilite_assemble", f.w, f.h, {0: f, 1: up, 2: a}, push=hpc, uniform=hl_par)
        up = a
    hl = Img(W, H, 1)
    run("hilite_doub", hw, hh, {0: dn, 1: up, 2: hl}, push=hpc, uniform=hl_par)
    if "hilite" in stages:
        out["hilite"] = hl.a[..., 0].copy()

    # ---- demosaic (demosaic/main.c:59-203)
    dm_par = i32(p.dm_colour, p.dm_method)
    dpc = f32(*wb) + u32(filters)
    ow = p.out_wd or (W if p.dm_method != 2 else (W + 1) // 2)   # demosaic/main.c:18-41
    oh = p.out_ht or (H if p.dm_method != 2 else (H + 1) // 2)
    scale = W / ow
    if scale >= 1.5 * block or p.dm_method == 2:
        hs = Img(W // block, H // block, 4)
        run("demosaic_halfsize", W // block, H // block, {0: hl, 1: hs}, push=dpc, uniform=dm_par)
        if block != scale:
            rgb = Img(ow, oh, 4)
            run("shared_resample", ow, oh, {0: [hs], 1: [rgb]})
        else:
            rgb = hs
    elif p.dm_method == 1:
        # demosaic/main.c:113-155: rcd_conv at full size, rcd_fill one workgroup per 58x26 tile
        vh, pq, lpi = Img(W, H, 1), Img(W // 2, H, 1), Img(W // 2, H, 1)
        run("demosaic_rcd_conv", W, H, {0: hl, 1: vh, 2: pq, 3: lpi})
        ntx, nty = (W + 57) // 58, (H + 25) // 26
        rgb = Img(W, H, 4)
        run("demosaic_rcd_fill", ntx * 8, nty * 8, {0: hl, 1: vh, 2: pq, 3: lpi, 4: rgb}, push=dpc)
    else:
        down = Img(W // block, H // block, 1)
        run("demosaic_down", W // block, H // block, {0: hl, 1: down}, push=dpc, uniform=dm_par)
        cov = Img(W // block, H // block, 4)
        run("demosaic_gauss", W // block, H // block, {0: down, 1: hl, 2: cov}, push=dpc, uniform=dm_par)
        g = Img(W, H, 1)
        run("demosaic_splat", W, H, {0: hl, 1: cov, 2: g}, push=dpc, uniform=dm_par)
        rgb = Img(W, H, 4)
        run("demosaic_fix", W, H, {0: hl, 1: g, 2: cov, 3: rgb}, push=dpc, uniform=dm_par)
    if "demosaic" in stages:
        out["demosaic"] = rgb.a.copy()

    # ---- crop (crop/main.comp on the block crop/main.c:276-343 commits)
    if p.cr_on:
        cr = Img(p.cr_wd, p.cr_ht, 4)
        run("crop_main", p.cr_wd, p.cr_ht, {0: rgb, 1: cr}, uniform=f32(*p.cr_block))
        rgb = cr
        if "crop" in stages:
            out["crop"] = rgb.a.copy()

    # ---- colour (colour/main.c:219-365 commit_params, 415-466 create_nodes)
    cw = [0.0, 0.0, 0.0]
    pw = [float(p.co_white[k]) for k in range(3)]
    if pw[0] == 0 and pw[1] == 0 and pw[2] == 0:
        w0 = [np.float32(0)] * 3
        wv = [np.float32(ip.whitebalance[k]) for k in range(3)]
        for j in range(3):
            for i in range(3):
                w0[j] = np.float32(w0[j] + np.float32(ip.cam_to_rec2020[3 * j + i]) / wv[i])
        w0 = [np.float32(w0[0] / w0[1]), np.float32(1.0), np.float32(w0[2] / w0[1])]
        pw = [np.float32(1) / w0[0], np.float32(1), np.float32(1) / w0[2]]
    mul = [np.float32(pw[0]) / np.float32(pw[1]), 1.0, np.float32(pw[2]) / np.float32(pw[1]), 2.0 ** p.co_exposure]
    f = np.zeros(4 + 12 + 4 + 12 + 96 + 96 + 5 + 8 + 5, np.float32)
    iv = f.view(np.uint32)
    f[0:4] = mul
    if p.co_matrix == 1:
        for j in range(3):
            for i in range(3):
                f[4 + 4 * i + j] = ip.cam_to_rec2020[3 * j + i]
        prim = 0  # s_colour_primaries_custom (i-raw/main.c:158)
    else:
        for j in range(3):
            for i in range(3):
                f[4 + 4 * j + i] = 1.0 if i == j else 0.0
        prim = 2
    off = 4 + 12 + 4 + 12 + 96 + 96
    f[off + 0] = 0.0
    iv[off + 1] = 0
    f[off + 2] = p.co_sat
    iv[off + 3] = 0
    iv[off + 4] = 0
    iv[off + 5] = prim
    iv[off + 6] = 0   # linear trc
    f[off + 7] = 0.0
    f[off + 8:off + 12] = [wb[0] / wb[1], 1.0, wb[2] / wb[1], 1.0]
    col = Img(rgb.w, rgb.h, 4)
    run("colour_main", rgb.w, rgb.h, {0: rgb, 1: col, 2: rgb, 3: rgb, 4: rgb, 5: rgb, 6: rgb}, push=i32(0, 0, 0),
        uniform=f.tobytes())
    if "colour" in stages:
        out["colour"] = col.a.copy()

    # ---- filmcurv (filmcurv/main.c:12-38)
    fc = Img(col.w, col.h, 4)
    run("filmcurv_main", col.w, col.h, {0: col, 1: fc},
        uniform=f32(p.fc_light, p.fc_contrast, p.fc_bias) + i32(p.fc_colour)
        + f32(p.fc_chroma, p.fc_rolloff, p.fc_red, p.fc_yellow, p.fc_blue, p.fc_shadows))
    if "filmcurv" in stages:
        out["filmcurv"] = fc.a.copy()

    # ---- llap (llap/main.c:6-106)
    ll_par = f32(p.ll_sigma, p.ll_shadows, p.ll_hilights, p.ll_clarity)
    ng = 10
    lev0 = [Img(fc.w, fc.h, 1) for _ in range(ng + 1)]
    run("llap_curve", fc.w, fc.h, {0: fc, 1: lev0}, push=u32(ng), uniform=ll_par)
    levels = [lev0]
    rcw, rch = (fc.w - 1) // 2 + 1, (fc.h - 1) // 2 + 1
    nl = 12
    for l in range(1, 12):
        lv = [Img(rcw, rch, 1) for _ in range(ng + 1)]
        run("llap_reduce", rcw, rch, {0: levels[-1], 1: lv}, uniform=ll_par, dp=ng + 1)
        levels.append(lv)
        rcw, rch = (rcw - 1) // 2 + 1, (rch - 1) // 2 + 1
        if rcw <= 1 or rch <= 1:
            nl = l + 1
            break
        if p.ll_levels > 0 and l + 1 == p.ll_levels:
            nl = l + 1
            break
    up = None
    for l in range(nl - 1, 0, -1):
        fine = levels[l - 1]
        a = Img(fine[0].w, fine[0].h, 1)
        first = 1 if l == nl - 1 else 0
        run("llap_assemble", a.w, a.h, {0: lev0[0] if first else up, 1: fine, 2: levels[l], 3: a},
            push=u32(ng, first), uniform=ll_par)
        up = a
    res = Img(fc.w, fc.h, 4)
    run("llap_colour", fc.w, fc.h, {0: up, 1: fc, 2: res}, uniform=ll_par)
    if "llap" in stages:
        out["llap"] = res.a.copy()
    out["llap_levels"] = nl
    return out


def rawhist(mosaic, ip, bins=1000):
    """rawhist/collect.comp (the reference shader) on a u16 mosaic with the
    uniforms rawhist/main.c:17-28 commits: (3, bins) counts, sums of means,
    sums of second moments, added in dispatch order as float atomics."""
    mosaic = np.ascontiguousarray(mosaic, np.uint16)
    ht, wd = mosaic.shape
    raw = Img(wd, ht, 1, UNORM16)
    raw.a[..., 0] = mosaic.astype(np.float32) / np.float32(65535.0)
    block = 3 if ip.filters == 9 else 2
    out = Img(bins, 5, 1, F32)
    uni = f32(ip.noise_a, ip.noise_b) + u32(ip.filters, max(1, int(ip.black[1])), int(ip.white[1]))
    run("rawhist_collect", wd // block, ht // block, {0: raw, 1: out}, uniform=uni)
    return out.a[:3, :, 0].astype(np.float64)


def waveform(rgba, wo=1000, ho=600):
    """hist/collect.comp (the reference shader) on an rgba f16 image: the wo x ho
    u32 waveform (rows of (1 - value) for values in [0, 1]: the shader converts
    negative floats to unsigned, which C++ leaves undefined, so the emulation is
    only meaningful on values in [0, 1])"""
    rgba = np.ascontiguousarray(rgba, np.float32)
    ht, wd = rgba.shape[:2]
    src = Img(wd, ht, 4)
    src.a[...] = rgba
    out = Img(wo, ho, 1, 3)
    run("hist_collect", wd, ht, {0: src, 1: out})
    return out.a[..., 0].copy().view(np.uint32)
