"""CPU oracle for the raw development path (test infrastructure only).

Restatement of the reference shaders in C++ (oracle.cpp), loaded with ctypes.
Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it,
as the reference results are compared against; the product library never
touches it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

# the oracle's OpenMP loops are short; spinning workers starve each other on
# shared hosts, so they sleep while idle (read once, when the runtime loads)
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(HERE, "oracle.h"), os.path.join(os.path.dirname(HERE), "vkdt_gb300", "csrc", "scene.h")]
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= max(os.path.getmtime(d) for d in deps):
        return SO
    # no contraction: the oracle's operation order is the reference's
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", SO, src]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout.decode())
    return SO


REF_DIR = os.path.join(HERE, "_ref")
STB_SO = os.path.join(REF_DIR, "libstb_dxt.so")
# the vkdt source tree the reference builds read (VKDT_REFERENCE, default: where this build found it)
VKDT_TREE = os.environ.get("VKDT_REFERENCE", "/root/reference")
STB_SRC = os.path.join(VKDT_TREE, "src", "pipe", "modules", "o-bc1")


def build_stb_ref():
    """Compile the reference's vendored stb_dxt (where it lies in the vkdt tree)
    into oracle/_ref/libstb_dxt.so; False where the vkdt tree is absent."""
    if os.path.exists(STB_SO):
        return True
    if not os.path.isfile(os.path.join(STB_SRC, "stb_dxt.h")):
        return False
    os.makedirs(REF_DIR, exist_ok=True)
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I" + STB_SRC, "-o", STB_SO,
           os.path.join(HERE, "stb_ref.c"), "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("stb_dxt build failed:\n" + r.stdout.decode())
    return True


def stb_bc1(rgba):
    """the reference's own encoder on an rgba u8 image (H x W x 4)"""
    rgba = np.ascontiguousarray(rgba, np.uint8)
    ht, wd = rgba.shape[:2]
    out = np.zeros((ht // 4) * (wd // 4) * 8, np.uint8)
    C.CDLL(STB_SO).stb_ref_bc1(rgba.ctypes.data_as(C.c_void_p), wd, ht, out.ctypes.data_as(C.c_void_p))
    return out


def colenc(rgba, prim, trc):
    """colenc restated: H x W x 4 float rgba in, FP32 rgba out"""
    rgba = np.ascontiguousarray(rgba, np.float32)
    ht, wd = rgba.shape[:2]
    out = np.zeros((ht, wd, 4), np.float32)
    lib().oracle_colenc(rgba.ctypes.data, wd, ht, prim, trc, out.ctypes.data)
    return out


def grade(rgba, lift=(0, 0, 0, 0), gamma=(1, 1, 1, 0), gain=(1, 1, 1, 0), offset=(0, 0, 0, 0), mode=0,
          sh_pivot=0.3, hi_pivot=0.4):
    """grade restated: H x W x 4 float rgba in (the llap output as stored), FP32 rgba out"""
    rgba = np.ascontiguousarray(rgba, np.float32)
    ht, wd = rgba.shape[:2]
    par = np.ascontiguousarray(np.concatenate([lift, gamma, gain, offset]).astype(np.float32))
    out = np.zeros((ht, wd, 4), np.float32)
    lib().oracle_grade(rgba.ctypes.data, wd, ht, par.ctypes.data, int(mode), float(sh_pivot), float(hi_pivot),
                       out.ctypes.data)
    return out


LENS_DEFAULTS = (0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 1.0, 1.0)   # lens/params: centre, scale, squish0/1, ca red/blue


def lens(rgba, par=LENS_DEFAULTS, out_size=None):
    """lens/main.comp restated: H x W x 4 float rgba in (as stored), f16-rounded rgba out of out_size (W, H)"""
    rgba = np.ascontiguousarray(rgba, np.float32)
    ht, wd = rgba.shape[:2]
    owd, oht = out_size or (wd, ht)
    par = np.ascontiguousarray(par, np.float32)
    assert par.size == 8
    out = np.zeros((oht, owd, 4), np.float32)
    lib().oracle_lens(rgba.ctypes.data, wd, ht, owd, oht, par.ctypes.data, out.ctypes.data)
    return out


def bc1_encode(rgba):
    """o-bc1 restated: BC1 blocks of an rgba u8 image (H x W x 4), 8 bytes per whole 4x4 block"""
    rgba = np.ascontiguousarray(rgba, np.uint8)
    ht, wd = rgba.shape[:2]
    out = np.zeros((ht // 4) * (wd // 4) * 8, np.uint8)
    lib().oracle_bc1_encode(rgba.ctypes.data, wd, ht, out.ctypes.data)
    return out


class ImgParam(C.Structure):
    _fields_ = [
        ("black", C.c_float * 4), ("white", C.c_float * 4), ("whitebalance", C.c_float * 4),
        ("filters", C.c_uint32), ("crop_aabb", C.c_uint32 * 4), ("cam_to_rec2020", C.c_float * 9),
        ("noise_a", C.c_float), ("noise_b", C.c_float),
    ]


class Params(C.Structure):
    _fields_ = [
        ("dn_strength", C.c_float), ("dn_luma", C.c_float), ("dn_detail", C.c_float), ("dn_pad", C.c_float),
        ("dn_edges", C.c_float * 4), ("dn_gainmap", C.c_int32),
        ("hl_white", C.c_float), ("hl_desat", C.c_float), ("hl_soft", C.c_float),
        ("dm_colour", C.c_int32), ("dm_method", C.c_int32),
        ("co_exposure", C.c_float), ("co_sat", C.c_float), ("co_matrix", C.c_int32), ("co_white", C.c_float * 4),
        ("fc_light", C.c_float), ("fc_contrast", C.c_float), ("fc_bias", C.c_float), ("fc_colour", C.c_int32),
        ("fc_chroma", C.c_float), ("fc_rolloff", C.c_float), ("fc_red", C.c_float), ("fc_yellow", C.c_float),
        ("fc_blue", C.c_float), ("fc_shadows", C.c_float),
        ("ll_sigma", C.c_float), ("ll_shadows", C.c_float), ("ll_hilights", C.c_float), ("ll_clarity", C.c_float),
        ("ll_levels", C.c_int32), ("out_wd", C.c_int32), ("out_ht", C.c_int32),
        ("cr_on", C.c_int32), ("cr_wd", C.c_int32), ("cr_ht", C.c_int32), ("cr_block", C.c_float * 20),
    ]


class Stages(C.Structure):
    _fields_ = [
        ("denoise", C.POINTER(C.c_float)), ("hilite", C.POINTER(C.c_float)), ("demosaic", C.POINTER(C.c_float)),
        ("colour", C.POINTER(C.c_float)), ("filmcurv", C.POINTER(C.c_float)), ("hist", C.POINTER(C.c_uint32)),
        ("llap", C.POINTER(C.c_float)), ("out_wd", C.c_int32), ("out_ht", C.c_int32),
        ("llap_levels", C.c_int32), ("hilite_levels", C.c_int32), ("crop", C.POINTER(C.c_float)),
    ]


class Decisions(C.Structure):
    _fields_ = [
        ("gauss", C.c_void_p), ("gauss_force", C.c_void_p), ("gauss_margin", C.c_void_p),
        ("dn_cov", C.c_void_p), ("dn_cov_force", C.c_void_p), ("dn_cov_margin", C.c_void_p),
        ("dn_thr", C.c_void_p), ("dn_thr_force", C.c_void_p), ("dn_thr_margin", C.c_void_p),
    ]


# decision kinds: (element type, margins per element)
DECISION_KINDS = {"gauss": (np.uint8, 2), "dn_cov": (np.uint32, 2), "dn_thr": (np.uint8, 4)}

_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(SO)
        l.oracle_default_params.argtypes = [C.POINTER(Params)]
        for f in (l.oracle_develop_f32, l.oracle_develop_f64):
            f.restype = C.c_int
            f.argtypes = [C.POINTER(C.c_uint16), C.c_int, C.c_int, C.POINTER(ImgParam), C.POINTER(Params), C.POINTER(Stages)]
        l.oracle_set_perturb.argtypes = [C.c_uint32]
        l.oracle_crop_commit.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_uint32, C.c_void_p,
                                         C.POINTER(C.c_int), C.POINTER(C.c_int)]
        l.oracle_denoise_nodes.restype = C.c_int
        l.oracle_denoise_nodes.argtypes = [C.POINTER(C.c_uint16), C.c_int, C.c_int, C.POINTER(ImgParam),
                                           C.POINTER(Params), C.c_void_p * 6, C.c_void_p * 7, C.POINTER(Decisions)]
        l.oracle_develop_from_f32.restype = C.c_int
        l.oracle_develop_from_f32.argtypes = [C.POINTER(C.c_uint16), C.c_int, C.c_int, C.POINTER(ImgParam),
                                              C.POINTER(Params), C.POINTER(Stages), C.POINTER(Decisions), C.c_int,
                                              C.c_void_p]
        for f in (l.oracle_develop_dec_f32, l.oracle_develop_dec_f64):
            f.restype = C.c_int
            f.argtypes = [C.POINTER(C.c_uint16), C.c_int, C.c_int, C.POINTER(ImgParam), C.POINTER(Params),
                          C.POINTER(Stages), C.POINTER(Decisions)]
        l.oracle_scene.argtypes = [C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_float,
                                   C.c_float, C.c_float, C.c_void_p, C.c_float, C.c_float, C.c_void_p]
        l.oracle_gauss_decisions.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint32, C.c_void_p, C.c_void_p]
        l.oracle_noop.argtypes = [C.POINTER(C.c_uint16), C.c_int, C.c_int, C.POINTER(ImgParam), C.POINTER(C.c_float)]
        l.oracle_hist.argtypes = [C.POINTER(C.c_float), C.c_int, C.c_int, C.POINTER(C.c_uint32)]
        l.oracle_waveform.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        l.oracle_hist_bin.restype = C.c_uint32
        l.oracle_hist_bin.argtypes = [C.c_float, C.c_float, C.c_float]
        l.oracle_cfa_colour.restype = C.c_int
        l.oracle_cfa_colour.argtypes = [C.c_uint32, C.c_int, C.c_int]
        l.oracle_rawhist.argtypes = [C.POINTER(C.c_uint16), C.c_int, C.c_int, C.c_uint32, C.c_float, C.c_float,
                                     C.c_int, C.POINTER(C.c_double)]
        l.oracle_f16.restype = C.c_float
        l.oracle_f16.argtypes = [C.c_float]
        l.oracle_unpack_mlv.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_size_t, C.c_void_p]
        l.oracle_pack_mlv.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p, C.c_size_t]
        l.oracle_mcraw_decode.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int, C.c_void_p]
        l.oracle_mcraw_encode.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_size_t]
        l.oracle_mcraw_encode.restype = C.c_size_t
        l.oracle_colenc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        l.oracle_bc1_encode.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        l.oracle_grade.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_void_p]
        l.oracle_lens.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        l.oracle_rcd.argtypes = [C.POINTER(C.c_float), C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        _lib = l
    return _lib


def default_params():
    p = Params()
    lib().oracle_default_params(C.byref(p))
    return p


def img_param(src):
    """Copy a vkdt_gb300.ImgParam (same layout) into the oracle's struct."""
    ip = ImgParam()
    C.memmove(C.byref(ip), C.byref(src), C.sizeof(ImgParam))
    return ip


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


START = {"hilite": 1, "demosaic": 2, "crop": 3, "colour": 4, "filmcurv": 5, "llap": 6}


def develop(mosaic, ip, params=None, double=False, stages=("llap",), record=False, force=None, start=None,
            input=None, perturb=0):
    """Run the oracle on a u16 mosaic; returns a dict of the requested stage images.

    record: also return the oracle's own discrete decisions and their margins
    ("dec_<kind>", "margin_<kind>" for the kinds of DECISION_KINDS that the
    graph has). force: {kind: array} decisions applied in place of the
    oracle's own (the grids of vkdt_cuda_graph_debug_decisions). start, input:
    run the path from stage `start` (a key of START) on `input`, the output of
    the stage before it (FP32 only). perturb: a nonzero seed rounds every f16
    store to a neighbouring f16 value at random (a sensitivity run)."""
    mosaic = np.ascontiguousarray(mosaic, dtype=np.uint16)
    ht, wd = mosaic.shape
    params = params or default_params()
    W = ip.crop_aabb[2] - ip.crop_aabb[0]
    H = ip.crop_aabb[3] - ip.crop_aabb[1]
    dw = params.out_wd or (W if params.dm_method != 2 else (W + 1) // 2)   # method 2 halves the size
    dh = params.out_ht or (H if params.dm_method != 2 else (H + 1) // 2)
    ow, oh = (params.cr_wd, params.cr_ht) if params.cr_on else (dw, dh)   # the stages after crop
    if "crop" in stages and not params.cr_on:
        raise ValueError("the crop stage needs params.cr_on (set_crop)")
    st = Stages()
    bufs = {}
    for name in stages:
        if name in ("denoise", "hilite"):
            bufs[name] = np.zeros((H, W), np.float32)
        elif name == "hist":
            bufs[name] = np.zeros(257, np.uint32)
        elif name == "demosaic":
            bufs[name] = np.zeros((dh, dw, 4), np.float32)
        else:
            bufs[name] = np.zeros((oh, ow, 4), np.float32)
        if name == "hist":
            st.hist = bufs[name].ctypes.data_as(C.POINTER(C.c_uint32))
        else:
            setattr(st, name, _fptr(bufs[name]))
    lib().oracle_set_perturb(int(perturb))
    try:
        return _develop(mosaic, ip, params, double, stages, record, force, start, input, W, H, ht, wd, st, bufs)
    finally:
        lib().oracle_set_perturb(0)


def _develop(mosaic, ip, params, double, stages, record, force, start, input, W, H, ht, wd, st, bufs):
    if start is not None:
        if double:
            raise ValueError("the path from a stage runs on the FP32 build")
        inp = np.ascontiguousarray(input, np.float32)
        dec = Decisions()
        keep = [inp]
        for kind, arr in (force or {}).items():
            a = np.ascontiguousarray(arr, DECISION_KINDS[kind][0])
            keep.append(a)
            setattr(dec, kind + "_force", a.ctypes.data)
        r = lib().oracle_develop_from_f32(mosaic.ctypes.data_as(C.POINTER(C.c_uint16)), wd, ht, C.byref(ip),
                                          C.byref(params), C.byref(st), C.byref(dec), START[start], inp.ctypes.data)
    elif record or force:
        block = 3 if ip.filters == 9 else 2
        gw, gh = W // block, H // block
        dec = Decisions()
        keep = []
        if record:
            for kind, (dt, nm) in DECISION_KINDS.items():
                bufs["dec_" + kind] = np.zeros((gh, gw), dt)
                bufs["margin_" + kind] = np.zeros((gh, gw, nm), np.float32)
                setattr(dec, kind, bufs["dec_" + kind].ctypes.data)
                setattr(dec, kind + "_margin", bufs["margin_" + kind].ctypes.data)
        for kind, arr in (force or {}).items():
            dt = DECISION_KINDS[kind][0]
            a = np.ascontiguousarray(arr, dt)
            if a.shape != (gh, gw):
                raise ValueError("forced %s decisions of shape %s, the grid is %s" % (kind, a.shape, (gh, gw)))
            keep.append(a)
            setattr(dec, kind + "_force", a.ctypes.data)
        f = lib().oracle_develop_dec_f64 if double else lib().oracle_develop_dec_f32
        r = f(mosaic.ctypes.data_as(C.POINTER(C.c_uint16)), wd, ht, C.byref(ip), C.byref(params), C.byref(st),
              C.byref(dec))
    else:
        f = lib().oracle_develop_f64 if double else lib().oracle_develop_f32
        r = f(mosaic.ctypes.data_as(C.POINTER(C.c_uint16)), wd, ht, C.byref(ip), C.byref(params), C.byref(st))
    if r != 0:
        raise RuntimeError("oracle develop failed with %d" % r)
    bufs["llap_levels"] = st.llap_levels
    bufs["hilite_levels"] = st.hilite_levels
    return bufs


DENOISE_NODES = ("half", "downcov", "down1", "down2", "down3", "assemble")


def denoise_nodes(mosaic, ip, params, inputs, force=None):
    """The wavelet denoise node by node on given inputs (a dict of DENOISE_NODES
    images, hw x hh x 4): each node's output from its inputs in `inputs`,
    plus "doub" (the denoised mosaic, W x H)."""
    mosaic = np.ascontiguousarray(mosaic, np.uint16)
    ht, wd = mosaic.shape
    ins = [np.ascontiguousarray(inputs[n], np.float32) for n in DENOISE_NODES]
    hh, hw = ins[0].shape[:2]
    W = ip.crop_aabb[2] - ip.crop_aabb[0]
    H = ip.crop_aabb[3] - ip.crop_aabb[1]
    outs = [np.zeros((hh, hw, 4), np.float32) for _ in DENOISE_NODES] + [np.zeros((H, W), np.float32)]
    dec = Decisions()
    keep = []
    for kind, arr in (force or {}).items():
        a = np.ascontiguousarray(arr, DECISION_KINDS[kind][0])
        keep.append(a)
        setattr(dec, kind + "_force", a.ctypes.data)
    pin = (C.c_void_p * 6)(*[a.ctypes.data for a in ins])
    pout = (C.c_void_p * 7)(*[a.ctypes.data for a in outs])
    r = lib().oracle_denoise_nodes(mosaic.ctypes.data_as(C.POINTER(C.c_uint16)), wd, ht, C.byref(ip), C.byref(params),
                                   pin, pout, C.byref(dec))
    if r:
        raise RuntimeError("oracle denoise nodes failed with %d" % r)
    res = dict(zip(DENOISE_NODES, outs[:6]))
    res["doub"] = outs[6]
    return res


def crop_commit(wd, ht, perspect=(0.25, 0.25, 0.75, 0.25, 0.75, 0.75, 0.25, 0.75), crop=(1.0, 3.0, 3.0, 7.0),
                rotate=1337.0, orientation=0):
    """crop/main.c commit_params and modify_roi_out restated for an input of
    wd x ht: (the 20 float committed block, output width, output height)"""
    blk = (C.c_float * 20)()
    ow, oh = C.c_int(), C.c_int()
    pp = (C.c_float * 8)(*perspect)
    cc = (C.c_float * 4)(*crop)
    lib().oracle_crop_commit(wd, ht, pp, cc, float(rotate), orientation, blk, C.byref(ow), C.byref(oh))
    return np.array(blk[:], np.float32), ow.value, oh.value


def set_crop(params, block, wd, ht):
    """switch the crop stage on in oracle params with a committed block and output size"""
    params.cr_on, params.cr_wd, params.cr_ht = 1, int(wd), int(ht)
    for i in range(20):
        params.cr_block[i] = float(block[i])
    return params


def scene(wd, ht, seed=0, image_id=0, filters=0x94949494, black=512.0, white=16383.0, a=2.0, b=0.4,
          wb=(2.0, 1.0, 1.6), pan=(0.0, 0.0)):
    """The benchmarks' seeded mosaic (u16 H x W), without the CUDA library."""
    out = np.zeros((ht, wd), np.uint16)
    w = np.ascontiguousarray(wb, np.float32)
    lib().oracle_scene(wd, ht, seed, image_id, filters, black, white, a, b, w.ctypes.data, pan[0], pan[1],
                       out.ctypes.data)
    return out


def gauss_decisions(mosaic, filters):
    """demosaic/gauss.comp's decisions on a given mosaic (H x W floats, the hilite
    output) and their margins: (H/block x W/block u8, ... x 2 f32)."""
    mosaic = np.ascontiguousarray(mosaic, np.float32)
    ht, wd = mosaic.shape
    block = 3 if filters == 9 else 2
    dec = np.zeros((ht // block, wd // block), np.uint8)
    mar = np.zeros((ht // block, wd // block, 2), np.float32)
    lib().oracle_gauss_decisions(mosaic.ctypes.data, wd, ht, filters, dec.ctypes.data, mar.ctypes.data)
    return dec, mar


def rcd(cfa, wb):
    """demosaic/rcd_conv + rcd_fill on an f16 bayer mosaic (H x W floats): H x W x 4"""
    cfa = np.ascontiguousarray(cfa, np.float32)
    ht, wd = cfa.shape
    out = np.zeros((ht, wd, 4), np.float32)
    w = (C.c_float * 3)(*[float(x) for x in wb[:3]])
    lib().oracle_rcd(_fptr(cfa), wd, ht, w, _fptr(out))
    return out


def mlv_bytes(npix, bpp):
    """bytes of an uncompressed magic lantern frame (video_mlv.c:630)"""
    return npix * bpp // 8


def unpack_mlv(packed, bpp, npix):
    packed = np.ascontiguousarray(packed, np.uint8)
    out = np.zeros(npix, np.uint16)
    lib().oracle_unpack_mlv(packed.ctypes.data, packed.size, bpp, npix, out.ctypes.data)
    return out


def pack_mlv(values, bpp):
    values = np.ascontiguousarray(values, np.uint16).ravel()
    out = np.zeros(mlv_bytes(values.size, bpp), np.uint8)
    lib().oracle_pack_mlv(values.ctypes.data, values.size, bpp, out.ctypes.data, out.size)
    return out


def mcraw_decode(bitcnt, refval, data, rwd, ht, ox=0, oy=0, wd_out=None, ht_out=None):
    """i-mcraw decode of one frame (nibble counts, u16 references, data bytes)"""
    wd_out = rwd - ox if wd_out is None else wd_out
    ht_out = ht - oy if ht_out is None else ht_out
    bitcnt = np.ascontiguousarray(bitcnt, np.uint8)
    refval = np.ascontiguousarray(refval, np.uint16)
    data = np.ascontiguousarray(data, np.uint8)
    out = np.zeros((ht_out, wd_out), np.uint16)
    lib().oracle_mcraw_decode(bitcnt.ctypes.data, refval.ctypes.data, data.ctypes.data, data.size, rwd, ht, ox, oy,
                              wd_out, ht_out, out.ctypes.data)
    return out


def mcraw_encode(img, force_cnt=-1):
    """a frame (ht x rwd u16, rwd a multiple of 64, ht of 4) as (bitcnt, refval, data)"""
    img = np.ascontiguousarray(img, np.uint16)
    ht, rwd = img.shape
    blocks = rwd * ht // 64
    bitcnt = np.zeros((blocks + 1) // 2, np.uint8)
    refval = np.zeros(blocks, np.uint16)
    data = np.zeros(blocks * 128, np.uint8)
    n = lib().oracle_mcraw_encode(img.ctypes.data, rwd, ht, force_cnt, bitcnt.ctypes.data, refval.ctypes.data,
                                  data.ctypes.data, data.size)
    if n == 0 and blocks:
        raise RuntimeError("mcraw encode failed")
    return bitcnt, refval, data[:n].copy()


def noop(mosaic, ip):
    mosaic = np.ascontiguousarray(mosaic, dtype=np.uint16)
    ht, wd = mosaic.shape
    W = ip.crop_aabb[2] - ip.crop_aabb[0]
    H = ip.crop_aabb[3] - ip.crop_aabb[1]
    out = np.zeros((H, W), np.float32)
    lib().oracle_noop(mosaic.ctypes.data_as(C.POINTER(C.c_uint16)), wd, ht, C.byref(ip), _fptr(out))
    return out


def hist(rgba):
    rgba = np.ascontiguousarray(rgba, dtype=np.float32)
    h = np.zeros(257, np.uint32)
    lib().oracle_hist(_fptr(rgba), rgba.shape[1], rgba.shape[0], h.ctypes.data_as(C.POINTER(C.c_uint32)))
    return h


def waveform(rgba, wo=1000, ho=600):
    """hist/collect.comp restated: the rgb waveform (ho x wo u32) of an H x W x 4 float image"""
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros((ho, wo), np.uint32)
    lib().oracle_waveform(rgba.ctypes.data, rgba.shape[1], rgba.shape[0], wo, ho, out.ctypes.data)
    return out


def hist_bin(r, g, b):
    return lib().oracle_hist_bin(r, g, b)


def cfa_colour(filters, x, y):
    return lib().oracle_cfa_colour(filters, x, y)


def f16(v):
    return lib().oracle_f16(v)


def rawhist(mosaic, filters, black, white, bins=1000):
    """rawhist/collect.comp statistics (counts, sums of means, sums of second moments), shape (3, bins)."""
    mosaic = np.ascontiguousarray(mosaic, dtype=np.uint16)
    ht, wd = mosaic.shape
    out = np.zeros(3 * bins, np.float64)
    lib().oracle_rawhist(mosaic.ctypes.data_as(C.POINTER(C.c_uint16)), wd, ht, filters, black, white, bins,
                         out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(3, bins)
