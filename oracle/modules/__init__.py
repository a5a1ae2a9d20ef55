"""The reference's module host code (create_nodes, commit_params, roi
callbacks) run on the CPU through oracle/modules/harness.c (test
infrastructure only): what the scheduler would hand to a device layer for a
cfg graph, as a node list and the modules' uniform blocks."""
import ctypes as C
import os

import numpy as np

from . import build as _build

HRN_MAX_NODES, HRN_MAX_MODULES = 512, 16


class HrnImg(C.Structure):
    _fields_ = [("black", C.c_float * 4), ("white", C.c_float * 4), ("whitebalance", C.c_float * 4),
                ("filters", C.c_uint32), ("crop_aabb", C.c_uint32 * 4), ("cam_to_rec2020", C.c_float * 9),
                ("noise_a", C.c_float), ("noise_b", C.c_float), ("orientation", C.c_uint32)]


class HrnNode(C.Structure):
    _fields_ = [("name", C.c_uint64), ("kernel", C.c_uint64), ("wd", C.c_int32), ("ht", C.c_int32),
                ("dp", C.c_int32), ("module", C.c_int32), ("push_size", C.c_int32), ("push", C.c_uint8 * 256)]


class HrnModule(C.Structure):
    _fields_ = [("name", C.c_uint64), ("inst", C.c_uint64), ("uniform_size", C.c_int32), ("param_size", C.c_int32),
                ("uniform", C.c_uint8 * 4096), ("param", C.c_uint8 * 4096), ("out_wd", C.c_int32),
                ("out_ht", C.c_int32)]


_lib = None


def available():
    return _build.available()


def lib():
    global _lib
    if _lib is None:
        # the module objects resolve the scheduler symbols from the harness
        _lib = C.CDLL(_build.HARNESS, mode=C.RTLD_GLOBAL)
        _lib.hrn_run.restype = C.c_int
        _lib.hrn_run.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(HrnImg), C.c_int,
                                 C.c_int, C.POINTER(HrnNode), C.c_int, C.POINTER(C.c_int), C.POINTER(HrnModule),
                                 C.c_int, C.POINTER(C.c_int)]
    return _lib


def token_str(t):
    return int(t).to_bytes(8, "little").rstrip(b"\0").decode()


def run(cfg, wd, ht, ip, out_wd=0, out_ht=0):
    """The reference's modules on the cfg text with an i-raw source of wd x ht and the
    image parameters ip (any struct with black, white, whitebalance, filters, crop_aabb,
    cam_to_rec2020, noise_a, noise_b). Returns (nodes, modules): nodes as dicts of
    name, kernel, wd, ht, dp, module, push (bytes); modules as dicts of name, inst,
    uniform (bytes), param (bytes), out (wd, ht)."""
    img = HrnImg()
    for k in range(4):
        img.black[k], img.white[k], img.whitebalance[k] = ip.black[k], ip.white[k], ip.whitebalance[k]
        img.crop_aabb[k] = ip.crop_aabb[k]
    img.filters = ip.filters
    for k in range(9):
        img.cam_to_rec2020[k] = ip.cam_to_rec2020[k]
    img.noise_a, img.noise_b = ip.noise_a, ip.noise_b
    img.orientation = getattr(ip, "orientation", 0)
    nodes = (HrnNode * HRN_MAX_NODES)()
    mods = (HrnModule * HRN_MAX_MODULES)()
    nn, nm = C.c_int(0), C.c_int(0)
    r = lib().hrn_run(_build.MODULES_DIR.encode(), _build.REF.encode(), cfg.encode(), wd, ht, C.byref(img), out_wd,
                      out_ht, nodes, HRN_MAX_NODES, C.byref(nn), mods, HRN_MAX_MODULES, C.byref(nm))
    if r:
        raise RuntimeError("module harness failed with %d" % r)
    out_n = [{"name": token_str(n.name), "kernel": token_str(n.kernel), "wd": n.wd, "ht": n.ht, "dp": n.dp,
              "module": n.module, "push": bytes(n.push[:n.push_size])} for n in nodes[:nn.value]]
    out_m = [{"name": token_str(m.name), "inst": token_str(m.inst), "uniform": bytes(m.uniform[:m.uniform_size]),
              "param": bytes(m.param[:m.param_size]), "out": (m.out_wd, m.out_ht)} for m in mods[:nm.value]]
    return out_n, out_m


def nprof(hist):
    """The reference's nprof/main.c fit (its write_sink) on a rawhist histogram
    (3 x bins: counts, sums of means, sums of second moments): (a, b) as the
    module writes them to its .nprof file ("%g %g")."""
    import tempfile
    h = np.ascontiguousarray(np.asarray(hist, np.float32).reshape(3, -1))
    fl = lib()
    fl.hrn_nprof.restype = C.c_int
    fl.hrn_nprof.argtypes = [C.c_char_p, C.c_void_p, C.c_int]
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as td:
        os.chdir(td)
        try:
            r = fl.hrn_nprof(_build.REF.encode(), h.ctypes.data, h.shape[1])
            if r:
                raise RuntimeError("nprof module failed with %d" % r)
            with open(os.path.join(td, "unknown--0.nprof")) as f:
                a, b = f.read().split()[:2]
        finally:
            os.chdir(cwd)
    return a, b
