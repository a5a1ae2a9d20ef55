"""vkdt_gb300: the raw development hot path of vkdt on GB300 (sm_103a CUDA).

Python mirror of the drop-in C-ABI (include/vkdt_cuda.h). The graph object
follows the reference's graph API: read a .cfg, set module parameters by
name, set the source image metadata, allocate, run, read the sink.
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import ImgParam, Scene, check, token, token_str, RUN_ALL, RUN_UPLOAD_SOURCE, RUN_DOWNLOAD_SINK, RUN_WAIT_DONE

__all__ = ["Graph", "Server", "ImgParam", "Scene", "init", "default_img_param", "scene_host", "scene_device",
           "DARKROOM_CFG", "DARKROOM_CROP_CFG", "DARKROOM_FULL_CFG", "CAM_TO_REC2020", "supports"]

# the synthetic camera: camera rgb -> rec2020, rows sum to one
CAM_TO_REC2020 = (1.20, -0.15, -0.05,
                  -0.10, 1.25, -0.15,
                  0.02, -0.22, 1.20)

# bin/default-darkroom.i-raw restricted to the modules of the path, with the
# cfg's parameter lines (DARKROOM_CROP_CFG: with its crop between demosaic and
# colour, at crop's defaults: exif rotation and a 3 px margin)
DARKROOM_CFG = """module:i-raw:main:43:400
module:denoise:01:218:400
module:hilite:01:393:400
module:demosaic:01:568:400
module:colour:01:931:400
module:filmcurv:01:1094:400
module:llap:01:1269:400
connect:i-raw:main:output:denoise:01:input
connect:denoise:01:output:hilite:01:input
connect:hilite:01:output:demosaic:01:input
connect:demosaic:01:output:colour:01:input
connect:colour:01:output:filmcurv:01:input
connect:filmcurv:01:output:llap:01:input
param:colour:01:exposure:0
param:llap:01:sigma:0.12
param:llap:01:shadows:1
param:llap:01:hilights:1
param:llap:01:clarity:0.2
"""
# the whole chain of bin/default-darkroom.i-raw: crop after demosaic, grade after llap (the cfg's
# histogram, zones, lens, pick and display modules are not on the path)
DARKROOM_CROP_CFG = (DARKROOM_CFG.replace("module:demosaic:01:568:400\n", "module:demosaic:01:568:400\nmodule:crop:01:743:400\n")
                     .replace("connect:demosaic:01:output:colour:01:input\n",
                              "connect:demosaic:01:output:crop:01:input\nconnect:crop:01:output:colour:01:input\n"))
DARKROOM_FULL_CFG = (DARKROOM_CROP_CFG.replace("module:llap:01:1269:400\n", "module:llap:01:1269:400\nmodule:grade:01:1444:400\n")
                     + "connect:llap:01:output:grade:01:input\n")

_inited = None


def init(device=0):
    """vkdt_cuda_init (replaces qvk_init)."""
    global _inited
    if _inited == device:
        return
    check(_lib.lib().vkdt_cuda_init(device, 0), "vkdt_cuda_init")
    _inited = device


def supports(name, kernel):
    return bool(_lib.lib().vkdt_cuda_supports(token(name), token(kernel)))


def default_img_param(black=512.0, white=16383.0, wb=(2.0, 1.0, 1.6), filters=0x94949494, wd=0, ht=0,
                      noise_a=0.0, noise_b=0.0, cam=CAM_TO_REC2020):
    ip = ImgParam()
    for k in range(4):
        ip.black[k] = black
        ip.white[k] = white
    ip.whitebalance[0], ip.whitebalance[1], ip.whitebalance[2], ip.whitebalance[3] = wb[0], wb[1], wb[2], 1.0
    ip.filters = filters
    ip.crop_aabb[0], ip.crop_aabb[1], ip.crop_aabb[2], ip.crop_aabb[3] = 0, 0, wd, ht
    for i in range(9):
        ip.cam_to_rec2020[i] = cam[i]
    ip.noise_a = noise_a
    ip.noise_b = noise_b
    return ip


def make_scene(wd, ht, seed=0, image_id=0, black=512.0, white=16383.0, a=2.0, b=0.4, wb=(2.0, 1.0, 1.6),
               filters=0x94949494, pan=(0.0, 0.0)):
    s = Scene()
    s.wd, s.ht, s.seed, s.image_id, s.filters = wd, ht, seed, image_id, filters
    s.black, s.white, s.noise_a, s.noise_b = black, white, a, b
    s.wb[0], s.wb[1], s.wb[2] = wb
    s.pan_x, s.pan_y = pan
    return s


def scene_host(scene):
    """The seeded mosaic, generated on the host (uint16 numpy array)."""
    out = np.empty((scene.ht, scene.wd), dtype=np.uint16)
    check(_lib.lib().vkdt_cuda_scene_generate_host(C.byref(scene), out.ctypes.data_as(C.POINTER(C.c_uint16))),
          "vkdt_cuda_scene_generate_host")
    return out


def scene_device(scene, d_ptr, stream=0):
    """Fill a device buffer (pointer) with the seeded mosaic."""
    check(_lib.lib().vkdt_cuda_scene_generate(C.byref(scene), C.c_void_p(d_ptr), C.c_void_p(stream)),
          "vkdt_cuda_scene_generate")


def unpack_mlv(d_packed, nbytes, bits_per_pixel, wd, ht, d_mosaic, stream=0):
    """vkdt_cuda_unpack_mlv: an uncompressed magic lantern frame (device bytes) into a
    device u16 mosaic of wd x ht (i-mlv's host unpack, on the device)."""
    check(_lib.lib().vkdt_cuda_unpack_mlv(C.c_void_p(d_packed), nbytes, bits_per_pixel, wd, ht, C.c_void_p(d_mosaic),
                                          C.c_void_p(stream)), "unpack_mlv")


def mcraw_decode(d_bitcnt, d_refval, d_data, data_bytes, rwd, ht, d_mosaic, ox=0, oy=0, wd=None, hgt=None,
                 d_scratch=None, stream=0):
    """vkdt_cuda_mcraw_decode: a motioncam frame (device buffers of bit counts, reference
    values and block data) into a device u16 mosaic of wd x hgt offset by (ox, oy). Without
    d_scratch a scratch buffer is allocated and the call waits for the device."""
    wd = rwd - ox if wd is None else wd
    hgt = ht - oy if hgt is None else hgt
    keep = None
    if d_scratch is None:
        import torch
        keep = torch.empty(max(8, _lib.lib().vkdt_cuda_mcraw_scratch_bytes(rwd, ht)), dtype=torch.uint8, device="cuda")
        d_scratch = keep.data_ptr()
    check(_lib.lib().vkdt_cuda_mcraw_decode(C.c_void_p(d_bitcnt), C.c_void_p(d_refval), C.c_void_p(d_data), data_bytes,
                                            rwd, ht, ox, oy, wd, hgt, C.c_void_p(d_mosaic), C.c_void_p(d_scratch),
                                            C.c_void_p(stream)), "mcraw_decode")
    if keep is not None:
        import torch
        torch.cuda.synchronize()


def colenc(d_rgba_f16, wd, ht, primaries, trc, d_out_f16=0, d_out_u8=0, stream=0):
    """vkdt_cuda_colenc: rec2020 rgba f16 to output primaries and transfer curve (f16 and/or u8)"""
    check(_lib.lib().vkdt_cuda_colenc(C.c_void_p(d_rgba_f16), wd, ht, primaries, trc, C.c_void_p(d_out_f16),
                                      C.c_void_p(d_out_u8), C.c_void_p(stream)), "colenc")


def bc1_encode(d_rgba_u8, wd, ht, d_blocks, stream=0):
    """vkdt_cuda_bc1_encode: BC1 blocks of a device rgba u8 image (o-bc1)"""
    check(_lib.lib().vkdt_cuda_bc1_encode(C.c_void_p(d_rgba_u8), wd, ht, C.c_void_p(d_blocks), C.c_void_p(stream)),
          "bc1_encode")


def rawhist(d_mosaic, wd, ht, img_param, bins=1000, d_scratch=None, stream=0):
    """vkdt_cuda_rawhist: noise statistics of a device mosaic (rawhist module), as a
    (3, bins) array of counts, sums of means and sums of second moments."""
    keep = None
    if d_scratch is None:
        import torch
        keep = torch.empty(_lib.lib().vkdt_cuda_rawhist_scratch_bytes(), dtype=torch.uint8, device="cuda")
        d_scratch = keep.data_ptr()
    out = np.zeros(3 * bins, np.float64)
    check(_lib.lib().vkdt_cuda_rawhist(C.c_void_p(d_mosaic), wd, ht, C.byref(img_param), bins, C.c_void_p(d_scratch),
                                       out.ctypes.data_as(C.POINTER(C.c_double)), C.c_void_p(stream)), "rawhist")
    return out.reshape(3, bins)


def waveform(d_rgba_f16, wd, ht, d_out_u32, out_wd=1000, out_ht=600, stream=0):
    """vkdt_cuda_waveform_rgba_f16: the hist module's rgb waveform (hist/collect.comp) of a
    device rgba f16 image into a device u32 image of out_wd x out_ht."""
    check(_lib.lib().vkdt_cuda_waveform_rgba_f16(C.c_void_p(d_rgba_f16), wd, ht, C.c_void_p(d_out_u32), out_wd, out_ht,
                                                 C.c_void_p(stream)), "waveform")


LENS_DEFAULTS = (0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 1.0, 1.0)   # lens/params: centre, scale, squish0/1, ca red/blue


def lens(d_in_rgba_f16, wd, ht, d_out_rgba_f16, params=LENS_DEFAULTS, out_wd=0, out_ht=0, stream=0):
    """vkdt_cuda_lens_rgba_f16: the lens module (lens/main.comp, the double sphere model) from a
    device rgba f16 image of wd x ht into one of out_wd x out_ht (default: the input's size)."""
    par = (C.c_float * 8)(*[float(x) for x in params])
    check(_lib.lib().vkdt_cuda_lens_rgba_f16(C.c_void_p(d_in_rgba_f16), wd, ht, C.c_void_p(d_out_rgba_f16),
                                             out_wd or wd, out_ht or ht, par, C.c_void_p(stream)), "lens")


def nprof_fit(hist):
    """vkdt_cuda_nprof_fit: the noise profile (a, b) of a rawhist histogram (nprof module)."""
    h = np.ascontiguousarray(np.asarray(hist, np.float64).reshape(-1))
    a, b = C.c_float(), C.c_float()
    code = _lib.lib().vkdt_cuda_nprof_fit(h.ctypes.data_as(C.POINTER(C.c_double)), h.size // 3, C.byref(a), C.byref(b))
    if code not in (_lib.SUCCESS, _lib.INCOMPLETE):
        check(code, "nprof_fit")
    return a.value, b.value, code == _lib.SUCCESS


class Graph:
    """A vkdt processing graph restricted to the development path."""

    def __init__(self, cfg=DARKROOM_CFG):
        self._l = _lib.lib()
        self._g = C.c_void_p()
        check(self._l.vkdt_cuda_graph_create(C.byref(self._g)), "vkdt_cuda_graph_create")
        if cfg is not None:
            b = cfg.encode()
            check(self._l.vkdt_cuda_graph_read_config(self._g, b, len(b)), "vkdt_cuda_graph_read_config")
        self.wd = self.ht = 0
        self.out_wd = self.out_ht = 0

    def close(self):
        if self._g:
            self._l.vkdt_cuda_graph_destroy(self._g)
            self._g = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- parameters
    def set_param(self, module, param, value, inst="01"):
        arr = np.atleast_1d(np.asarray(value))
        kind = np.int32 if np.issubdtype(arr.dtype, np.integer) else np.float32
        arr = np.ascontiguousarray(arr.astype(kind))
        check(self._l.vkdt_cuda_graph_set_param(self._g, token(module), token(inst), token(param),
                                                arr.ctypes.data, arr.nbytes), "set_param %s:%s" % (module, param))

    def get_param(self, module, param, count=1, dtype=np.float32, inst="01"):
        arr = np.zeros(count, dtype=dtype)
        check(self._l.vkdt_cuda_graph_get_param(self._g, token(module), token(inst), token(param),
                                                arr.ctypes.data, arr.nbytes), "get_param %s:%s" % (module, param))
        return arr

    def unsupported(self):
        n = self._l.vkdt_cuda_graph_unsupported(self._g, None, 0)
        buf = (C.c_uint64 * max(n, 1))()
        self._l.vkdt_cuda_graph_unsupported(self._g, buf, n)
        return [token_str(buf[i]) for i in range(n)]

    def set_input(self, wd, ht, img_param):
        self.wd, self.ht = wd, ht
        b = img_param.crop_aabb   # the denoise output: the crop window
        self.crop_wd, self.crop_ht = int(b[2] - b[0]), int(b[3] - b[1])
        self._filters = int(img_param.filters)
        check(self._l.vkdt_cuda_graph_set_input(self._g, wd, ht, C.byref(img_param)), "set_input")

    def set_llap_levels(self, n):
        check(self._l.vkdt_cuda_graph_set_llap_levels(self._g, n), "set_llap_levels")

    def set_output_size(self, wd, ht):
        check(self._l.vkdt_cuda_graph_set_output_size(self._g, wd, ht), "set_output_size")

    def set_hist(self, on=True):
        check(self._l.vkdt_cuda_graph_set_hist(self._g, 1 if on else 0), "set_hist")

    def set_timing(self, on=True):
        check(self._l.vkdt_cuda_graph_set_timing(self._g, 1 if on else 0), "set_timing")

    def set_debug(self, on=True):
        check(self._l.vkdt_cuda_graph_set_debug(self._g, 1 if on else 0), "set_debug")

    # ---- allocation and nodes
    def set_nodes(self, in_wd, in_ht, nodes):
        """vkdt_cuda_graph_set_nodes: the scheduler's nodes of the path's modules after
        create_nodes and commit_params, each a dict of name, kernel, wd, ht, dp, push
        (bytes) and uniform (bytes, its module's uniform block)."""
        keep = []
        arr = (_lib.NodeDesc * len(nodes))()
        for i, n in enumerate(nodes):
            push = C.create_string_buffer(bytes(n["push"]), max(1, len(n["push"])))
            uni = C.create_string_buffer(bytes(n.get("uniform", b"")), max(1, len(n.get("uniform", b""))))
            keep += [push, uni]
            arr[i] = _lib.NodeDesc(token(n["name"]), token(n["kernel"]), n["wd"], n["ht"], n["dp"], len(n["push"]),
                                   C.cast(push, C.c_void_p), len(n.get("uniform", b"")),
                                   C.cast(uni, C.c_void_p) if n.get("uniform") else None)
        check(self._l.vkdt_cuda_graph_set_nodes(self._g, in_wd, in_ht, arr, len(nodes)), "set_nodes")
        self.wd, self.ht = in_wd, in_ht
        return self

    def create_nodes(self):
        check(self._l.vkdt_cuda_graph_create_nodes(self._g), "create_nodes")

    def alloc(self):
        nbytes = C.c_uint64(0)
        check(self._l.vkdt_cuda_graph_alloc(self._g, C.byref(nbytes)), "alloc")
        w, h = C.c_int(), C.c_int()
        check(self._l.vkdt_cuda_graph_output_size(self._g, C.byref(w), C.byref(h)), "output_size")
        self.out_wd, self.out_ht = w.value, h.value
        return nbytes.value

    def nodes(self):
        out = []
        info = _lib.NodeInfo()
        for i in range(self._l.vkdt_cuda_graph_node_count(self._g)):
            check(self._l.vkdt_cuda_graph_node(self._g, i, C.byref(info)), "node")
            out.append((token_str(info.name), token_str(info.kernel), info.wd, info.ht, info.dp, info.fused))
        return out

    def device_buffers(self):
        s, d = C.c_void_p(), C.c_void_p()
        check(self._l.vkdt_cuda_graph_device_buffers(self._g, C.byref(s), C.byref(d)), "device_buffers")
        return s.value, d.value

    # ---- running
    def source(self):
        n = C.c_size_t()
        p = self._l.vkdt_cuda_graph_map_source(self._g, C.byref(n))
        if not p:
            raise RuntimeError("graph not allocated")
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint16)), shape=(self.ht, self.wd))

    def sink(self):
        n = C.c_size_t()
        p = self._l.vkdt_cuda_graph_map_sink(self._g, C.byref(n))
        if not p:
            raise RuntimeError("graph not allocated")
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint16)), shape=(self.out_ht, self.out_wd, 4)).view(np.float16)

    def run(self, mosaic=None, flags=RUN_ALL, stream=0):
        """Upload `mosaic` (if given), run, download and return the rgba f16 output."""
        if mosaic is not None:
            self.source()[...] = mosaic
        check(self._l.vkdt_cuda_graph_run(self._g, C.c_void_p(stream), flags), "run")
        if flags & RUN_DOWNLOAD_SINK and flags & RUN_WAIT_DONE:
            return self.sink().copy()
        return None

    def wait(self, timeout_ms=600000):
        check(self._l.vkdt_cuda_graph_wait(self._g, timeout_ms), "wait")

    def develop(self, d_mosaic, d_rgba, stream=0):
        check(self._l.vkdt_cuda_graph_develop(self._g, C.c_void_p(d_mosaic), C.c_void_p(d_rgba), C.c_void_p(stream)),
              "develop")

    def develop_static(self, d_mosaic, d_rgba, stream=0):
        """vkdt_cuda_graph_develop_static: develop a small image on the
        library's fixed device scratch, allocating nothing (the graph must
        not be allocated; call create_nodes first)."""
        check(self._l.vkdt_cuda_graph_develop_static(self._g, C.c_void_p(d_mosaic), C.c_void_p(d_rgba),
                                                     C.c_void_p(stream)), "develop_static")

    def times(self):
        n = self._l.vkdt_cuda_graph_query_times(self._g, None, None, None, 0)
        ms = (C.c_float * max(n, 1))()
        nm = (C.c_uint64 * max(n, 1))()
        kn = (C.c_uint64 * max(n, 1))()
        self._l.vkdt_cuda_graph_query_times(self._g, ms, nm, kn, n)
        return [("%s:%s" % (token_str(nm[i]), token_str(kn[i])), ms[i]) for i in range(n)]

    def hist(self):
        h = (C.c_uint32 * 257)()
        check(self._l.vkdt_cuda_graph_hist(self._g, h), "hist")
        return np.array(h[:], dtype=np.uint32)

    def debug_stage(self, stage):
        """0 denoise, 1 hilite (crop size, one channel); 2 filmcurv, 4 colour
        (output size, rgba); 3 demosaic (its own size, rgba); 11 crop (output
        size, rgba); wavelet denoise nodes (half size, rgba): 5 half, 6 downcov,
        7..9 down levels 1..3, 10 assemble."""
        w, h, c = C.c_int(), C.c_int(), C.c_int()
        check(self._l.vkdt_cuda_graph_debug_stage_size(self._g, stage, C.byref(w), C.byref(h), C.byref(c)),
              "debug_stage_size")
        out = np.empty((h.value, w.value, c.value), np.float32)
        check(self._l.vkdt_cuda_graph_debug_stage(self._g, stage, out.ctypes.data_as(C.POINTER(C.c_float)), out.size),
              "debug_stage")
        return out if c.value == 4 else out[..., 0]

    DECISIONS = {"gauss": (0, np.uint8), "dn_cov": (1, np.uint32), "dn_thr": (2, np.uint8)}

    def debug_decisions(self, kind):
        """The discrete decisions of the last run (vkdt_cuda_graph_debug_decisions):
        'gauss' (demosaic/gauss entries), 'dn_cov' and 'dn_thr' (wavelet denoise,
        half size texels), as an (ht, wd) array."""
        k, dt = self.DECISIONS[kind]
        w, h = C.c_int(), C.c_int()
        check(self._l.vkdt_cuda_graph_debug_decisions(self._g, k, None, 0, C.byref(w), C.byref(h)), "debug_decisions")
        out = np.zeros((h.value, w.value), dt)
        check(self._l.vkdt_cuda_graph_debug_decisions(self._g, k, out.ctypes.data, out.nbytes, None, None),
              "debug_decisions")
        return out


class Server:
    """The develop server (vkdt_cuda_server_*): continuous batching of develop
    jobs of any size on one device, `slots` in flight, graphs pooled by shape
    under a device memory cap."""

    def __init__(self, slots=4, hbm_cap=0, llap_levels=0, cfg=DARKROOM_CFG):
        self._l = _lib.lib()
        self._s = C.c_void_p()
        self._cfg = cfg.encode() if cfg is not None else None
        c = _lib.ServerCfg(self._cfg, len(self._cfg) if self._cfg else 0, slots, hbm_cap, llap_levels)
        check(self._l.vkdt_cuda_server_create(C.byref(c), C.byref(self._s)), "vkdt_cuda_server_create")
        self._keep = {}

    def submit(self, src, dst, wd, ht, img_param, out_wd=0, out_ht=0, src_on_device=True, dst_on_device=True):
        """src/dst: device pointers (ints) or host numpy arrays; returns the job id."""
        keep = []
        if not isinstance(src, int):
            keep.append(src)
            src_on_device, src = False, src.ctypes.data
        if not isinstance(dst, int):
            keep.append(dst)
            dst_on_device, dst = False, dst.ctypes.data
        j = _lib.Job(wd, ht, img_param, out_wd, out_ht, src, dst, int(src_on_device), int(dst_on_device))
        jid = C.c_uint64()
        check(self._l.vkdt_cuda_server_submit(self._s, C.byref(j), C.byref(jid)), "server_submit")
        if keep:
            self._keep[jid.value] = keep
        return jid.value

    def wait(self, job, timeout_ms=600000):
        try:
            check(self._l.vkdt_cuda_server_wait(self._s, job, timeout_ms), "server_wait")
        finally:
            pass
        self._keep.pop(job, None)

    def drain(self, timeout_ms=600000):
        check(self._l.vkdt_cuda_server_drain(self._s, timeout_ms), "server_drain")
        self._keep.clear()

    def job_times(self, job):
        q, l = C.c_double(), C.c_double()
        check(self._l.vkdt_cuda_server_job_times(self._s, job, C.byref(q), C.byref(l)), "server_job_times")
        return q.value, l.value

    def stats(self):
        st = _lib.ServerStats()
        check(self._l.vkdt_cuda_server_stats(self._s, C.byref(st)), "server_stats")
        return {f: getattr(st, f) for f, _ in _lib.ServerStats._fields_}

    def reset_stats(self):
        check(self._l.vkdt_cuda_server_reset_stats(self._s), "server_reset_stats")

    def close(self):
        if self._s:
            self._l.vkdt_cuda_server_destroy(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
