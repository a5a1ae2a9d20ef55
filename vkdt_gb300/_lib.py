"""ctypes binding of libvkdt_cuda (include/vkdt_cuda.h).

The library is built in-tree by vkdt_gb300.build; there is no fallback: if
the shared object is missing or fails to load, every entry point raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvkdt_cuda.so")

SUCCESS = 0
NOT_READY = 1
TIMEOUT = 2
INCOMPLETE = 5
ERROR_OUT_OF_HOST_MEMORY = -1
ERROR_OUT_OF_DEVICE_MEMORY = -2
ERROR_INITIALIZATION_FAILED = -3
ERROR_DEVICE_LOST = -4
ERROR_FORMAT_NOT_SUPPORTED = -11

RUN_ROI = 1 << 0
RUN_CREATE_NODES = 1 << 1
RUN_ALLOC = 1 << 2
RUN_RECORD_CMD_BUF = 1 << 3
RUN_UPLOAD_SOURCE = 1 << 4
RUN_DOWNLOAD_SINK = 1 << 5
RUN_WAIT_DONE = 1 << 6
RUN_ALL = 0xFFFFFFFF


class ImgParam(C.Structure):
    """dt_image_params_t subset (src/pipe/module.h:72-109)"""
    _fields_ = [
        ("black", C.c_float * 4),
        ("white", C.c_float * 4),
        ("whitebalance", C.c_float * 4),
        ("filters", C.c_uint32),
        ("crop_aabb", C.c_uint32 * 4),
        ("cam_to_rec2020", C.c_float * 9),
        ("noise_a", C.c_float),
        ("noise_b", C.c_float),
        ("orientation", C.c_uint32),
    ]


class NodeInfo(C.Structure):
    _fields_ = [
        ("name", C.c_uint64),
        ("kernel", C.c_uint64),
        ("wd", C.c_uint32),
        ("ht", C.c_uint32),
        ("dp", C.c_uint32),
        ("fused", C.c_uint32),
    ]


class NodeDesc(C.Structure):
    """vkdt_cuda_node_desc_t: a scheduler node with its module's uniform block"""
    _fields_ = [("name", C.c_uint64), ("kernel", C.c_uint64), ("wd", C.c_int32), ("ht", C.c_int32), ("dp", C.c_int32),
                ("push_size", C.c_uint32), ("push", C.c_void_p), ("uniform_size", C.c_uint32), ("uniform", C.c_void_p)]


class Scene(C.Structure):
    _fields_ = [
        ("wd", C.c_int32),
        ("ht", C.c_int32),
        ("seed", C.c_uint32),
        ("image_id", C.c_uint32),
        ("filters", C.c_uint32),
        ("black", C.c_float),
        ("white", C.c_float),
        ("noise_a", C.c_float),
        ("noise_b", C.c_float),
        ("wb", C.c_float * 3),
        ("pan_x", C.c_float),
        ("pan_y", C.c_float),
    ]


class ServerCfg(C.Structure):
    _fields_ = [("cfg", C.c_char_p), ("cfg_len", C.c_size_t), ("slots", C.c_int), ("hbm_cap", C.c_uint64),
                ("llap_levels", C.c_int)]


class Job(C.Structure):
    _fields_ = [("wd", C.c_int), ("ht", C.c_int), ("ip", ImgParam), ("out_wd", C.c_int), ("out_ht", C.c_int),
                ("src", C.c_void_p), ("dst", C.c_void_p), ("src_on_device", C.c_int), ("dst_on_device", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("failed", C.c_uint64), ("mpix", C.c_double),
                ("latency_p50_ms", C.c_double), ("latency_p99_ms", C.c_double),
                ("peak_device_bytes", C.c_uint64), ("graphs", C.c_int)]


# every symbol the header declares, with its ctypes signature
_P = C.c_void_p
_SIGS = {
    "vkdt_cuda_init": (C.c_int, [C.c_int, C.c_uint32]),
    "vkdt_cuda_cleanup": (None, []),
    "vkdt_cuda_supports": (C.c_int, [C.c_uint64, C.c_uint64]),
    "vkdt_cuda_graph_create": (C.c_int, [C.POINTER(_P)]),
    "vkdt_cuda_graph_destroy": (None, [_P]),
    "vkdt_cuda_graph_read_config": (C.c_int, [_P, C.c_char_p, C.c_size_t]),
    "vkdt_cuda_graph_unsupported": (C.c_int, [_P, C.POINTER(C.c_uint64), C.c_int]),
    "vkdt_cuda_graph_set_param": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_uint64, _P, C.c_size_t]),
    "vkdt_cuda_graph_get_param": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_uint64, _P, C.c_size_t]),
    "vkdt_cuda_graph_set_input": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(ImgParam)]),
    "vkdt_cuda_graph_set_output_size": (C.c_int, [_P, C.c_int, C.c_int]),
    "vkdt_cuda_graph_set_llap_levels": (C.c_int, [_P, C.c_int]),
    "vkdt_cuda_graph_create_nodes": (C.c_int, [_P]),
    "vkdt_cuda_graph_alloc": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "vkdt_cuda_graph_node_count": (C.c_int, [_P]),
    "vkdt_cuda_graph_node": (C.c_int, [_P, C.c_int, C.POINTER(NodeInfo)]),
    "vkdt_cuda_graph_output_size": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "vkdt_cuda_graph_map_source": (_P, [_P, C.POINTER(C.c_size_t)]),
    "vkdt_cuda_graph_map_sink": (_P, [_P, C.POINTER(C.c_size_t)]),
    "vkdt_cuda_graph_device_buffers": (C.c_int, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "vkdt_cuda_graph_run": (C.c_int, [_P, _P, C.c_uint32]),
    "vkdt_cuda_graph_wait": (C.c_int, [_P, C.c_uint32]),
    "vkdt_cuda_graph_develop": (C.c_int, [_P, _P, _P, _P]),
    "vkdt_cuda_graph_develop_static": (C.c_int, [_P, _P, _P, _P]),
    "vkdt_cuda_graph_set_capture": (C.c_int, [_P, C.c_int]),
    "vkdt_cuda_graph_stream": (_P, [_P]),
    "vkdt_cuda_graph_plan_bytes": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "vkdt_cuda_unpack_mlv": (C.c_int, [_P, C.c_size_t, C.c_int, C.c_int, C.c_int, _P, _P]),
    "vkdt_cuda_mcraw_scratch_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "vkdt_cuda_mcraw_decode": (C.c_int, [_P, _P, _P, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         _P, _P, _P]),
    "vkdt_cuda_colenc": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P]),
    "vkdt_cuda_bc1_encode": (C.c_int, [_P, C.c_int, C.c_int, _P, _P]),
    "vkdt_cuda_rawhist_scratch_bytes": (C.c_size_t, []),
    "vkdt_cuda_rawhist": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(ImgParam), C.c_int, _P, C.POINTER(C.c_double), _P]),
    "vkdt_cuda_nprof_fit": (C.c_int, [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "vkdt_cuda_server_create": (C.c_int, [C.POINTER(ServerCfg), C.POINTER(_P)]),
    "vkdt_cuda_server_submit": (C.c_int, [_P, C.POINTER(Job), C.POINTER(C.c_uint64)]),
    "vkdt_cuda_server_wait": (C.c_int, [_P, C.c_uint64, C.c_uint32]),
    "vkdt_cuda_server_drain": (C.c_int, [_P, C.c_uint32]),
    "vkdt_cuda_server_job_times": (C.c_int, [_P, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "vkdt_cuda_server_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "vkdt_cuda_server_reset_stats": (C.c_int, [_P]),
    "vkdt_cuda_server_destroy": (None, [_P]),
    "vkdt_cuda_graph_set_timing": (C.c_int, [_P, C.c_int]),
    "vkdt_cuda_graph_query_times": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int]),
    "vkdt_cuda_graph_set_hist": (C.c_int, [_P, C.c_int]),
    "vkdt_cuda_graph_hist": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "vkdt_cuda_hist_rgba_f16": (C.c_int, [_P, C.c_int, C.c_int, _P, _P]),
    "vkdt_cuda_waveform_rgba_f16": (C.c_int, [_P, C.c_int, C.c_int, _P, C.c_int, C.c_int, _P]),
    "vkdt_cuda_lens_rgba_f16": (C.c_int, [_P, C.c_int, C.c_int, _P, C.c_int, C.c_int, C.POINTER(C.c_float), _P]),
    "vkdt_cuda_graph_set_debug": (C.c_int, [_P, C.c_int]),
    "vkdt_cuda_graph_debug_stage": (C.c_int, [_P, C.c_int, C.POINTER(C.c_float), C.c_size_t]),
    "vkdt_cuda_graph_debug_stage_size": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "vkdt_cuda_graph_set_nodes": (C.c_int, [_P, C.c_int, C.c_int, _P, C.c_int]),
    "vkdt_cuda_graph_debug_decisions": (C.c_int, [_P, C.c_int, _P, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "vkdt_cuda_scene_generate": (C.c_int, [C.POINTER(Scene), _P, _P]),
    "vkdt_cuda_scene_generate_host": (C.c_int, [C.POINTER(Scene), C.POINTER(C.c_uint16)]),
    "vkdt_cuda_last_error": (C.c_char_p, []),
}

_lib = None


def lib():
    """Load libvkdt_cuda.so (raises if it is missing: there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libvkdt_cuda.so is not built (run __graft_entry__.build() or vkdt_gb300/build.py)")
    l = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(l, name)
        f.restype = res
        f.argtypes = args
    _lib = l
    return l


def declared_symbols(header=None):
    """Function names declared in include/vkdt_cuda.h."""
    import re
    header = header or os.path.join(os.path.dirname(HERE), "include", "vkdt_cuda.h")
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(vkdt_cuda_\w+)\s*\(", txt)))


class VkdtError(RuntimeError):
    def __init__(self, code, where):
        msg = lib().vkdt_cuda_last_error().decode(errors="replace")
        super().__init__("%s failed with %d: %s" % (where, code, msg))
        self.code = code


def check(code, where):
    if code != SUCCESS:
        raise VkdtError(code, where)
    return code


def token(s):
    """dt_token (src/pipe/token.h): up to 8 chars packed little endian."""
    b = s.encode()[:8]
    v = 0
    for i, c in enumerate(b):
        v |= c << (8 * i)
    return v


def token_str(t):
    return int(t).to_bytes(8, "little").rstrip(b"\0").decode(errors="replace")
