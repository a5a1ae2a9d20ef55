"""Build libvkdt_cuda.so in-tree for sm_103a (nvcc + g++, parallel, no cmake).

Arithmetic is FP32 with contraction (FMA), approximate division and the
hardware exp where a result only feeds continuous arithmetic before its f16
store. The computations whose rounding decides a branch of the reference
(the demosaic covariance and its eigen decomposition, the llap gamma
selection, the luminance, histogram bins, denoise/noop) are written with
explicit IEEE intrinsics in the kernels, so they evaluate exactly as the CPU
oracle does. VKDT_FMAD=false VKDT_NVCC_EXTRA=-prec-div=true VKDT_DEFINES=
builds the fully IEEE variant for comparison.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvkdt_cuda.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["k_hilite.cu", "k_develop.cu", "k_llap.cu", "k_misc.cu", "k_static.cu", "k_denoise.cu", "k_nodes.cu", "k_rawhist.cu", "k_rcd.cu", "k_unpack.cu", "k_mcraw.cu", "k_encode.cu"]
CPP_SOURCES = ["graph.cpp", "server.cpp"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(nv))
    raise RuntimeError("nvcc not found")


def _newer(src_list, out):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in src_list)


def build(verbose=False, force=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "vkdt_cuda.h"))
    inc = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
    jobs, objs = [], []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            fmad = os.environ.get("VKDT_FMAD", "true")
            defs = (os.environ.get("VKDT_DEFINES", "-DVKDT_FAST_EXP").split()
                    + os.environ.get("VKDT_NVCC_EXTRA", "-prec-div=false").split())
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=" + fmad, "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"] + defs + inc + ["-c", src, "-o", obj]
            jobs.append(cmd)
    for f in CPP_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-fvisibility=hidden",
                   "-I" + os.path.join(cuda, "include")] + inc + ["-c", src, "-o", obj]
            jobs.append(cmd)
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in jobs]
    err = False
    for c, p in procs:
        out = p.communicate()[0].decode()
        if p.returncode != 0:
            err = True
            sys.stderr.write("FAILED: %s\n%s\n" % (" ".join(c), out))
        elif verbose and out.strip():
            sys.stderr.write(out)
    if err:
        raise RuntimeError("libvkdt_cuda build failed")
    if force or _newer(objs, LIB):
        cmd = [nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode())
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
