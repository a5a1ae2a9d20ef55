"""The exact arithmetic shortcuts of the kernels (common.cuh, hilite.cuh):
rcp_f16v must equal the IEEE reciprocal on every input the kernels give it
(all f16 values and their squares), div_ry the IEEE quotient, noop_code
the denoise/noop code table on every u16 code and unorm16_exact the IEEE
quotient v / 65535 of every u16 code. The check is
a small CUDA program built against the kernels' own header; it runs on the
device and compares bit for bit."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _nvcc():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return os.path.join(c, "bin", "nvcc")
    return shutil.which("nvcc")


@pytest.mark.gpu
def test_rcp_f16v_and_div_ry_equal_ieee(tmp_path):
    nvcc = _nvcc()
    assert nvcc, "nvcc not found"
    exe = str(tmp_path / "check_division")
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I" + os.path.join(ROOT, "vkdt_gb300", "csrc"), "-o", exe,
                    os.path.join(HERE, "cuda", "check_division.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 of 65536 f16 values differ, 0 of their squares" in r.stdout, r.stdout
    assert "noop_code: 0 of" in r.stdout, r.stdout
    assert "unorm16_exact: 0 of 65536 codes differ" in r.stdout, r.stdout


@pytest.mark.gpu
def test_paired_fp32_intrinsics_against_scalar(tmp_path):
    # per class of operand, how often the paired forms (add/mul/fma.f32x2) differ from the scalar IEEE
    # operations; and a product followed by a sum, paired throughout (contracted into one fma by the
    # code generator: reported, not asserted) and in the covariance's form
    nvcc = _nvcc()
    assert nvcc, "nvcc not found"
    exe = str(tmp_path / "check_paired")
    subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", exe,
                    os.path.join(HERE, "cuda", "check_paired.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "normal " in r.stdout and "remainder" in r.stdout, r.stdout
    # single paired operations round as the scalar ones; a paired product summed by scalar IEEE adds
    # (the covariance's form) keeps both roundings
    assert "add 0 mul 0 fma 0" in r.stdout and "paired mul, scalar add 0 " in r.stdout, r.stdout
    # the denoise structure tensor: a product by a paired fma with an opaque -0 addend, then a paired add
    assert "paired fma -0, paired add 0 " in r.stdout, r.stdout
