"""Noise statistics (rawhist/collect.comp) and the noise profile fit
(nprof/main.c). The GPU statistics equal the oracle's exactly: integer bin
counts and 64-bit fixed point sums. The fit is host code: on flat mosaics with
a known Poisson-Gaussian profile it recovers the profile the way the
reference's estimator sees it (the green-pair variance mom2 - mean^2 of n
samples has expectation sigma^2 (n-1)/n: half of it for the two greens of a
bayer block, 4/5 for the five of an x-trans block)."""
import numpy as np
import pytest

import oracle
import vkdt_gb300 as v

BAYER, XTRANS = 0x94949494, 9
BLACK, WHITE = 512.0, 16383.0


def flat_mosaic(wd, ht, a_dn, b_dn, seed, black=BLACK, white=WHITE):
    """a smooth ramp (no structure a green pair would see) with Poisson-Gaussian noise in DN"""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, wd)[None, :]
    y = np.linspace(0.0, 1.0, ht)[:, None]
    dn = (0.01 + 0.85 * (0.7 * x + 0.3 * y)) * (white - black)
    noisy = b_dn * rng.poisson(dn / b_dn) + rng.normal(0.0, np.sqrt(a_dn), dn.shape)
    return np.clip(np.round(black + noisy), 0, white).astype(np.uint16)


@pytest.mark.parametrize("a_dn,b_dn", [(8.0, 1.6), (16.0, 3.0), (2.0, 0.4)])
@pytest.mark.parametrize("filters,factor", [(BAYER, 0.5), (XTRANS, 0.8)])
def test_nprof_fit_recovers_the_profile(a_dn, b_dn, filters, factor):
    m = flat_mosaic(2040, 1530, a_dn, b_dn, seed=int(a_dn * 10))
    h = oracle.rawhist(m, filters, BLACK, WHITE)
    a, b, ok = v.nprof_fit(h)
    assert ok
    b_norm = b_dn / (WHITE - BLACK)
    assert abs(b / (factor * b_norm) - 1.0) < 0.1, (b, factor * b_norm)   # a statistical fit
    assert a >= 0.0


def test_nprof_fit_without_data_uses_the_default():
    a, b, ok = v.nprof_fit(np.zeros((3, 1000)))
    assert not ok and (a, b) == (100.0, 1.0)


def test_rawhist_oracle_counts_every_block():
    m = flat_mosaic(640, 480, 8.0, 1.6, seed=2)
    h = oracle.rawhist(m, BAYER, BLACK, WHITE)
    assert h[0].sum() == (640 // 2) * (480 // 2)          # every block lands in a bin below 1000
    mean = h[1].sum() / h[0].sum()
    g = (m[0::2, 1::2].astype(np.float64) + m[1::2, 0::2]) / 2.0
    want = np.clip((g / 65535.0 - 512 / 65536.0) / (16383 / 65536.0 - 512 / 65536.0), 0, 1).mean()
    assert abs(mean - want) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["flat", "scene"])
@pytest.mark.parametrize("filters", [BAYER, XTRANS])
@pytest.mark.parametrize("bins", [1000, 333])
def test_rawhist_gpu_equals_oracle(gpu, kind, filters, bins):
    import torch
    wd, ht = 1206, 798
    if kind == "flat":
        m = flat_mosaic(wd, ht, 8.0, 1.6, seed=5)
    else:
        m = v.scene_host(v.make_scene(wd, ht, seed=9, filters=filters))
    d = torch.from_numpy(m.view(np.int16)).cuda()
    torch.cuda.synchronize()
    ip = v.default_img_param(wd=wd, ht=ht, filters=filters, black=BLACK, white=WHITE)
    got = v.rawhist(d.data_ptr(), wd, ht, ip, bins=bins)
    want = oracle.rawhist(m, filters, BLACK, WHITE, bins=bins)
    assert np.array_equal(got, want)


# ---------------------------------------------------------------- pinned to the reference

def test_nprof_fit_equals_the_reference_module():
    # tests/golden/nprof.json: the reference's own nprof/main.c (write_sink) fit of the same
    # histograms, as it prints them ("%g %g"); the library's fit prints the same
    import json
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    import make_nprof
    for rec in json.load(open(os.path.join(here, "nprof.json"))):
        a, b, ok = v.nprof_fit(make_nprof.histogram(tuple(rec["case"])))
        assert ["%g" % a, "%g" % b] == rec["ab"], (rec, a, b)


def test_nprof_fixture_is_what_the_module_emits_now():
    from oracle.modules import build as MB
    import os
    if not os.path.isdir(MB.MODULES_DIR) or not MB.build():
        pytest.skip("no vkdt tree here")
    from oracle import modules as M
    import json
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    import make_nprof
    for rec in json.load(open(os.path.join(here, "nprof.json"))):
        assert list(M.nprof(make_nprof.histogram(tuple(rec["case"])))) == rec["ab"]


@pytest.mark.parametrize("filters", [BAYER, XTRANS])
def test_oracle_rawhist_equals_the_reference_shader(filters):
    # rawhist/collect.comp compiled for the CPU: the counts bit for bit, the float atomic sums to their
    # rounding (the shader adds floats in any order)
    from oracle import glsl_ref
    if not glsl_ref.available():
        pytest.skip("reference shaders not built (oracle/_ref)")
    wd, ht = (600, 400) if filters == BAYER else (606, 402)
    m = oracle.scene(wd, ht, seed=5, a=8.0, b=1.6, filters=filters)
    ip = oracle.img_param(v.default_img_param(wd=wd, ht=ht, filters=filters))
    ref = glsl_ref.rawhist(m, ip)
    ours = oracle.rawhist(m, filters, BLACK, WHITE)
    assert np.array_equal(ref[0], ours[0])
    assert np.allclose(ref[1:], ours[1:], rtol=1e-5, atol=1e-4)
