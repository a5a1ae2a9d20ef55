"""lens (lens/main.comp): the double sphere lens model with Catmull-Rom
resampling, a node of the reference's darkroom graph (declared in
bin/default-darkroom.i-raw). The library runs it as a standalone node
(vkdt_cuda_lens_rgba_f16).

CPU: the restatement in the oracle equals the reference's shader compiled for
the CPU bit for bit (where the vkdt tree is present) and the committed fixture
made from it (everywhere). GPU: the library's output equals the oracle's within
one f16 step (the sample positions are formed with the shader's IEEE
operations in both; the filter's sums round differently)."""
import numpy as np
import pytest

import golden_cases as gc
import oracle


def _ordered(x):
    """f16 values as integers in the order of the values (one f16 step apart: 1 apart)"""
    i = np.asarray(x, np.float32).astype(np.float16).view(np.int16).astype(np.int32)
    return np.where(i < 0, -(i & 0x7fff), i)


def _ref_available():
    try:
        from oracle import glsl_ref
        return glsl_ref.available()
    except Exception:
        return False


def test_lens_oracle_matches_golden():
    f = gc.lens_input()
    want = gc.load_lens()
    for k, par in enumerate(gc.LENS_CASES):
        got = oracle.lens(f, par).astype(np.float16)
        assert np.array_equal(got.view(np.uint16), want[k].view(np.uint16)), k


def test_lens_default_is_close_to_identity():
    # centre 0, scale 1, both spheres 0: the model maps every position to itself up to rounding,
    # so the Catmull-Rom filter samples the texel centres
    f = gc.lens_input()
    got = oracle.lens(f)
    assert np.abs(got[..., :3] - f[..., :3]).max() < 2e-3


@pytest.mark.skipif(not _ref_available(), reason="reference shaders not compiled here (oracle/_ref)")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_lens_oracle_matches_reference_shader(seed):
    from oracle import glsl_ref as gr
    rng = np.random.default_rng(seed)
    wd, ht = 44 + 3 * seed, 30 + seed
    f = rng.uniform(-0.05, 1.3, (ht, wd, 4)).astype(np.float16).astype(np.float32)
    par = (rng.uniform(-0.05, 0.05), rng.uniform(-0.05, 0.05), rng.uniform(0.8, 1.2), rng.uniform(0.8, 1.2),
           rng.uniform(-0.5, 0.6), rng.uniform(-0.5, 0.6), 1.0 if seed == 1 else rng.uniform(0.98, 1.02),
           1.0 if seed == 1 else rng.uniform(0.98, 1.02))
    src, dst = gr.Img(wd, ht, 4), gr.Img(wd, ht, 4)
    src.a[...] = f
    gr.run("lens_main", wd, ht, {0: src, 1: dst}, uniform=gr.f32(*par))
    got = oracle.lens(f, par).astype(np.float16)
    assert np.array_equal(got.view(np.uint16), dst.a.astype(np.float16).view(np.uint16))


def _gpu_lens(v, img, par, out_size=None):
    import torch
    ht, wd = img.shape[:2]
    owd, oht = out_size or (wd, ht)
    d = torch.from_numpy(np.ascontiguousarray(img.astype(np.float16)).view(np.uint16)).cuda()
    out = torch.full((oht, owd, 4), 0x7e00, dtype=torch.int16, device="cuda")   # f16 NaN: every texel written
    v.lens(d.data_ptr(), wd, ht, out.data_ptr(), par, owd, oht)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.float16).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(len(gc.LENS_CASES)))
def test_lens_gpu_fixture(gpu, k):
    # the fixture's cases against the reference shader's stored output
    f = gc.lens_input()
    got = _gpu_lens(gpu, f, gc.LENS_CASES[k])
    want = gc.load_lens()[k].astype(np.float32)
    steps = np.abs(_ordered(got) - _ordered(want))
    print("lens case %d: max %d f16 steps, %d of %d values differ" % (k, steps.max(), (steps > 0).sum(), steps.size))
    assert steps.max() <= 1
    assert np.array_equal(got[..., 3], np.ones_like(got[..., 3]))


@pytest.mark.gpu
@pytest.mark.parametrize("wd,ht,seed", [(6000, 4000, 1), (1001, 667, 2), (17, 9, 3)])
def test_lens_gpu_random(gpu, wd, ht, seed):
    # an image of the path's output size and odd sizes, parameters across their ranges, against the oracle
    rng = np.random.default_rng(seed)
    img = rng.uniform(-0.05, 1.3, (ht, wd, 4)).astype(np.float16).astype(np.float32)
    par = (rng.uniform(-0.05, 0.05), rng.uniform(-0.05, 0.05), rng.uniform(0.8, 1.2), rng.uniform(0.8, 1.2),
           rng.uniform(-0.5, 0.6), rng.uniform(-0.5, 0.6), rng.uniform(0.98, 1.02), rng.uniform(0.98, 1.02))
    got = _gpu_lens(gpu, img, par)
    want = oracle.lens(img, par)
    steps = np.abs(_ordered(got) - _ordered(want))
    print("lens %dx%d: max %d f16 steps, %d of %d values differ" % (wd, ht, steps.max(), (steps > 0).sum(), steps.size))
    assert steps.max() <= 1


@pytest.mark.gpu
def test_lens_gpu_other_output_size(gpu):
    # the shader takes its aspect and positions from the output image's size
    f = gc.lens_input()
    par = gc.LENS_CASES[2]
    got = _gpu_lens(gpu, f, par, out_size=(40, 50))
    want = oracle.lens(f, par, out_size=(40, 50))
    assert np.abs(_ordered(got) - _ordered(want)).max() <= 1
