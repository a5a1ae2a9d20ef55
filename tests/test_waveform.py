"""The hist module's rgb waveform (hist/collect.comp) on the GPU, bit exact
against the oracle: integer counts (red +1, green +1024, blue +1048576 per
pixel) in the column int(out_wd/wd * x) and the row of (1 - value) * out_ht +
0.5, negative and NaN values in row 0, values past the last row in the last."""
import numpy as np
import pytest

import oracle


def test_oracle_waveform_known_answer():
    img = np.zeros((2, 3, 4), np.float32)
    img[0, 0, :3] = (0.0, 0.5, 1.0)
    img[1, 2, :3] = (-1.0, 2.0, np.nan)
    w = oracle.waveform(img, wo=6, ho=10)
    want = np.zeros((10, 6), np.uint32)
    zero = 1 + 1024 + 1048576                       # a black pixel: all three counters in the last row
    want[9, 0] = zero + 1                           # (0,0) red 0 -> last row; the black pixel below it
    want[5, 0] = 1024                               # (0,0) green 0.5 -> row 5
    want[0, 0] = 1048576                            # (0,0) blue 1 -> row 0
    want[9, 2] = 2 * zero                           # column x = 1 -> 2 (scale 2)
    want[9, 4] = zero + 1                           # (1,2) red -1 -> clamped to the last row
    want[0, 4] = 1024 + 1048576                     # green 2 -> negative -> row 0; blue NaN -> row 0
    assert np.array_equal(w, want)


@pytest.mark.gpu
@pytest.mark.parametrize("wd,ht,wo,ho", [(6000, 4000, 1000, 600), (1000, 742, 1000, 600), (500, 300, 1000, 600),
                                         (37, 19, 16, 9), (2048, 1536, 490, 300)])
def test_waveform_bit_exact(gpu, wd, ht, wo, ho):
    import torch
    v = gpu
    rng = np.random.default_rng(wd + ht)
    img = rng.uniform(-0.2, 1.3, size=(ht, wd, 4)).astype(np.float16)
    img.reshape(-1, 4)[rng.integers(0, wd * ht, 64), 0] = np.nan
    img.reshape(-1, 4)[rng.integers(0, wd * ht, 64), 2] = np.inf
    img.reshape(-1, 4)[rng.integers(0, wd * ht, 64), 1] = -np.inf
    d = torch.from_numpy(img.view(np.uint16)).cuda()
    out = torch.full((ho, wo), 7, dtype=torch.int32, device="cuda")   # cleared by the call
    for _ in range(2):
        v.waveform(d.data_ptr(), wd, ht, out.data_ptr(), wo, ho)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint32), oracle.waveform(img.astype(np.float32), wo, ho))


@pytest.mark.gpu
def test_waveform_of_a_develop(gpu):
    # the display waveform of the path's output (the darkroom graph's hist module input)
    import torch
    v = gpu
    wd, ht = 2048, 1536
    m = v.scene_host(v.make_scene(wd, ht, seed=4))
    with v.Graph() as g:
        g.set_input(wd, ht, v.default_img_param(wd=wd, ht=ht))
        g.alloc()
        out = g.run(m)
    d = torch.from_numpy(np.ascontiguousarray(out).view(np.uint16)).cuda()
    w = torch.zeros((600, 1000), dtype=torch.int32, device="cuda")
    v.waveform(d.data_ptr(), wd, ht, w.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(w.cpu().numpy().view(np.uint32), oracle.waveform(out.astype(np.float32)))


def test_oracle_waveform_equals_the_reference_shader():
    # hist/collect.comp compiled for the CPU, on values in [0, 1] (its float to unsigned conversion
    # of negative values has no defined result in the C++ the shader is compiled to)
    from oracle import glsl_ref
    if not glsl_ref.available():
        pytest.skip("reference shaders not built (oracle/_ref)")
    rng = np.random.default_rng(1)
    for (ht, wd, wo, ho) in ((90, 130, 64, 40), (300, 420, 1000, 600), (37, 19, 16, 9)):
        img = rng.uniform(0, 1, (ht, wd, 4)).astype(np.float16).astype(np.float32)
        assert np.array_equal(glsl_ref.waveform(img, wo, ho), oracle.waveform(img, wo, ho))
