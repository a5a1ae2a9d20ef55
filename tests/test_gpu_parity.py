"""GPU parity of the CUDA path against the CPU oracle, through the C-ABI.

Every case is held to the tolerance of tests/parity.py at every pixel of the
denoise, hilite, demosaic, colour, filmcurv and llap outputs: max
|a-b|/max(1,|b|) <= 2e-3, mean <= 1e-4, CIEDE2000 < 0.5 after filmcurv and at
the llap output, against the oracle run with the CUDA path's discrete
decisions, each of which is shown to be the reference's own decision on the
CUDA path's input or a near tie. Integer work is bit exact: the denoise/noop
normalisation of every mosaic value, the histogram bins of the colour output.
Each case prints (and appends to $VKDT_PARITY_LOG) its errors per stage.

Sizes: the 2048x1536 and 6000x4000 mosaics are the two single image
configurations the benchmark is quoted on (2 and 8 DN^2 noise recipes), the
latter at the forced 6 llap levels and at the reference's automatic depth, each
with denoise off and at strength 1.
"""
import numpy as np
import pytest

import oracle
import parity as P
import vkdt_gb300 as v

pytestmark = pytest.mark.gpu

BAYER = 0x94949494


def scene(wd, ht, seed, a=2.0, b=0.4, filters=BAYER):
    m = v.scene_host(v.make_scene(wd, ht, seed=seed, a=a, b=b, filters=filters))
    ip = v.default_img_param(wd=wd, ht=ht, filters=filters, noise_a=a / (16383 - 512) ** 2, noise_b=b / (16383 - 512))
    return m, ip


def graph_setup(op):
    """The graph calls that give the C-ABI path the oracle parameters `op`."""
    d = oracle.default_params()

    def setup(g):
        if op.dn_strength != d.dn_strength:
            g.set_param("denoise", "strength", float(op.dn_strength))
        if op.dm_method != d.dm_method:
            g.set_param("demosaic", "method", np.int32(op.dm_method))
        if op.dm_colour != d.dm_colour:
            g.set_param("demosaic", "colour", np.int32(op.dm_colour))
        if op.ll_levels:
            g.set_llap_levels(op.ll_levels)
        if op.out_wd:
            g.set_output_size(op.out_wd, op.out_ht)
        for mod, name, f in (("colour", "exposure", "co_exposure"), ("llap", "clarity", "ll_clarity"),
                             ("filmcurv", "contrast", "fc_contrast"), ("hilite", "white", "hl_white")):
            if getattr(op, f) != getattr(d, f):
                g.set_param(mod, name, float(getattr(op, f)))
        if op.fc_colour != d.fc_colour:
            g.set_param("filmcurv", "colour", np.int32(op.fc_colour))
    return setup


def params(**kw):
    op = oracle.default_params()
    for k, val in kw.items():
        setattr(op, k, val)
    return op


def run(name, m, ip, op, hist=False, **kw):
    g = P.develop_gpu(v, m, ip, setup=graph_setup(op), hist=hist)
    return g, P.check(name, v, m, ip, op, g, **kw)


@pytest.mark.parametrize("wd,ht", [(256, 192), (1000, 742), (2048, 1536)])
def test_default_graph(gpu, wd, ht):
    m, ip = scene(wd, ht, seed=wd)
    g, rec = run("default_%dx%d" % (wd, ht), m, ip, params(), hist=True)
    # integer normalisation: bit exact
    assert np.array_equal(g["denoise"], oracle.noop(m, oracle.img_param(ip)))


def test_config0_denoise(gpu):
    # the 2048x1536 recipe with the wavelet denoise at strength 1
    m, ip = scene(2048, 1536, seed=2048)
    run("config0_denoise", m, ip, params(dn_strength=1.0), hist=True)


@pytest.mark.parametrize("levels,strength", [(6, 0.0), (0, 0.0), (6, 1.0), (0, 1.0)])
def test_config1_24mp(gpu, levels, strength):
    # the 24 MP darkroom recipe the benchmark times: 6 llap levels, and the
    # reference's automatic depth (12 at this size), denoise off and on
    m, ip = scene(6000, 4000, seed=6001, a=8.0, b=1.6)
    g, rec = run("config1_l%d_s%g" % (levels, strength), m, ip, params(ll_levels=levels, dn_strength=strength),
                 hist=True)
    assert rec["levels"] == (levels or 12)


def test_small_and_odd_tiles(gpu):
    # sizes that are not multiples of the 32 px tile, down to the 16 px minimum
    for wd, ht in ((16, 16), (34, 18), (66, 130)):
        m, ip = scene(wd, ht, seed=3)
        g, _ = run("small_%dx%d" % (wd, ht), m, ip, params())
        assert np.array_equal(g["denoise"], oracle.noop(m, oracle.img_param(ip)))


def test_forced_llap_depth(gpu):
    m, ip = scene(512, 384, seed=11)
    run("llap6_512x384", m, ip, params(ll_levels=6))


def test_parameters(gpu):
    m, ip = scene(384, 256, seed=5)
    run("params_384x256", m, ip, params(co_exposure=0.7, ll_clarity=0.0, fc_colour=1, fc_contrast=1.5, hl_white=0.9))


@pytest.mark.parametrize("wd,ht", [(1000, 742), (2048, 1536)])
def test_wavelet_denoise(gpu, wd, ht):
    # denoise strength 1: the wavelet nodes (half, downcov, down x3, assemble, doub)
    # before the rest of the path; the noisier profile of the 24 MP recipe
    m, ip = scene(wd, ht, seed=wd + 1, a=8.0, b=1.6)
    run("wavelet_%dx%d" % (wd, ht), m, ip, params(dn_strength=1.0))


@pytest.mark.parametrize("wd,ht,strength", [(606, 402, 0.0), (1206, 798, 0.0), (606, 402, 1.0), (611, 397, 0.0)])
def test_xtrans(gpu, wd, ht, strength):
    # x-trans 6x6 CFA through the per-node chain: hilite on 3x3 blocks, demosaic gauss/splat/fix
    m, ip = scene(wd, ht, seed=wd + 7, filters=9)
    g, _ = run("xtrans_%dx%d_s%g" % (wd, ht, strength), m, ip, params(dn_strength=strength), hist=True)
    if strength == 0.0:
        assert np.array_equal(g["denoise"], oracle.noop(m, oracle.img_param(ip)))


@pytest.mark.parametrize("wd,ht,strength", [(1024, 768, 0.0), (600, 400, 0.0), (130, 78, 0.0), (2000, 1332, 0.0),
                                            (606, 402, 1.0)])
def test_rcd(gpu, wd, ht, strength):
    # demosaic method 1 (rcd_conv + rcd_fill, the default of the raw video graphs): on the same
    # input the demosaic output equals the oracle's bit for bit (IEEE arithmetic in the shader's
    # order, the reference's 58x26 tiles with zero reads past the shared tile); the path end to
    # end within the tolerance
    m, ip = scene(wd, ht, seed=wd + 3)
    g, _ = run("rcd_%dx%d_s%g" % (wd, ht, strength), m, ip, params(dm_method=1, dn_strength=strength), hist=True)
    want = oracle.rcd(g["hilite"], [ip.whitebalance[k] for k in range(3)])
    assert np.array_equal(g["demosaic"], want)


@pytest.mark.parametrize("case", ["xtrans", "crop"])
def test_rcd_variants(gpu, case):
    # rcd on an x-trans mosaic (the reference module runs it whatever the pattern) and on a
    # cropped bayer window: the rcd kernels bit for bit on the path's own hilite output, the
    # path end to end within the tolerance
    filters = 9 if case == "xtrans" else BAYER
    wd, ht = (606, 402) if case == "xtrans" else (1000, 742)
    m, ip = scene(wd, ht, seed=wd + 11, filters=filters)
    if case == "crop":
        ip.crop_aabb[0], ip.crop_aabb[1], ip.crop_aabb[2], ip.crop_aabb[3] = 8, 6, 992, 738
    g, _ = run("rcd_" + case, m, ip, params(dm_method=1))
    want = oracle.rcd(g["hilite"], [ip.whitebalance[k] for k in range(3)])
    assert np.array_equal(g["demosaic"], want)


@pytest.mark.parametrize("filters,wd,ht", [(BAYER, 1000, 742), (9, 606, 402)])
def test_wide_fix_radius(gpu, filters, wd, ht):
    # demosaic colour param 1: the fix radius clamp(fixup+1, 1, 2) = 2 on bayer (the node chain:
    # gauss, splat, fix as separate kernels) and clamp(fixup+2, 2, 3) = 3 on x-trans
    m, ip = scene(wd, ht, seed=wd + 13, filters=filters)
    run("fix_radius_%dx%d_%d" % (wd, ht, filters == 9), m, ip, params(dm_colour=1), hist=True)


def test_halfsize_method(gpu):
    # demosaic method 2: the half size demosaic at the module's half output size
    m, ip = scene(1000, 742, seed=5)
    g, _ = run("halfsize_1000x742", m, ip, params(dm_method=2))
    assert g["llap"].shape == (371, 500, 4)


@pytest.mark.parametrize("wd,ht,ow,oh,filters", [(1000, 742, 250, 185, BAYER), (2048, 1536, 256, 192, BAYER),
                                                 (1000, 742, 333, 247, BAYER), (606, 402, 101, 67, 9),
                                                 (1206, 798, 150, 99, 9)])
def test_thumbnail(gpu, wd, ht, ow, oh, filters):
    # reduced output size: denoise and hilite at full size, demosaic/halfsize (+ shared/resample
    # with the catmull-rom taps unless the scale is the block), the rest at the output size
    m, ip = scene(wd, ht, seed=ow, filters=filters)
    run("thumb_%dx%d_%dx%d_%d" % (wd, ht, ow, oh, filters == 9), m, ip, params(out_wd=ow, out_ht=oh))


@pytest.mark.parametrize("strength", [0.0, 1.0])
def test_fp64_reference_error(gpu, strength):
    # the error of the CUDA path against the FP64 build of the same restatement (the
    # decisions that differ from the FP64 build's own are forced there the same way)
    m, ip = scene(2048, 1536, seed=21)
    run("fp64_2048x1536_s%g" % strength, m, ip, params(dn_strength=strength), double=True)


def test_reference_shaders_2048(gpu):
    # the reference's own shaders compiled for the CPU on the 2048x1536 recipe: they give the
    # oracle's results bit for bit, and the CUDA path meets the tolerance against them
    from oracle import glsl_ref
    if not glsl_ref.available():
        pytest.skip("reference shaders not built (oracle/_ref)")
    m, ip = scene(2048, 1536, seed=2049)
    stages = ("denoise", "hilite", "demosaic", "colour", "filmcurv", "llap")
    ref = glsl_ref.develop(m, oracle.img_param(ip), oracle.default_params(), stages=stages)
    own = oracle.develop(m, oracle.img_param(ip), stages=stages)
    for s in stages:
        if s in ref:
            assert np.array_equal(ref[s], own[s]), s
    run("reference_shaders_2048x1536", m, ip, params(), hist=True)


def test_histogram_bit_exact_standalone(gpu):
    import torch
    rng = np.random.default_rng(0)
    img = rng.uniform(-0.05, 3.0, size=(300, 420, 4)).astype(np.float16)
    img[..., 3] = 1
    d = torch.from_numpy(img.view(np.uint16)).cuda()
    h = torch.zeros(257, dtype=torch.int32, device="cuda")
    v._lib.check(v._lib.lib().vkdt_cuda_hist_rgba_f16(d.data_ptr(), 420, 300, h.data_ptr(), 0), "hist")
    torch.cuda.synchronize()
    want = oracle.hist(img.astype(np.float32))
    assert np.array_equal(h.cpu().numpy().view(np.uint32), want)


def test_deterministic_and_device_entry(gpu):
    import torch
    wd, ht = 640, 480
    m, ip = scene(wd, ht, seed=9)
    with v.Graph() as g:
        g.set_input(wd, ht, ip)
        g.alloc()
        a = g.run(m).copy()
        b = g.run(m).copy()
        assert np.array_equal(a.view(np.uint16), b.view(np.uint16))
        dm = torch.from_numpy(m.view(np.int16)).cuda()
        do = torch.zeros((ht, wd, 4), dtype=torch.float16, device="cuda")
        g.develop(dm.data_ptr(), do.data_ptr())
        g.wait()
        assert np.array_equal(do.cpu().numpy().view(np.uint16), a.view(np.uint16))


def test_debug_stages_do_not_change_the_result(gpu):
    # the debug copies and decision maps are written beside the production outputs
    wd, ht = 640, 480
    m, ip = scene(wd, ht, seed=19)
    with v.Graph() as g:
        g.set_input(wd, ht, ip)
        g.alloc()
        a = g.run(m).copy()
    b = P.develop_gpu(v, m, ip)["llap"].astype(np.float16)
    assert np.array_equal(a.view(np.uint16), b.view(np.uint16))


def test_timing_reports_every_launch(gpu):
    wd, ht = 512, 384
    m, ip = scene(wd, ht, seed=2)
    with v.Graph() as g:
        g.set_input(wd, ht, ip)
        g.set_timing(True)
        g.alloc()
        g.run(m)
        t = g.times()
    names = [n for n, _ in t]
    assert names[0] == "hilite:reduce" and names[-1] == "llap:colour" and "demosaic:fix" in names
    assert all(ms >= 0 for _, ms in t)


# ---------------------------------------------------------------- golden
# The committed fixtures hold the reference's own shaders' output (compiled
# for the CPU) on seeded mosaics. The oracle reproduces them bit for bit
# (tests/test_oracle.py); the CUDA path is held to the tolerance against the
# oracle on the same case, with its decisions explained as above.

import golden_cases as gc   # noqa: E402


@pytest.mark.parametrize("name", sorted(gc.CASES))
def test_cuda_matches_reference_golden(gpu, name):
    m, case, want = gc.load(name)
    wd, ht, filters, seed, white, overrides, stages = case
    ip = gc.img_param(v, wd, ht, filters, white)
    op = gc.oracle_params(oracle, overrides, wd, ht)
    # the oracle's own result is the fixture's
    own = oracle.develop(m, oracle.img_param(ip), params=op, stages=tuple(s for s in want if s != "hist"))
    for s in want:
        if s in own:
            a = own[s] if own[s].ndim == 2 else own[s][..., :want[s].shape[-1]]
            assert np.array_equal(a, want[s]), (name, s)
    base = graph_setup(op)

    def setup(g):
        base(g)
        if "crop" in overrides:
            gc.graph_crop(v, g, ip, overrides)
            g.set_input(wd, ht, ip)   # with its exif orientation
    try:
        g = P.develop_gpu(v, m, ip, setup=setup, cfg=v.DARKROOM_CROP_CFG if "crop" in overrides else None)
    except v._lib.VkdtError as e:
        if e.code in (v._lib.ERROR_FORMAT_NOT_SUPPORTED, v._lib.INCOMPLETE):
            pytest.skip("not on the CUDA path: %s" % e)
        raise
    P.check("golden_" + name, v, m, ip, op, g)


# ---------------------------------------------------------------- crop between demosaic and colour
# bin/default-darkroom.i-raw connects crop (crop/main.c, main.comp) after demosaic: at its
# defaults a 3 px margin (nearest texel), or with the exif orientation a half or quarter turn,
# or a perspective quad and a rotation (Catmull-Rom); the stages after it run at its size.

QUAD = (0.25, 0.25, 0.75, 0.25, 0.75, 0.75, 0.25, 0.75)
CROP_CASES = {
    # name: (wd, ht, filters, orientation, perspect, crop window, rotate, oracle overrides)
    "darkroom_2048x1536": (2048, 1536, BAYER, 0, QUAD, (1, 3, 3, 7), 1337, {}),
    "darkroom_6000x4000": (6000, 4000, BAYER, 0, QUAD, (1, 3, 3, 7), 1337, {}),
    "orient6_1000x742": (1000, 742, BAYER, 6, QUAD, (1, 3, 3, 7), 1337, {}),
    "orient3_1000x742": (1000, 742, BAYER, 3, QUAD, (1, 3, 3, 7), 1337, {}),
    "perspective_1024x768": (1024, 768, BAYER, 0, (0.2, 0.22, 0.8, 0.25, 0.77, 0.8, 0.21, 0.75),
                             (0.1, 0.9, 0.05, 0.95), 3.5, {}),
    "window_1000x742": (1000, 742, BAYER, 0, QUAD, (0.13, 0.71, 0.2, 0.9), 0, {}),
    # no rotation but a perspective quad: nearest texels through the homography (the crop kernel)
    "keystone_1000x742": (1000, 742, BAYER, 0, (0.24, 0.25, 0.76, 0.25, 0.75, 0.75, 0.25, 0.75), (0, 1, 0, 1), 0, {}),
    # a window corner on half a texel: the whole texel offsets may differ between columns
    "halftexel_1000x742": (1000, 742, BAYER, 0, QUAD, (0.0035, 0.9, 0.0, 1.0), 0, {}),
    "xtrans_606x402": (606, 402, 9, 0, QUAD, (1, 3, 3, 7), -7.25, {}),
    "rcd_1000x742": (1000, 742, BAYER, 0, QUAD, (1, 3, 3, 7), 1337, {"dm_method": 1}),
    "wavelet_1000x742": (1000, 742, BAYER, 0, QUAD, (0.05, 0.95, 0.0, 1.0), 2.0, {"dn_strength": 1.0}),
}


def crop_case(name):
    wd, ht, filters, orient, persp, win, rot, kw = CROP_CASES[name]
    m, ip = scene(wd, ht, seed=wd + orient + 77, filters=filters)
    ip.orientation = orient
    op = params(**kw)
    blk, cw, ch = oracle.crop_commit(wd, ht, perspect=persp, crop=win, rotate=rot, orientation=orient)
    oracle.set_crop(op, blk, cw, ch)
    base = graph_setup(op)

    def setup(g):
        base(g)
        g.set_param("crop", "perspect", np.array(persp, np.float32))
        g.set_param("crop", "crop", np.array(win, np.float32))
        g.set_param("crop", "rotate", np.float32(rot))
    return m, ip, op, setup, (cw, ch), (win, rot)


@pytest.mark.parametrize("name", sorted(CROP_CASES))
def test_crop(gpu, name):
    m, ip, op, setup, (cw, ch), _ = crop_case(name)
    g = P.develop_gpu(v, m, ip, setup=setup, cfg=v.DARKROOM_CROP_CFG)
    assert g["llap"].shape == (ch, cw, 4)
    assert "crop" in g   # none of the cases is the identity: the crop stage ran
    P.check("crop_" + name, v, m, ip, op, g)


def test_crop_by_whole_texels_rides_on_the_fused_kernel(gpu):
    # without rotation and with the default quad the crop fetches texels (x + 3, y + 3): the
    # fused develop kernel applies it, and the result equals the crop kernel's output fed to
    # the rest of the chain (the oracle with the CUDA path's own crop as colour's input)
    m, ip, op, setup, (cw, ch), _ = crop_case("darkroom_2048x1536")
    with v.Graph(v.DARKROOM_CROP_CFG) as g:
        g.set_input(2048, 1536, ip)
        setup(g)
        g.create_nodes()
        fused = {(n[0], n[1]): n[5] for n in g.nodes()}
    assert fused[("crop", "main")] == fused[("demosaic", "fix")] != fused[("llap", "curve")]
    g = P.develop_gpu(v, m, ip, setup=setup, cfg=v.DARKROOM_CROP_CFG)
    ox, oy = int(round(op.cr_block[16] * 2048)), int(round(op.cr_block[18] * 1536))
    assert (ox, oy) == (3, 3)
    want = oracle.develop(m, oracle.img_param(ip), params=op, stages=("crop",), start="crop",
                          input=g["demosaic"])["crop"]
    assert np.array_equal(g["crop"], want)


def test_crop_identity_has_no_launch(gpu):
    # crop at the identity (no rotation, the whole frame, the default quad) copies its input:
    # the fused path runs, and the result equals the graph without crop
    m, ip = scene(1000, 742, seed=3)

    def setup(g):
        g.set_param("crop", "crop", np.array((0, 1, 0, 1), np.float32))
        g.set_param("crop", "rotate", np.float32(0))
    with v.Graph(v.DARKROOM_CROP_CFG) as g:
        g.set_input(1000, 742, ip)
        setup(g)
        g.alloc()
        a = g.run(m)
        fused = {(n[0], n[1]): n[5] for n in g.nodes()}
        assert fused[("crop", "main")] == fused[("colour", "main")]   # computed by the fused launch
    with v.Graph() as g:
        g.set_input(1000, 742, ip)
        g.alloc()
        b = g.run(m)
    assert np.array_equal(a, b)
