"""CPU tests of the oracle: known-answer tests on its integer and storage
semantics, and agreement of its FP32 and FP64 builds."""
import numpy as np
import pytest

import oracle
import vkdt_gb300 as v

from metrics import delta_e2000, delta_e2000_lab, summary


def test_f16_rounding_kat():
    # IEEE binary16 round to nearest even, including subnormals and overflow
    kat = {
        0.0: 0.0, 1.0: 1.0, 65504.0: 65504.0, 65519.0: 65504.0, 65520.0: np.inf, -65520.0: -np.inf,
        1.0 + 2 ** -11: 1.0,                     # tie -> even
        1.0 + 3 * 2 ** -11: 1.0 + 2 ** -9,       # tie -> even (up)
        2 ** -24: 2 ** -24, 2 ** -25: 0.0,       # smallest subnormal, tie to even zero
        3 * 2 ** -26: 2 ** -24,
        0.1: float(np.float16(0.1)), 1e-5: float(np.float16(1e-5)),
    }
    for x, want in kat.items():
        assert oracle.f16(np.float32(x)) == np.float32(want), x


def test_f16_rounding_matches_numpy():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-70000, 70000, 20000), rng.uniform(-1e-4, 1e-4, 20000),
                        rng.uniform(-2, 2, 20000)]).astype(np.float32)
    got = np.array([oracle.f16(float(a)) for a in x], np.float32)
    assert np.array_equal(got, x.astype(np.float16).astype(np.float32))


def test_noop_exhaustive_u16():
    # denoise/noop.comp: max(0, (v/65535 - b)/(w - b)) stored as f16, all 65536 codes
    codes = np.arange(65536, dtype=np.uint16).reshape(256, 256)
    for black, white in ((512.0, 16383.0), (256.0, 4095.0), (0.0, 65535.0), (2048.0, 15000.0)):
        ip = oracle.img_param(v.default_img_param(black=black, white=white, wd=256, ht=256))
        got = oracle.noop(codes, ip)
        b = np.float32(black / np.float32(65535.0))
        w = np.float32(white / np.float32(65535.0))
        x = codes.astype(np.float32) / np.float32(65535.0)
        want = np.maximum(np.float32(0), (x - b) / (w - b)).astype(np.float16).astype(np.float32)
        assert np.array_equal(got, want), (black, white)


def test_cfa_pattern():
    # bayer rggb at (0,0)
    for y in range(-4, 8):
        for x in range(-4, 8):
            want = 0 if (x % 2 == 0 and y % 2 == 0) else (2 if (x % 2 == 1 and y % 2 == 1) else 1)
            assert oracle.cfa_colour(0x94949494, x, y) == want
    # x-trans 6x6 as demosaic/splat.comp:229-235 draws it (r . b = red, blue; g elsewhere)
    rows = ["GRGGBG", "BGBRGR", "GRGGBG", "GBGGRG", "RGRBGB", "GBGGRG"]
    idx = {"R": 0, "G": 1, "B": 2}
    for y in range(12):
        for x in range(12):
            assert oracle.cfa_colour(9, x, y) == idx[rows[y % 6][x % 6]], (x, y)


def test_hist_bins_constructed():
    # luminances placed at bin centres: l = eotf_filmlight_tlog(lum), bin = uint(256 l + 0.5)
    for b in list(range(1, 256, 7)) + [255]:
        l = b / 256.0
        lum = np.exp((l - 0.5520126568606655) / 0.09232902596577353) - 0.0057048244042473785
        if lum < 0:
            lum = (l - 0.075) / 16.184376489665897
        assert oracle.hist_bin(float(lum), float(lum), float(lum)) == b, b
    assert oracle.hist_bin(-10.0, -10.0, -10.0) == 0
    assert oracle.hist_bin(1e6, 1e6, 1e6) == 255
    # counts on a constructed image: each bin value repeated (bin) times
    vals, want = [], np.zeros(257, np.uint32)
    for b in range(1, 256):
        l = b / 256.0
        lum = np.exp((l - 0.5520126568606655) / 0.09232902596577353) - 0.0057048244042473785
        if lum < 0:
            lum = (l - 0.075) / 16.184376489665897
        vals += [lum] * (b % 5 + 1)
        want[b] += b % 5 + 1
    want[256] = want[:256].sum()
    n = len(vals)
    img = np.zeros((1, n, 4), np.float32)
    img[0, :, 0] = img[0, :, 1] = img[0, :, 2] = vals
    assert np.array_equal(oracle.hist(img), want)


def _scene(wd, ht, seed=0):
    s = v.make_scene(wd, ht, seed=seed)
    m = v.scene_host(s)
    ip = v.default_img_param(wd=wd, ht=ht, noise_a=2.0 / (16383 - 512) ** 2, noise_b=0.4 / (16383 - 512))
    return m, ip


def test_scene_recipe():
    m, _ = _scene(512, 384)
    assert m.dtype == np.uint16
    clipped = (m == 16383).mean()
    assert 0.01 < clipped < 0.03          # the seeded 2% at white
    assert m[m < 16383].max() < 16383
    assert m.min() >= 0


def test_fp32_matches_fp64():
    m, ip = _scene(192, 128, seed=3)
    oip = oracle.img_param(ip)
    a = oracle.develop(m, oip, stages=("colour", "filmcurv", "llap"))
    b = oracle.develop(m, oip, double=True, stages=("colour", "filmcurv", "llap"))
    s = summary(a["colour"], b["colour"])
    assert s["mean"] < 1e-4 and s["flipped_frac"] < 1e-3, s
    de = delta_e2000(a["llap"], b["llap"])
    assert np.percentile(de, 99.9) < 0.5, de.max()


@pytest.mark.parametrize("wd,ht,nl,nh", [(6000, 4000, 12, 10), (2048, 1536, 11, 9), (256, 192, 8, 6)])
def test_pyramid_depths(wd, ht, nl, nh):
    m = np.zeros((ht, wd), np.uint16) + 4000 if wd * ht < 100000 else None
    if m is None:
        pytest.skip("depth arithmetic checked through the library for large sizes")
    r = oracle.develop(m, oracle.img_param(v.default_img_param(wd=wd, ht=ht)), stages=())
    assert r["llap_levels"] == nl and r["hilite_levels"] == nh


# ---------------------------------------------------------------- pinning
# The restatement against the reference's own shaders, compiled for the CPU:
# committed fixtures (tests/golden, written by tests/golden/make_golden.py)
# and, where that build exists here, fresh random cases.

import golden_cases as gc   # noqa: E402


@pytest.mark.parametrize("name", sorted(gc.CASES))
def test_oracle_matches_reference_golden(name):
    m, case, want = gc.load(name)
    wd, ht, filters, seed, white, overrides, stages = case
    ip = oracle.img_param(gc.img_param(v, wd, ht, filters, white))
    got = oracle.develop(m, ip, params=gc.oracle_params(oracle, overrides, wd, ht), stages=stages)
    for s in stages:
        g = got[s] if got[s].ndim == 2 else got[s][..., :3]
        assert g.shape == want[s].shape, (s, g.shape, want[s].shape)
        assert np.array_equal(g, want[s]), (name, s, summary(g if g.ndim == 3 else g[..., None],
                                                             want[s] if want[s].ndim == 3 else want[s][..., None]))


def _ref_available():
    try:
        from oracle import glsl_ref
        return glsl_ref.available()
    except Exception:
        return False


@pytest.mark.skipif(not _ref_available(), reason="reference shaders not compiled here (oracle/_ref)")
@pytest.mark.parametrize("seed", [101, 102, 103, 104, 105, 106, 107, 108, 109])
def test_oracle_matches_reference_shaders_random(seed):
    # 104: rcd; 105: rcd on an x-trans mosaic (the module runs it whatever the pattern);
    # 106: rcd on a cropped bayer mosaic; 107: the half size method on x-trans (resampled)
    from oracle import glsl_ref
    rng = np.random.default_rng(seed)
    filters = gc.XTRANS if seed in (103, 105, 107, 109) else gc.BAYER
    blk = 2 if filters == gc.BAYER else 6
    wd, ht = int(rng.integers(8, 40)) * blk, int(rng.integers(8, 30)) * blk
    m = v.scene_host(v.make_scene(wd, ht, seed=seed, a=gc.NOISE_A, b=gc.NOISE_B, filters=filters))
    ip = oracle.img_param(gc.img_param(v, wd, ht, filters, float(rng.uniform(9000, 16383))))
    p = oracle.default_params()
    p.dn_strength = float(rng.choice([0.0, 0.5, 1.0]))
    p.co_exposure = float(rng.uniform(-1, 1))
    p.ll_clarity = float(rng.uniform(0, 0.6))
    p.dm_method = {104: 1, 105: 1, 106: 1, 107: 2}.get(seed, 0)
    p.dm_colour = {108: 1, 109: 1}.get(seed, 0)     # the wider fix radius (fix.comp:111,124)
    if seed == 106:
        ip.crop_aabb[0], ip.crop_aabb[1], ip.crop_aabb[2], ip.crop_aabb[3] = 4, 2, wd - 6, ht - 4
    st = ("denoise", "hilite", "demosaic", "colour", "filmcurv", "llap")
    a = glsl_ref.develop(m, ip, p, stages=st)
    b = oracle.develop(m, ip, params=p, stages=st)
    for s in st:
        x, y = (a[s], b[s]) if a[s].ndim == 2 else (a[s][..., :3], b[s][..., :3])
        assert np.array_equal(x, y), (seed, wd, ht, s)


@pytest.mark.skipif(not _ref_available(), reason="reference shaders not compiled here (oracle/_ref)")
@pytest.mark.parametrize("seed", [201, 202, 203, 204])
def test_oracle_crop_matches_reference_shader_random(seed):
    # crop/main.comp on random quads, windows and rotations (with the exif quarter and half
    # turns): the oracle's crop stage and what follows it equal the reference's shaders
    from oracle import glsl_ref
    rng = np.random.default_rng(seed)
    filters = gc.XTRANS if seed == 204 else gc.BAYER
    blk = 2 if filters == gc.BAYER else 6
    wd, ht = int(rng.integers(10, 40)) * blk, int(rng.integers(8, 30)) * blk
    m = v.scene_host(v.make_scene(wd, ht, seed=seed, a=gc.NOISE_A, b=gc.NOISE_B, filters=filters))
    ip = oracle.img_param(gc.img_param(v, wd, ht, filters, 16383.0))
    quad = np.array(gc.QUAD) + rng.uniform(-0.06, 0.06, 8)
    win = (1, 3, 3, 7) if seed == 203 else tuple(np.sort(rng.uniform(0, 1, 2)).tolist() + np.sort(rng.uniform(0, 1, 2)).tolist())
    rot = 1337.0 if seed == 203 else float(rng.uniform(-20, 20))
    b, cw, ch = oracle.crop_commit(wd, ht, perspect=quad, crop=win, rotate=rot, orientation=6 if seed == 203 else 0)
    if cw < 4 or ch < 4:
        pytest.skip("window too small")
    p = oracle.set_crop(oracle.default_params(), b, cw, ch)
    st = ("crop", "colour", "llap")
    a = glsl_ref.develop(m, ip, p, stages=st)
    o = oracle.develop(m, ip, params=p, stages=st)
    for s in st:
        assert np.array_equal(a[s][..., :3], o[s][..., :3]), (seed, s)


def test_denoise_nodes_chain_equals_develop():
    # the node-by-node entry fed with its own outputs reproduces the wavelet denoise of the develop
    import vkdt_gb300 as v
    wd, ht = 256, 192
    m = oracle.scene(wd, ht, seed=3, a=8.0, b=1.6)
    ip = oracle.img_param(v.default_img_param(wd=wd, ht=ht, noise_a=8.0 / 15871 ** 2, noise_b=1.6 / 15871))
    op = oracle.default_params()
    op.dn_strength = 1.0
    want = oracle.develop(m, ip, params=op, stages=("denoise",))["denoise"]
    ins = {n: np.zeros((ht // 2, wd // 2, 4), np.float32) for n in oracle.DENOISE_NODES}
    for _ in range(len(oracle.DENOISE_NODES) + 1):
        got = oracle.denoise_nodes(m, ip, op, ins)
        ins = {n: got[n] for n in oracle.DENOISE_NODES}
    assert np.array_equal(got["doub"], want)


def test_stage_injection_reproduces_the_path():
    # the path from each stage on, fed with the oracle's own stage outputs, is the path
    import vkdt_gb300 as v
    wd, ht = 256, 192
    m = oracle.scene(wd, ht, seed=4)
    ip = oracle.img_param(v.default_img_param(wd=wd, ht=ht))
    st = ("denoise", "hilite", "demosaic", "colour", "filmcurv", "llap")
    r = oracle.develop(m, ip, stages=st)
    for s, prev in zip(st[1:], st[:-1]):
        q = oracle.develop(m, ip, stages=(s, "llap"), start=s, input=r[prev])
        assert np.array_equal(q[s], r[s]) and np.array_equal(q["llap"], r["llap"]), s


def test_sensitivity_runs_move_values_by_one_f16_step():
    # a perturbed run rounds stores to a neighbouring f16 value: the denoise/noop output moves by at most one step
    import vkdt_gb300 as v
    wd, ht = 128, 96
    m = oracle.scene(wd, ht, seed=5)
    ip = oracle.img_param(v.default_img_param(wd=wd, ht=ht))
    a = oracle.develop(m, ip, stages=("denoise",))["denoise"]
    b = oracle.develop(m, ip, stages=("denoise",), perturb=7)["denoise"]
    c = oracle.develop(m, ip, stages=("denoise",))["denoise"]
    assert np.array_equal(a, c)                       # the perturbation is off again
    step = np.abs(np.spacing(a.astype(np.float16)).astype(np.float32))
    assert (np.abs(b - a) <= step * 1.0001).all() and (b != a).any()
