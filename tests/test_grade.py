"""grade after llap (grade/main.comp) and the crop between demosaic and colour,
as the reference's darkroom graph (bin/default-darkroom.i-raw) connects them.

CPU: the grade restatement equals the reference's shader compiled for the CPU
bit for bit (where the vkdt tree is present) and the committed fixture made
from it (everywhere); a graph with crop in the chain is developed only when
crop is the identity, otherwise the library answers VKDT_CUDA_INCOMPLETE (the
caller keeps its own nodes). GPU: the library's graded output equals the
oracle's grade of the library's own llap output within two f16 steps (pow and
log2 as the device evaluates them)."""
import numpy as np
import pytest

import golden_cases as gc
import oracle
import vkdt_gb300 as v
from vkdt_gb300._lib import VkdtError


def _ordered(x):
    """f16 values as integers in the order of the values (one f16 step apart: 1 apart)"""
    i = np.asarray(x, np.float32).astype(np.float16).view(np.int16).astype(np.int32)
    return np.where(i < 0, -(i & 0x7fff), i)


def _cfg(crop=True, grade=True):
    cfg = v.DARKROOM_CFG
    mods = ""
    if crop:
        mods += "module:crop:01:743:400\n"
        cfg = cfg.replace("connect:demosaic:01:output:colour:01:input",
                          "connect:demosaic:01:output:crop:01:input\nconnect:crop:01:output:colour:01:input")
    if grade:
        mods += "module:grade:01:1444:400\n"
        cfg += "connect:llap:01:output:grade:01:input\n"
    return mods + cfg


def test_grade_oracle_matches_golden():
    f = gc.grade_input()
    want = gc.load_grade()
    for k, (lift, gamma, gain, off, mode, sp, hp) in enumerate(gc.GRADE_CASES):
        got = oracle.grade(f, lift, gamma, gain, off, mode, sp, hp).astype(np.float16)
        assert np.array_equal(got.view(np.uint16), want[k].view(np.uint16)), k


def _ref_available():
    try:
        from oracle import glsl_ref
        return glsl_ref.available()
    except Exception:
        return False


@pytest.mark.skipif(not _ref_available(), reason="reference shaders not compiled here (oracle/_ref)")
@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_grade_oracle_matches_reference_shader(seed):
    from oracle import glsl_ref as gr
    rng = np.random.default_rng(seed)
    wd, ht = 40, 24
    f = rng.uniform(-0.05, 1.3, (ht, wd, 4)).astype(np.float16).astype(np.float32)
    lift, off = rng.uniform(-0.2, 0.2, 4), rng.uniform(-0.2, 0.2, 4)
    gamma, gain = 1 + rng.uniform(-0.1, 0.1, 4), 1 + rng.uniform(-0.1, 0.1, 4)
    mode, sp, hp = seed % 2, rng.uniform(0.05, 0.5), rng.uniform(0.2, 0.95)
    src, dst = gr.Img(wd, ht, 4), gr.Img(wd, ht, 4)
    src.a[...] = f
    gr.run("grade_main", wd, ht, {0: src, 1: dst}, uniform=gr.f32(*lift, *gamma, *gain, *off) + gr.i32(mode) + gr.f32(sp, hp))
    got = oracle.grade(f, lift, gamma, gain, off, mode, sp, hp).astype(np.float16)
    assert np.array_equal(got.view(np.uint16), dst.a.astype(np.float16).view(np.uint16))


def test_crop_and_grade_in_the_chain():
    ip = v.default_img_param(wd=420, ht=300)
    with v.Graph(cfg=_cfg()) as g:
        assert "crop" not in g.unsupported() and "grade" not in g.unsupported()
        g.set_input(420, 300, ip)
        # crop/params defaults: rotation from the exif orientation (none here) and a 3 px margin
        # on the sides longer than 400 px
        g.create_nodes()
        nodes = {(n[0], n[1]): (n[2], n[3]) for n in g.nodes()}
        assert nodes[("crop", "main")] == (414, 300) == nodes[("grade", "main")]
        # a crop with a scaled output is not built
        g.set_output_size(210, 150)
        with pytest.raises(VkdtError) as e:
            g.create_nodes()
        assert e.value.code == 5


def _develop(cfg, wd, ht, m, params=()):
    ip = v.default_img_param(wd=wd, ht=ht)
    with v.Graph(cfg=cfg) as g:
        g.set_input(wd, ht, ip)
        for mod, name, val in params:
            g.set_param(mod, name, val)
        g.alloc()
        return g.run(m).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(gc.GRADE_CASES)))
def test_grade_gpu(gpu, case):
    wd, ht = 420, 300
    m = v.scene_host(v.make_scene(wd, ht, seed=11 + case))
    identity_crop = [("crop", "rotate", 0.0), ("crop", "crop", [0.0, 1.0, 0.0, 1.0])]
    plain = _develop(_cfg(crop=True, grade=False), wd, ht, m, identity_crop)
    lift, gamma, gain, off, mode, sp, hp = gc.GRADE_CASES[case]
    params = identity_crop + [("grade", "lift", np.float32(lift)), ("grade", "gamma", np.float32(gamma)),
                              ("grade", "gain", np.float32(gain)), ("grade", "offset", np.float32(off)),
                              ("grade", "mode", np.int32(mode)), ("grade", "sh_pivot", np.float32(sp)),
                              ("grade", "hi_pivot", np.float32(hp))]
    got = _develop(_cfg(crop=True, grade=True), wd, ht, m, params)
    want = oracle.grade(plain, lift, gamma, gain, off, mode, sp, hp)
    steps = np.abs(_ordered(got[..., :3]) - _ordered(want[..., :3]))
    assert steps.max() <= 2 and (steps > 0).mean() <= 0.02, (int(steps.max()), float((steps > 0).mean()))
    assert (got[..., 3] == 1.0).all()
