"""The boundary against the reference's own module host code.

tests/golden/nodes.json holds what the reference's denoise, hilite, demosaic,
colour, filmcurv and llap main.c (compiled unmodified from the vkdt tree,
oracle/modules) emit for a set of graphs: every node with its push constants
and its module's uniform block, after create_nodes and commit_params. These
tests hold the library to it on the CPU: its own create_nodes gives the same
nodes (name, kernel, wd, ht, dp), and vkdt_cuda_graph_set_nodes takes the
reference's nodes as they are, with the parameters the cfg path derives. The
GPU test develops through both and compares the results bit for bit."""
import collections
import os
import sys

import numpy as np
import pytest

import vkdt_gb300 as v

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_nodes as MN   # noqa: E402

CASES = MN.load()
SKIP = {("filmcurv", "dspy")}   # filmcurv's display curve: not on the path


def ref_multiset(case, W, H):
    c = collections.Counter()
    for n in case["nodes"]:
        if (n["name"], n["kernel"]) in SKIP:
            continue
        if (n["name"], n["kernel"]) == ("shared", "resample") and (n["wd"], n["ht"]) == (W, H):
            continue   # the demosaic output resampled to its own size: the identity
        c[(n["name"], n["kernel"], n["wd"], n["ht"], n["dp"])] += 1
    return c


def cfg_graph(case):
    wd, ht = case["in"]
    g = v.Graph(case["cfg"])
    g.set_input(wd, ht, MN.case_ip(wd, ht, case["filters"], case.get("orientation", 0)))
    if case["out"][0]:
        g.set_output_size(*case["out"])
    return g


@pytest.mark.parametrize("name", sorted(CASES))
def test_create_nodes_matches_the_reference_modules(name):
    case = CASES[name]
    with cfg_graph(case) as g:
        g.create_nodes()
        ours = collections.Counter((n[0], n[1], n[2], n[3], n[4]) for n in g.nodes())
    wd, ht = case["in"]
    assert ours == ref_multiset(case, wd, ht), (dict(ours - ref_multiset(case, wd, ht)),
                                                dict(ref_multiset(case, wd, ht) - ours))


@pytest.mark.parametrize("name", sorted(CASES))
def test_set_nodes_takes_the_reference_nodes(name):
    case = CASES[name]
    wd, ht = case["in"]
    with v.Graph(None) as g, cfg_graph(case) as c:
        g.set_nodes(wd, ht, case["nodes"])
        c.create_nodes()
        assert sorted(g.nodes()) == sorted(c.nodes())
        for mod, pars in (("denoise", ("strength", "luma", "detail")), ("hilite", ("white", "desat", "soft")),
                          ("filmcurv", ("light", "contrast", "bias")), ("llap", ("sigma", "shadows", "hilights", "clarity"))):
            for p in pars:
                assert np.array_equal(g.get_param(mod, p), c.get_param(mod, p)), (mod, p)
        for p in ("colour", "method"):
            assert np.array_equal(g.get_param("demosaic", p, dtype=np.int32), c.get_param("demosaic", p, dtype=np.int32))


def test_colour_white_written_back_as_the_reference():
    # colour/main.c:241-253 derives the white from the camera matrix and writes it back into the params
    case = CASES["darkroom_2048x1536"]
    with cfg_graph(case) as g:
        g.create_nodes()
        ours = g.get_param("colour", "white", count=4)[:3]
    ref = np.frombuffer(case["modules"]["colour"], np.float32)
    # the params file order: exposure sat picked matrix gamut clip clipmax temp white[4] ...
    assert np.array_equal(ours, ref[8:11])


CROP = sorted(n for n in CASES if n.startswith("crop_"))


@pytest.mark.parametrize("name", CROP)
def test_crop_written_back_as_the_reference(name):
    # crop/main.c:334-342: with automatic rotation the resolved window and rotation are
    # written back into the params; the output size is its modify_roi_out's
    case = CASES[name]
    with cfg_graph(case) as g:
        g.create_nodes()
        ours = np.concatenate([g.get_param("crop", "crop", count=4), g.get_param("crop", "rotate")])
        size = {(n[0], n[1]): (n[2], n[3]) for n in g.nodes()}
    ref = np.frombuffer(case["modules"]["crop"], np.float32)   # perspect[8] crop[4] rotate
    assert np.array_equal(ours.view(np.uint32), ref[8:13].view(np.uint32))
    want = [(n["wd"], n["ht"]) for n in case["nodes"] if n["name"] == "crop"]
    assert [size[("crop", "main")]] == want and size[("llap", "colour")] == want[0]


def crop_block(nodes):
    return np.frombuffer([n for n in nodes if n["name"] == "crop"][0]["uniform"], np.float32)[:20]


@pytest.mark.parametrize("name", CROP)
def test_crop_block_as_the_reference_commits(name):
    # the oracle's restatement of crop's commit_params gives the reference's block bit for bit
    import oracle
    case = CASES[name]
    wd, ht = case["in"]
    extra = {}
    for line in case["cfg"].split("\n"):
        f = line.split(":")
        if f[0] == "param" and f[1] == "crop":
            extra[f[3]] = [float(x) for x in f[4:]]
    blk, cw, ch = oracle.crop_commit(wd, ht, perspect=extra.get("perspect", MN.QUAD), crop=extra.get("crop", (1, 3, 3, 7)),
                                     rotate=extra.get("rotate", [1337.0])[0], orientation=case["orientation"])
    assert np.array_equal(blk.view(np.uint32), crop_block(case["nodes"]).view(np.uint32)), name
    assert [(cw, ch)] == [(n["wd"], n["ht"]) for n in case["nodes"] if n["name"] == "crop"]


def test_unsupported_chains_return_incomplete():
    case = CASES["darkroom_2048x1536"]
    wd, ht = case["in"]
    nodes = [dict(n) for n in case["nodes"]]
    # a colour block asking for saturation 0.5: not on the CUDA path
    for n in nodes:
        if n["name"] == "colour":
            u = bytearray(n["uniform"])
            u[4 * 226:4 * 227] = np.float32(0.5).tobytes()
            n["uniform"] = bytes(u)
    with v.Graph(None) as g:
        with pytest.raises(v._lib.VkdtError) as e:
            g.set_nodes(wd, ht, nodes)
        assert e.value.code == v._lib.INCOMPLETE
    # a DNG gain map on the denoise node (denoise/main.c:172-196: the noop push constant after the
    # CFA filters, the doub push constant after the noise profile): not built
    for name, node, at in (("darkroom_2048x1536", "noop", 17), ("wavelet_1000x742", "doub", 19)):
        c = CASES[name]
        nodes = [dict(n) for n in c["nodes"]]
        for n in nodes:
            if n["name"] == "denoise" and n["kernel"] == node:
                u = bytearray(n["push"])
                u[4 * at:4 * at + 4] = np.int32(1).tobytes()
                n["push"] = bytes(u)
        with v.Graph(None) as g:
            with pytest.raises(v._lib.VkdtError) as e:
                g.set_nodes(c["in"][0], c["in"][1], nodes)
            assert e.value.code == v._lib.INCOMPLETE and "gain map" in str(e.value)
    # a node the library does not compute (an extra llap level)
    nodes = [dict(n) for n in case["nodes"]] + [dict(case["nodes"][-1], kernel="reduce", wd=2, ht=1, dp=11)]
    with v.Graph(None) as g:
        with pytest.raises(v._lib.VkdtError) as e:
            g.set_nodes(wd, ht, nodes)
        assert e.value.code == v._lib.INCOMPLETE


def test_fixture_is_what_the_reference_modules_emit_now():
    # where the vkdt tree is present: the committed fixture equals a fresh run of the reference's module code
    from oracle import modules as M
    from oracle.modules import build as MB
    if not os.path.isdir(MB.MODULES_DIR) or not MB.build():
        pytest.skip("no vkdt tree here")
    for name, case in CASES.items():
        wd, ht = case["in"]
        nodes, mods = M.run(case["cfg"], wd, ht, MN.case_ip(wd, ht, case["filters"], case.get("orientation", 0)),
                            *case["out"])
        assert [(n["name"], n["kernel"], n["wd"], n["ht"], n["dp"], n["push"]) for n in nodes] == \
               [(n["name"], n["kernel"], n["wd"], n["ht"], n["dp"], n["push"]) for n in case["nodes"]], name
        assert {m["name"]: m["param"] for m in mods} == case["modules"], name


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["darkroom_2048x1536", "wavelet_1000x742", "rcd_1000x742", "thumb_2048x1536",
                                  "xtrans_606x402", "params_384x256", "fixup_1000x742", "crop_2048x1536",
                                  "crop_orient6_1000x742", "crop_persp_1024x768", "crop_orient8_606x402"])
def test_develop_through_set_nodes_equals_cfg(gpu, name):
    case = CASES[name]
    wd, ht = case["in"]
    m = v.scene_host(v.make_scene(wd, ht, seed=wd, filters=case["filters"]))
    with v.Graph(None) as g, cfg_graph(case) as c:
        g.set_nodes(wd, ht, case["nodes"])
        g.alloc()
        c.alloc()
        a = g.run(m).copy()
        b = c.run(m).copy()
    assert np.array_equal(a.view(np.uint16), b.view(np.uint16))
