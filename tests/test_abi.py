"""CPU tests of the C-ABI library: it loads, exports every declared entry
point, and its host side (cfg reading, parameters, create_nodes) behaves like
the reference's module layer. No compute calls (no GPU here)."""
import ctypes as C

import numpy as np
import pytest

import vkdt_gb300 as v
from vkdt_gb300 import _lib


def test_library_exports_every_declared_symbol():
    l = _lib.lib()
    declared = _lib.declared_symbols()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(l, name), name
        assert name in _lib._SIGS, name


def test_token_packing():
    # src/pipe/token.h: little endian chars, at most 8
    assert v.token("llap") == ord("l") | ord("l") << 8 | ord("a") << 16 | ord("p") << 24
    assert v.token_str(v.token("demosaic")) == "demosaic"
    assert v.token("toolongname") == v.token("toolongn")


def test_supports():
    for n, k in [("denoise", "noop"), ("hilite", "reduce"), ("demosaic", "splat"), ("demosaic", "rcd_fill"),
                 ("llap", "assemble"), ("OpenDRT", "hist"), ("hist", "collect")]:
        assert v.supports(n, k)
    assert not v.supports("crop", "main")
    assert not v.supports("resize", "main")


def test_default_params_and_cfg_overrides():
    g = v.Graph()
    assert np.isclose(g.get_param("denoise", "strength")[0], 0.0)
    assert np.isclose(g.get_param("hilite", "white")[0], 0.985)
    assert np.isclose(g.get_param("filmcurv", "light")[0], 3.0)
    assert g.get_param("filmcurv", "colour", dtype=np.int32)[0] == 3
    assert np.isclose(g.get_param("llap", "clarity")[0], 0.2)   # the cfg line
    assert np.isclose(g.get_param("llap", "sigma")[0], 0.12)
    g.set_param("colour", "exposure", 0.5)
    assert np.isclose(g.get_param("colour", "exposure")[0], 0.5)
    g.set_param("denoise", "edges", [0.1, 0.2, 0.3, 0.4])
    assert np.allclose(g.get_param("denoise", "edges", 4), [0.1, 0.2, 0.3, 0.4])
    with pytest.raises(_lib.VkdtError) as e:
        g.set_param("colour", "nosuch", 1.0)
    assert e.value.code == _lib.ERROR_FORMAT_NOT_SUPPORTED
    with pytest.raises(_lib.VkdtError):
        g.set_param("denoise", "edges", 1.0)    # wrong count
    g.close()


FULL_CFG = v.DARKROOM_CFG.replace(
    "connect:demosaic:01:output:colour:01:input\n",
    "module:crop:01:743:400\nmodule:grade:01:1444:400\nmodule:display:main:1545:400\n"
    "connect:demosaic:01:output:crop:01:input\nconnect:crop:01:output:colour:01:input\n"
    "connect:llap:01:output:grade:01:input\nconnect:grade:01:output:display:main:input\n") + "param:grade:01:vib:1\n"


def test_cfg_with_modules_outside_the_path():
    # crop (checked for the identity) and grade (applied after llap) are known; the display is not
    g = v.Graph(FULL_CFG)
    assert sorted(g.unsupported()) == ["display"]
    g.close()


def test_cfg_errors():
    broken = v.DARKROOM_CFG.replace("connect:hilite:01:output:demosaic:01:input\n", "")
    with pytest.raises(_lib.VkdtError) as e:
        v.Graph(broken)
    assert e.value.code == _lib.INCOMPLETE
    with pytest.raises(_lib.VkdtError) as e:
        v.Graph(v.DARKROOM_CFG + "bogus line\n")
    assert e.value.code == _lib.ERROR_FORMAT_NOT_SUPPORTED


def _nodes(wd, ht, levels=0):
    g = v.Graph()
    g.set_input(wd, ht, v.default_img_param(wd=wd, ht=ht))
    if levels:
        g.set_llap_levels(levels)
    g.create_nodes()
    n = g.nodes()
    g.close()
    return n


def test_create_nodes_24mp():
    n = _nodes(6000, 4000)
    kinds = [(a, b) for a, b, *_ in n]
    # hilite/main.c: reduce/assemble pairs until a level has one pixel row or column
    assert kinds.count(("hilite", "reduce")) == 10 and kinds.count(("hilite", "assemble")) == 10
    # llap/main.c: 12 levels at 24 MP (11 reduce + 11 assemble nodes)
    assert kinds.count(("llap", "reduce")) == 11 and kinds.count(("llap", "assemble")) == 11
    red = [x for x in n if x[0] == "llap" and x[1] == "reduce"]
    assert red[0][2:5] == (3000, 2000, 11) and red[-1][2:4] == (3, 2)
    hred = [x for x in n if x[0] == "hilite" and x[1] == "reduce"]
    assert hred[0][2:4] == (1500, 1000) and hred[-1][2:4] == (3, 2)
    for name, kernel, *_ in n:
        assert v.supports(name, kernel), (name, kernel)


def test_create_nodes_forced_depth():
    n = _nodes(6000, 4000, levels=6)
    kinds = [(a, b) for a, b, *_ in n]
    assert kinds.count(("llap", "reduce")) == 5


def test_create_nodes_wavelet_denoise():
    # denoise/main.c:225-333: four half size scales, assemble, half, full size doub, one launch each
    # but half, which the downcov launch makes on a bayer mosaic
    g = v.Graph()
    g.set_input(6000, 4000, v.default_img_param(wd=6000, ht=4000))
    g.set_param("denoise", "strength", 1.0)
    g.create_nodes()
    n = g.nodes()
    g.close()
    dn = [x for x in n if x[0] == "denoise"]
    assert [x[1] for x in dn] == ["downcov", "down", "down", "down", "assemble", "half", "doub"]
    assert all(x[2:4] == (3000, 2000) for x in dn[:6]) and dn[6][2:4] == (6000, 4000)
    assert len({x[5] for x in dn}) == 6
    assert dn[5][5] == dn[0][5]
    for name, kernel, *_ in n:
        assert v.supports(name, kernel), (name, kernel)


def test_create_nodes_xtrans():
    # x-trans: 3x3 blocks (hilite and demosaic/gauss at a third of the size), per node launches
    g = v.Graph()
    g.set_input(6240, 4160, v.default_img_param(wd=6240, ht=4160, filters=9))
    g.create_nodes()
    n = g.nodes()
    g.close()
    by = {(a, b): x for x in n for a, b in [x[:2]]}
    assert by[("hilite", "half")][2:4] == (2080, 1386) and by[("demosaic", "gauss")][2:4] == (2080, 1386)
    assert by[("demosaic", "fix")][2:4] == (6240, 4160)
    fused = [x[5] for x in n]
    assert min(fused) >= 0 and len(set(fused)) >= 20


def test_create_nodes_xtrans_wavelet_denoise():
    # x-trans with the wavelet denoise: the half node keeps a launch of its own (3x3 blocks)
    g = v.Graph()
    g.set_input(6240, 4160, v.default_img_param(wd=6240, ht=4160, filters=9))
    g.set_param("denoise", "strength", 1.0)
    g.create_nodes()
    n = g.nodes()
    g.close()
    dn = [x for x in n if x[0] == "denoise"]
    assert [x[1] for x in dn] == ["downcov", "down", "down", "down", "assemble", "half", "doub"]
    assert all(x[2:4] == (2080, 1386) for x in dn[:6]) and dn[6][2:4] == (6240, 4160)
    assert len({x[5] for x in dn}) == 7


def test_create_nodes_rcd():
    # demosaic method 1 (demosaic/main.c:113-155): rcd_conv at full size, one rcd_fill
    # workgroup per 58x26 tile, no gaussian splat nodes; method 2: always half size
    g = v.Graph()
    g.set_input(4096, 2160, v.default_img_param(wd=4096, ht=2160))
    g.set_param("demosaic", "method", 1)
    g.create_nodes()
    n = g.nodes()
    g.close()
    by = {(a, b): x for x in n for a, b in [x[:2]]}
    assert by[("demosaic", "rcd_conv")][2:4] == (4096, 2160)
    assert by[("demosaic", "rcd_fill")][2:4] == ((4096 + 57) // 58 * 8, (2160 + 25) // 26 * 8)
    assert ("demosaic", "splat") not in by and ("demosaic", "gauss") not in by
    assert by[("llap", "colour")][2:4] == (4096, 2160)
    for name, kernel, *_ in n:
        assert v.supports(name, kernel), (name, kernel)
    g = v.Graph()
    g.set_input(4096, 2160, v.default_img_param(wd=4096, ht=2160))
    g.set_param("demosaic", "method", 2)
    g.create_nodes()
    by = {(a, b): x for x in g.nodes() for a, b in [x[:2]]}
    g.close()
    assert by[("demosaic", "halfsize")][2:4] == (2048, 1080) and ("shared", "resample") not in by
    assert by[("llap", "colour")][2:4] == (2048, 1080)


def test_create_nodes_thumbnail():
    # demosaic/main.c: 1/8 size -> halfsize + resample; denoise and hilite stay full size
    g = v.Graph()
    g.set_input(6000, 4000, v.default_img_param(wd=6000, ht=4000))
    g.set_output_size(750, 500)
    g.create_nodes()
    n = g.nodes()
    g.close()
    kinds = [x[:2] for x in n]
    assert ("demosaic", "halfsize") in kinds and ("shared", "resample") in kinds and ("demosaic", "splat") not in kinds
    assert [x for x in n if x[:2] == ("demosaic", "halfsize")][0][2:4] == (3000, 2000)
    assert [x for x in n if x[:2] == ("llap", "colour")][0][2:4] == (750, 500)
    assert [x for x in n if x[:2] == ("hilite", "half")][0][2:4] == (3000, 2000)
    for name, kernel, *_ in n:
        assert v.supports(name, kernel), (name, kernel)
    # a scale below 1.5 blocks would need a resample after the full size demosaic
    g = v.Graph()
    g.set_input(6000, 4000, v.default_img_param(wd=6000, ht=4000))
    g.set_output_size(4000, 2666)
    with pytest.raises(_lib.VkdtError) as e:
        g.create_nodes()
    assert e.value.code == _lib.INCOMPLETE
    g.close()


def test_create_nodes_rejects_bad_input():
    g = v.Graph()
    ip = v.default_img_param(wd=101, ht=100)
    g.set_input(101, 100, ip)
    with pytest.raises(_lib.VkdtError):
        g.create_nodes()
    g.close()


def test_standalone_nodes_reject_bad_arguments():
    # the standalone node entries check their arguments before any device work
    with pytest.raises(_lib.VkdtError) as e:
        v.lens(0, 64, 48, 0)
    assert e.value.code == _lib.ERROR_FORMAT_NOT_SUPPORTED
    with pytest.raises(_lib.VkdtError) as e:
        v.lens(256, 0, 48, 512)
    assert e.value.code == _lib.ERROR_FORMAT_NOT_SUPPORTED
    with pytest.raises(_lib.VkdtError) as e:
        v.lens(260, 64, 48, 512)                       # an rgba f16 image is 8-byte aligned
    assert e.value.code == _lib.ERROR_FORMAT_NOT_SUPPORTED
    with pytest.raises(_lib.VkdtError) as e:
        v.waveform(0, 64, 48, 0)
    assert e.value.code == _lib.ERROR_FORMAT_NOT_SUPPORTED
