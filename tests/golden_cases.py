"""Golden cases of the development path: their inputs, and the reader of the
fixtures tests/golden/make_golden.py writes from the reference's own shaders
(compiled for the CPU).

Each case is a seeded synthetic mosaic (the product's scene generator), an
image parameter set and module parameter overrides. The overrides are named
by the oracle's parameter fields; PARAM_MAP gives the module parameter of the
graph configuration each one sets.
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

BAYER, XTRANS = 0x94949494, 9
QUAD = (0.25, 0.25, 0.75, 0.25, 0.75, 0.75, 0.25, 0.75)   # crop/params: the untouched perspective quad

# noise profile of the generated mosaics, in raw DN (gaussian a, poissonian b)
NOISE_A, NOISE_B = 8.0, 1.6

CASES = {
    # name: (wd, ht, filters, seed, white, overrides, stages kept)
    "bayer_96x64": (96, 64, BAYER, 5, 16383.0, {}, ("hilite", "demosaic", "filmcurv", "llap")),
    "bayer_16x16": (16, 16, BAYER, 6, 16383.0, {}, ("hilite", "demosaic", "llap")),
    "bayer_130x98_clipped": (130, 98, BAYER, 7, 9000.0, {}, ("hilite", "demosaic", "llap")),
    "bayer_128x96_params": (128, 96, BAYER, 8, 16383.0,
                            {"co_exposure": 0.5, "fc_contrast": 1.4, "fc_colour": 1, "hl_white": 0.9,
                             "ll_clarity": 0.5, "ll_levels": 4},
                            ("filmcurv", "llap")),
    "bayer_128x96_wavelet": (128, 96, BAYER, 9, 16383.0, {"dn_strength": 1.0},
                             ("denoise", "hilite", "llap")),
    "bayer_256x192_thumb": (256, 192, BAYER, 10, 16383.0, {"out_wd": 64, "out_ht": 48}, ("demosaic", "llap")),
    "xtrans_132x96": (132, 96, XTRANS, 11, 16383.0, {}, ("hilite", "demosaic", "llap")),
    "xtrans_132x96_wavelet": (132, 96, XTRANS, 12, 16383.0, {"dn_strength": 1.0}, ("denoise", "llap")),
    # demosaic RCD over 3x4 of the shader's 58x26 tiles (seams included), and with clipping
    "bayer_140x80_rcd": (140, 80, BAYER, 13, 16383.0, {"dm_method": 1}, ("hilite", "demosaic", "llap")),
    "bayer_124x58_rcd_clipped": (124, 58, BAYER, 14, 9000.0, {"dm_method": 1}, ("demosaic", "llap")),
    # demosaic method 2: the half size demosaic at half the output size
    "bayer_120x90_halfsize": (120, 90, BAYER, 15, 16383.0, {"dm_method": 2}, ("demosaic", "llap")),
    # crop after demosaic ("crop": [perspect, window, rotate, exif orientation]): a whole texel
    # shift (nearest texel), a perspective quad with a rotation and a quarter turn (Catmull-Rom)
    "bayer_96x64_crop_shift": (96, 64, BAYER, 16, 16383.0, {"crop": [list(QUAD), [0.03125, 0.96875, 0.0625, 0.9375], 0.0, 0]},
                               ("crop", "llap")),
    "bayer_112x80_crop_persp": (112, 80, BAYER, 17, 16383.0,
                                {"crop": [[0.2, 0.22, 0.8, 0.25, 0.77, 0.8, 0.21, 0.75], [0.1, 0.9, 0.05, 0.95], 3.5, 0]},
                                ("crop", "llap")),
    "xtrans_132x96_crop_turn": (132, 96, XTRANS, 18, 16383.0, {"crop": [list(QUAD), [1.0, 3.0, 3.0, 7.0], 1337.0, 6]},
                                ("crop", "llap")),
}

# i-mcraw decode cases: (rwd, ht, ox, oy, seed) of a random frame stream (every bit count)
MCRAW_CASES = {
    "mcraw_256x16": (256, 16, 0, 0, 1),
    "mcraw_320x24_crop": (320, 24, 1, 1, 2),
}
MCRAW_BYTES = {0: 0, 1: 8, 2: 16, 3: 24, 4: 32, 5: 40, 6: 48, 7: 64, 8: 64, 9: 80, 10: 80}


def mcraw_stream(rwd, ht, seed):
    """the random stream of a case: nibble counts (every count 0..15), references, data"""
    rng = np.random.default_rng(seed)
    blocks = rwd * ht // 64
    nib = rng.integers(0, 16, blocks)
    nib[:min(16, blocks)] = np.arange(min(16, blocks))
    bitcnt = np.zeros((blocks + 1) // 2, np.uint8)
    for i, n in enumerate(nib):
        bitcnt[i // 2] |= int(n) << (4 * (i & 1))
    size = sum(MCRAW_BYTES.get(int(n), 128) for n in nib)
    refval = rng.integers(0, 20000, blocks).astype(np.uint16)
    data = rng.integers(0, 256, size).astype(np.uint8)
    return bitcnt, refval, data


def load_mcraw(name):
    z = np.load(path(name))
    meta = json.loads(bytes(z["meta"]).decode())
    if tuple(meta["case"]) != tuple(MCRAW_CASES[name]):
        raise RuntimeError("fixture %s was made for another case definition" % name)
    return z["bitcnt"], z["refval"], z["data"], MCRAW_CASES[name], z["out"]


# output encode: BC1 blocks of an rgba u8 image (o-bc1's stb_dxt) and colenc of an rgba f16
# image at these (primaries, transfer curve) pairs
ENCODE_COLENC = [(2, 2), (1, 1), (3, 6), (5, 0), (6, 3), (7, 5), (10, 4), (4, 2)]


def encode_inputs(seed=3):
    """the u8 image of the BC1 fixture (random, gradient, few colour and flat blocks side by side)
    and the f16 image of the colenc fixture"""
    rng = np.random.default_rng(seed)
    ht, wd = 48, 64
    y, x = np.mgrid[0:ht, 0:wd]
    img = np.zeros((ht, wd, 4), np.uint8)
    img[:, :16] = rng.integers(0, 256, (ht, 16, 4))
    img[:, 16:32, 0] = (x[:, 16:32] * 7) % 256
    img[:, 16:32, 1] = (y[:, 16:32] * 5) % 256
    img[:, 16:32, 2] = ((x + y)[:, 16:32] * 3) % 256
    pal = rng.integers(0, 256, (3, 4))
    img[:, 32:48] = pal[rng.integers(0, 3, (ht, 16))]
    img[:, 48:] = np.clip(100 + rng.integers(-2, 3, (ht, 16, 4)), 0, 255)
    img[..., 3] = 255
    img[:4, 48:52] = (17, 200, 33, 255)    # a constant block
    f = rng.uniform(-0.05, 1.3, (32, 48, 4)).astype(np.float16).astype(np.float32)
    f[..., 3] = 1.0
    return img, f


def load_encode():
    z = np.load(path("encode"))
    return z["bc1"], z["colenc"]


# grade after llap: (lift, gamma, gain, offset, mode, sh_pivot, hi_pivot); the first is the params file's default
GRADE_CASES = [
    ((0, 0, 0, 0), (1, 1, 1, 0), (1, 1, 1, 0), (0, 0, 0, 0), 0, 0.3, 0.4),
    ((0.05, -0.02, 0.1, 0.01), (0.95, 1.05, 1.0, 0.02), (1.1, 0.98, 1.02, -0.03), (-0.01, 0.02, 0.0, 0.005), 0, 0.3, 0.4),
    ((0.12, 0.0, -0.08, 0.0), (1.08, 0.92, 1.0, 0.0), (0.95, 1.05, 1.1, 0.0), (0.0, -0.02, 0.03, 0.0), 1, 0.3, 0.4),
    ((-0.1, 0.05, 0.0, 0.02), (1.0, 1.1, 0.9, -0.01), (1.05, 1.0, 0.97, 0.01), (0.02, 0.0, -0.01, 0.0), 1, 0.15, 0.8),
]


def grade_input(seed=5):
    """the f16 rgba image of the grade fixture (llap outputs as stored: f16, a few below 0 and above 1)"""
    rng = np.random.default_rng(seed)
    f = rng.uniform(-0.05, 1.4, (24, 40, 4)).astype(np.float16).astype(np.float32)
    f[..., 3] = 1.0
    return f


def load_grade():
    return np.load(path("grade"))["out"]


# lens (lens/main.comp): the uniform block centre (2), scale (2), squish0, squish1, ca red, ca blue;
# the first is the params file's default (close to the identity)
LENS_CASES = [
    (0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 1.0, 1.0),
    (0.0, 0.0, 1.0, 1.0, 0.3, 0.1, 1.0, 1.0),
    (0.02, -0.01, 1.1, 0.95, 0.5, -0.2, 1.0, 1.0),
    (0.0, 0.0, 0.9, 0.9, 0.2, 0.4, 1.003, 0.996),
    (-0.03, 0.02, 1.2, 1.2, -0.3, 0.6, 0.99, 1.01),
]


def lens_input(seed=6):
    """the f16 rgba image of the lens fixture (an input as stored: f16, a smooth field plus noise)"""
    rng = np.random.default_rng(seed)
    ht, wd = 36, 52
    y, x = np.mgrid[0:ht, 0:wd].astype(np.float32)
    f = np.stack([0.5 + 0.4 * np.sin(x / 5.0), 0.5 + 0.4 * np.cos(y / 4.0), (x + y) / (wd + ht), np.ones_like(x)], -1)
    f[..., :3] += rng.normal(0, 0.03, (ht, wd, 3)).astype(np.float32)
    return f.astype(np.float16).astype(np.float32)


def load_lens():
    return np.load(path("lens"))["out"]


# oracle parameter field -> (module, parameter) of the graph configuration
PARAM_MAP = {
    "dn_strength": ("denoise", "strength"),
    "dm_method": ("demosaic", "method"),
    "hl_white": ("hilite", "white"),
    "co_exposure": ("colour", "exposure"),
    "fc_contrast": ("filmcurv", "contrast"),
    "fc_colour": ("filmcurv", "colour"),
    "ll_clarity": ("llap", "clarity"),
}


def img_param(v, wd, ht, filters, white):
    """The image parameters of a case, as a vkdt_gb300.ImgParam (noise in
    the normalised form the modules read)."""
    return v.default_img_param(wd=wd, ht=ht, filters=filters, white=white,
                               noise_a=NOISE_A / (16383.0 - 512.0) ** 2, noise_b=NOISE_B / (16383.0 - 512.0))


def oracle_params(oracle, overrides, wd=0, ht=0):
    """oracle parameters of a case; a "crop" override commits crop for the demosaic output of
    a full size wd x ht case (oracle.crop_commit)"""
    p = oracle.default_params()
    for k, val in overrides.items():
        if k == "crop":
            persp, win, rot, orient = val
            blk, cw, ch = oracle.crop_commit(wd, ht, perspect=persp, crop=win, rotate=rot, orientation=orient)
            oracle.set_crop(p, blk, cw, ch)
        else:
            setattr(p, k, val)
    return p


def graph_crop(v, g, ip, overrides):
    """the crop override of a case on a graph made from v.DARKROOM_CROP_CFG"""
    persp, win, rot, orient = overrides["crop"]
    ip.orientation = orient
    g.set_param("crop", "perspect", np.array(persp, np.float32))
    g.set_param("crop", "crop", np.array(win, np.float32))
    g.set_param("crop", "rotate", np.float32(rot))


def path(name):
    return os.path.join(GOLDEN, name + ".npz")


def load(name):
    """(mosaic, case tuple, {stage: float32 array}) of a committed fixture."""
    z = np.load(path(name))
    meta = json.loads(bytes(z["meta"]).decode())
    if tuple(meta["case"][:5]) != tuple(CASES[name][:5]) or meta["case"][5] != CASES[name][5]:
        raise RuntimeError("fixture %s was made for another case definition" % name)
    out = {k[4:]: z[k].astype(np.float32) for k in z.files if k.startswith("out_")}
    return z["mosaic"], CASES[name], out
