"""Write tests/golden/nodes.json: the node lists the reference's own module host
code (create_nodes, commit_params; oracle/modules, compiled from the vkdt tree)
emits for the cases below, with push constants and uniform blocks, so that
machines without the vkdt tree can feed them to vkdt_cuda_graph_set_nodes.

    python tests/golden/make_nodes.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import vkdt_gb300 as v                     # noqa: E402
from oracle import modules as M            # noqa: E402
from oracle.modules import build as MB     # noqa: E402

BAYER = 0x94949494
QUAD = (0.25, 0.25, 0.75, 0.25, 0.75, 0.75, 0.25, 0.75)   # crop/params: the default perspective quad
# name: (wd, ht, filters, extra cfg lines, output size)
CASES = {
    "darkroom_2048x1536": (2048, 1536, BAYER, "", (0, 0)),
    "darkroom_6000x4000": (6000, 4000, BAYER, "", (0, 0)),
    "wavelet_1000x742": (1000, 742, BAYER, "param:denoise:01:strength:1\n", (0, 0)),
    "rcd_1000x742": (1000, 742, BAYER, "param:demosaic:01:method:1\n", (0, 0)),
    "halfsize_1000x742": (1000, 742, BAYER, "param:demosaic:01:method:2\n", (0, 0)),
    "thumb_2048x1536": (2048, 1536, BAYER, "", (256, 192)),
    "xtrans_606x402": (606, 402, 9, "", (0, 0)),
    "fixup_1000x742": (1000, 742, BAYER, "param:demosaic:01:colour:1\n", (0, 0)),
    "params_384x256": (384, 256, BAYER, "param:colour:01:exposure:0.7\nparam:llap:01:clarity:0\n"
                       "param:filmcurv:01:colour:1\nparam:filmcurv:01:contrast:1.5\nparam:hilite:01:white:0.9\n", (0, 0)),
}
# with crop between demosaic and colour (the darkroom cfg's own): name: (wd, ht, filters, extra, exif orientation)
CROP_CASES = {
    "crop_2048x1536": (2048, 1536, BAYER, "", 0),
    "crop_6000x4000": (6000, 4000, BAYER, "", 0),
    "crop_orient6_1000x742": (1000, 742, BAYER, "", 6),
    "crop_orient8_606x402": (606, 402, 9, "", 8),
    "crop_persp_1024x768": (1024, 768, BAYER, "param:crop:01:perspect:0.2:0.22:0.8:0.25:0.77:0.8:0.21:0.75\n"
                            "param:crop:01:crop:0.1:0.9:0.05:0.95\nparam:crop:01:rotate:3.5\n", 0),
    "crop_rcd_1000x742": (1000, 742, BAYER, "param:demosaic:01:method:1\n", 0),
}
NA, NB = 2.0 / (16383 - 512) ** 2, 0.4 / (16383 - 512)


def case_ip(wd, ht, filters, orientation=0):
    ip = v.default_img_param(wd=wd, ht=ht, filters=filters, noise_a=NA, noise_b=NB)
    ip.orientation = orientation
    return ip


def generate():
    if not MB.build():
        raise SystemExit("the vkdt tree is needed (VKDT_REFERENCE)")
    out = {}
    todo = [(n, wd, ht, f, v.DARKROOM_CFG + e, o, 0) for n, (wd, ht, f, e, o) in CASES.items()]
    todo += [(n, wd, ht, f, v.DARKROOM_CROP_CFG + e, (0, 0), r) for n, (wd, ht, f, e, r) in CROP_CASES.items()]
    for name, wd, ht, filters, cfg, (ow, oh), orient in todo:
        nodes, mods = M.run(cfg, wd, ht, case_ip(wd, ht, filters, orient), ow, oh)
        out[name] = {
            "in": [wd, ht], "filters": filters, "cfg": cfg, "out": [ow, oh], "orientation": orient,
            "nodes": [{"name": n["name"], "kernel": n["kernel"], "wd": n["wd"], "ht": n["ht"], "dp": n["dp"],
                       "push": n["push"].hex(),
                       "uniform": mods[n["module"]]["uniform"].hex() if n["module"] >= 0 else ""} for n in nodes],
            "modules": {m["name"]: m["param"].hex() for m in mods}}
    with open(os.path.join(HERE, "nodes.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)


def load():
    with open(os.path.join(HERE, "nodes.json")) as f:
        d = json.load(f)
    for c in d.values():
        for n in c["nodes"]:
            n["push"] = bytes.fromhex(n["push"])
            n["uniform"] = bytes.fromhex(n["uniform"])
        c["modules"] = {k: bytes.fromhex(h) for k, h in c["modules"].items()}
    return d


if __name__ == "__main__":
    generate()
