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
NA, NB = 2.0 / (16383 - 512) ** 2, 0.4 / (16383 - 512)


def case_ip(wd, ht, filters):
    return v.default_img_param(wd=wd, ht=ht, filters=filters, noise_a=NA, noise_b=NB)


def generate():
    if not MB.build():
        raise SystemExit("the vkdt tree is needed (VKDT_REFERENCE)")
    out = {}
    for name, (wd, ht, filters, extra, (ow, oh)) in CASES.items():
        cfg = v.DARKROOM_CFG + extra
        nodes, mods = M.run(cfg, wd, ht, case_ip(wd, ht, filters), ow, oh)
        out[name] = {
            "in": [wd, ht], "filters": filters, "cfg": cfg, "out": [ow, oh],
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
