"""Write the golden fixtures of tests/golden_cases.py from the reference's
own GLSL shaders, translated and compiled for the CPU (oracle/glsl ->
oracle/_ref/libvkdt_ref.so, run by oracle/glsl_ref.py as the modules'
create_nodes build the node graph).

Needs the vkdt source tree (to compile the shaders) where oracle/glsl/
translate.py looks for it. Every stored stage is an f16 image of the
reference (stored as float16, which is lossless) with the alpha channel
dropped.

    python tests/golden/make_golden.py [case names]   (all cases without names)
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle                      # noqa: E402
import vkdt_gb300 as v             # noqa: E402
from oracle import glsl_ref        # noqa: E402
from golden_cases import CASES, NOISE_A, NOISE_B, img_param, oracle_params, path   # noqa: E402


def main():
    if not glsl_ref.build():
        raise SystemExit("the reference shaders could not be compiled (vkdt sources missing)")
    only = set(sys.argv[1:])
    for name, case in CASES.items():
        if only and name not in only:
            continue
        wd, ht, filters, seed, white, overrides, stages = case
        m = v.scene_host(v.make_scene(wd, ht, seed=seed, a=NOISE_A, b=NOISE_B, filters=filters))
        ip = oracle.img_param(img_param(v, wd, ht, filters, white))
        p = oracle_params(oracle, overrides)
        r = glsl_ref.develop(m, ip, p, stages=stages)
        arrays = {"mosaic": m}
        for s in stages:
            a = r[s] if r[s].ndim == 2 else r[s][..., :3]
            h = a.astype(np.float16)
            if not np.array_equal(h.astype(np.float32), a):
                raise RuntimeError("%s/%s is not an f16 image" % (name, s))
            arrays["out_" + s] = h
        meta = {"case": list(case[:6]), "llap_levels": r["llap_levels"]}
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
        np.savez_compressed(path(name), **arrays)
        print("%-24s %s" % (name, ", ".join(stages)))


if __name__ == "__main__":
    main()
