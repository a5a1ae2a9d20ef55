"""Write tests/golden/nprof.json: the noise profile the reference's own nprof
module (nprof/main.c:82-198 write_sink, compiled from the vkdt tree by
oracle/modules) fits to the rawhist histograms of the cases below, as it writes
them ("%g %g"). The histograms are the oracle's rawhist of the seeded mosaics,
rounded to f32 as the module reads its input.

    python tests/golden/make_nprof.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle                              # noqa: E402

BAYER = 0x94949494
# (wd, ht, seed, noise a DN, noise b DN, filters)
CASES = [(2048, 1536, 5, 8.0, 1.6, BAYER), (1000, 742, 3, 2.0, 0.4, BAYER), (1206, 798, 7, 4.0, 0.8, 9),
         (3000, 2000, 1, 16.0, 3.0, BAYER), (640, 480, 9, 1.0, 0.2, BAYER)]


def histogram(case):
    wd, ht, seed, a, b, filters = case
    m = oracle.scene(wd, ht, seed=seed, a=a, b=b, filters=filters)
    return oracle.rawhist(m, filters, 512.0, 16383.0).astype(np.float32).astype(np.float64)


if __name__ == "__main__":
    from oracle import modules as M
    from oracle.modules import build as MB
    if not MB.build():
        raise SystemExit("the vkdt tree is needed (VKDT_REFERENCE)")
    out = [{"case": list(c), "ab": list(M.nprof(histogram(c)))} for c in CASES]
    with open(os.path.join(HERE, "nprof.json"), "w") as f:
        json.dump(out, f, indent=1)
