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
from golden_cases import (CASES, ENCODE_COLENC, GRADE_CASES, LENS_CASES, MCRAW_BYTES, MCRAW_CASES,   # noqa: E402
                          NOISE_A, NOISE_B, encode_inputs, grade_input, img_param, lens_input, mcraw_stream,
                          oracle_params, path)


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
        p = oracle_params(oracle, overrides, wd, ht)
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
    for name, case in MCRAW_CASES.items():
        if only and name not in only:
            continue
        rwd, ht, ox, oy, seed = case
        bitcnt, refval, data = mcraw_stream(rwd, ht, seed)
        W, H = (rwd - ox) // 2 * 2, (ht - oy) // 2 * 2
        sizes = [MCRAW_BYTES.get((int(bitcnt[i // 2]) >> (4 * (i & 1))) & 15, 128) for i in range(rwd * ht // 64)]
        offs = np.cumsum(sizes).astype(np.uint32)   # i-mcraw/prefix.comp: the inclusive sum
        out = glsl_ref.Img(W, H, 1, glsl_ref.UNORM16)
        glsl_ref.run("i_mcraw_decode", rwd * ht // 64 * 8, 1, {0: out}, push=glsl_ref.u32(ox, oy, rwd, ht),
                     buffers={1: bitcnt, 2: offs, 3: refval, 4: np.concatenate([data, np.zeros(128, np.uint8)])})
        codes = np.rint(out.a[..., 0] * 65535).astype(np.uint16)
        meta = {"case": list(case)}
        np.savez_compressed(path(name), bitcnt=bitcnt, refval=refval, data=data, out=codes,
                            meta=np.frombuffer(json.dumps(meta).encode(), np.uint8))
        print("%-24s i-mcraw decode" % name)
    if not only or "encode" in only:
        # o-bc1: the reference's own stb_dxt (compiled from the vkdt tree); colenc: its shader
        if not oracle.build_stb_ref():
            raise SystemExit("stb_dxt could not be compiled (vkdt sources missing)")
        img, f = encode_inputs()
        bc1 = oracle.stb_bc1(img)
        outs = []
        for prim, trc in ENCODE_COLENC:
            src, dst = glsl_ref.Img(f.shape[1], f.shape[0], 4), glsl_ref.Img(f.shape[1], f.shape[0], 4)
            src.a[...] = f
            glsl_ref.run("colenc_main", f.shape[1], f.shape[0], {0: src, 1: dst}, uniform=glsl_ref.i32(prim, trc))
            outs.append(dst.a[..., :3].astype(np.float16))
        np.savez_compressed(path("encode"), bc1=bc1, colenc=np.stack(outs))
        print("%-24s o-bc1 (stb_dxt), colenc" % "encode")
    if not only or "grade" in only:
        # grade after llap: its shader on the f16 input, the output as stored (f16)
        f = grade_input()
        outs = []
        for lift, gamma, gain, off, mode, sp, hp in GRADE_CASES:
            src, dst = glsl_ref.Img(f.shape[1], f.shape[0], 4), glsl_ref.Img(f.shape[1], f.shape[0], 4)
            src.a[...] = f
            glsl_ref.run("grade_main", f.shape[1], f.shape[0], {0: src, 1: dst},
                         uniform=glsl_ref.f32(*lift, *gamma, *gain, *off) + glsl_ref.i32(mode) + glsl_ref.f32(sp, hp))
            outs.append(dst.a.astype(np.float16))
        np.savez_compressed(path("grade"), out=np.stack(outs))
        print("%-24s grade" % "grade")
    if not only or "lens" in only:
        # lens/main.comp on the f16 input, the output as stored (f16), at the input's size
        f = lens_input()
        outs = []
        for par in LENS_CASES:
            src, dst = glsl_ref.Img(f.shape[1], f.shape[0], 4), glsl_ref.Img(f.shape[1], f.shape[0], 4)
            src.a[...] = f
            glsl_ref.run("lens_main", f.shape[1], f.shape[0], {0: src, 1: dst}, uniform=glsl_ref.f32(*par))
            outs.append(dst.a.astype(np.float16))
        np.savez_compressed(path("lens"), out=np.stack(outs))
        print("%-24s lens" % "lens")


if __name__ == "__main__":
    main()
