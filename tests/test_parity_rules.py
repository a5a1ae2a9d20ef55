"""The parity rules of tests/parity.py, on the CPU: the oracle's own results
pass them, and mistakes planted in a copy of those results (standing in for a
CUDA path's output) are caught."""
import numpy as np
import pytest

import oracle
import parity as P
import vkdt_gb300 as v

STAGES = ("denoise", "hilite", "demosaic", "colour", "filmcurv", "llap", "hist")


def fake_gpu(strength):
    wd, ht = 256, 192
    m = oracle.scene(wd, ht, seed=3, a=8.0, b=1.6)
    ip = v.default_img_param(wd=wd, ht=ht, noise_a=8.0 / 15871 ** 2, noise_b=1.6 / 15871)
    op = oracle.default_params()
    op.dn_strength = strength
    r = oracle.develop(m, oracle.img_param(ip), params=op, stages=STAGES, record=True)
    g = {k: r[k].copy() for k in STAGES}
    kinds = ("gauss", "dn_cov", "dn_thr") if strength else ("gauss",)
    g["dec"] = {k: r["dec_" + k].copy() for k in kinds}
    return m, ip, op, g, r


@pytest.mark.parametrize("strength", [0.0, 1.0])
def test_oracle_results_pass(strength):
    m, ip, op, g, _ = fake_gpu(strength)
    assert P.check("self_s%g" % strength, v, m, ip, op, g)["ok"]


def test_planted_stage_error_is_caught():
    m, ip, op, g, _ = fake_gpu(0.0)
    g["demosaic"][40, 50, 1] += 0.01
    with pytest.raises(AssertionError, match="node"):
        P.check("planted_demosaic", v, m, ip, op, g)


def test_planted_colour_error_is_caught():
    m, ip, op, g, _ = fake_gpu(0.0)
    g["colour"][40, 50, 2] *= 1.01
    with pytest.raises(AssertionError):
        P.check("planted_colour", v, m, ip, op, g)


def test_unexplained_gauss_decision_is_caught():
    m, ip, op, g, r = fake_gpu(0.0)
    g["dec"]["gauss"][10, 10] ^= 2     # a snapped direction the hilite input does not give
    with pytest.raises(AssertionError, match="gauss decisions not explained"):
        P.check("planted_gauss", v, m, ip, op, g)


def test_threshold_switch_away_from_a_tie_is_caught():
    m, ip, op, g, r = fake_gpu(1.0)
    mar = r["margin_dn_thr"][..., 0]
    y, x = np.unravel_index(int(np.argmax(mar)), mar.shape)      # the decision farthest from its tie
    g["dec"]["dn_thr"][y, x] ^= 1
    with pytest.raises(AssertionError, match="away from a tie"):
        P.check("planted_threshold", v, m, ip, op, g)
