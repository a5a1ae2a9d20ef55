"""Error metrics of the parity tests (numpy, float64)."""
import numpy as np

# src/pipe/modules/matrices.h matrix_rec2020_to_xyz (row major)
REC2020_TO_XYZ = np.array([[0.636958048301290991, 0.144616903586208406, 0.168880975164172054],
                           [0.26270021201126692, 0.677998071518871148, 0.0593017164698619384],
                           [4.9999999999999999e-17, 0.0280726930490874452, 1.06098505771079066]])
D65 = np.array([0.95047, 1.0, 1.08883])


def rel_err(out, ref):
    """Per pixel max over rgb of |out-ref| / max(1, |ref|): absolute below 1,
    relative above (f16 storage has a relative resolution)."""
    out = np.asarray(out, np.float64)[..., :3]
    ref = np.asarray(ref, np.float64)[..., :3]
    e = np.abs(out - ref) / np.maximum(1.0, np.abs(ref))
    e = np.where(np.isnan(e), np.inf, e)
    return e.max(axis=-1)


def summary(out, ref, tol=2e-3):
    e = rel_err(out, ref)
    bad = e > tol
    good = e[~bad]
    return {
        "max": float(e.max()),
        "max_good": float(good.max()) if good.size else 0.0,
        "mean": float(np.mean(np.minimum(e, 1.0))),
        "flipped": int(bad.sum()),
        "flipped_frac": float(bad.mean()),
    }


def lab(rgb2020):
    xyz = np.einsum("ij,...j->...i", REC2020_TO_XYZ, np.asarray(rgb2020, np.float64)[..., :3]) / D65
    d = 6.0 / 29.0
    f = np.where(xyz > d ** 3, np.cbrt(np.maximum(xyz, 0)), xyz / (3 * d * d) + 4.0 / 29.0)
    L = 116 * f[..., 1] - 16
    a = 500 * (f[..., 0] - f[..., 1])
    b = 200 * (f[..., 1] - f[..., 2])
    return L, a, b


def delta_e2000(rgb_a, rgb_b):
    """CIEDE2000 between two linear rec2020 images (D65 white = 1)."""
    L1, a1, b1 = lab(rgb_a)
    L2, a2, b2 = lab(rgb_b)
    return delta_e2000_lab(L1, a1, b1, L2, a2, b2)


def delta_e2000_lab(L1, a1, b1, L2, a2, b2):
    """CIEDE2000 colour difference (Sharma, Wu, Dalal, Color Res. Appl. 30, 2005)."""
    L1, a1, b1, L2, a2, b2 = [np.asarray(x, np.float64) for x in (L1, a1, b1, L2, a2, b2)]
    C1 = np.hypot(a1, b1)
    C2 = np.hypot(a2, b2)
    Cm = 0.5 * (C1 + C2)
    G = 0.5 * (1 - np.sqrt(Cm ** 7 / (Cm ** 7 + 25.0 ** 7)))
    a1p, a2p = (1 + G) * a1, (1 + G) * a2
    C1p, C2p = np.hypot(a1p, b1), np.hypot(a2p, b2)
    h1p = np.degrees(np.arctan2(b1, a1p)) % 360
    h2p = np.degrees(np.arctan2(b2, a2p)) % 360
    dLp = L2 - L1
    dCp = C2p - C1p
    dh = h2p - h1p
    dh = np.where(C1p * C2p == 0, 0, np.where(dh > 180, dh - 360, np.where(dh < -180, dh + 360, dh)))
    dHp = 2 * np.sqrt(C1p * C2p) * np.sin(np.radians(dh / 2))
    Lpm = 0.5 * (L1 + L2)
    Cpm = 0.5 * (C1p + C2p)
    hs = h1p + h2p
    hpm = np.where(C1p * C2p == 0, hs,
                   np.where(np.abs(h1p - h2p) <= 180, hs / 2, np.where(hs < 360, (hs + 360) / 2, (hs - 360) / 2)))
    T = (1 - 0.17 * np.cos(np.radians(hpm - 30)) + 0.24 * np.cos(np.radians(2 * hpm))
         + 0.32 * np.cos(np.radians(3 * hpm + 6)) - 0.20 * np.cos(np.radians(4 * hpm - 63)))
    dtheta = 30 * np.exp(-(((hpm - 275) / 25) ** 2))
    Rc = 2 * np.sqrt(Cpm ** 7 / (Cpm ** 7 + 25.0 ** 7))
    Sl = 1 + 0.015 * (Lpm - 50) ** 2 / np.sqrt(20 + (Lpm - 50) ** 2)
    Sc = 1 + 0.045 * Cpm
    Sh = 1 + 0.015 * Cpm * T
    Rt = -np.sin(np.radians(2 * dtheta)) * Rc
    return np.sqrt((dLp / Sl) ** 2 + (dCp / Sc) ** 2 + (dHp / Sh) ** 2 + Rt * (dCp / Sc) * (dHp / Sh))
