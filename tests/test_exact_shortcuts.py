"""Exact shortcuts of the kernels checked on the CPU, where numpy evaluates
them exactly (the device checks of the same run with the GPU tests,
tests/test_gpu_math.py).

- unorm16_exact (denoise.cuh): v / 65535 for every u16 code v as q = RN(v y),
  r = v - q 65535 (exact), RN(q + r y) (one fma), y = RN(1/65535). float64 holds
  every intermediate exactly (at most 48 significant bits), so rounding each
  fma result once to float32 gives the device's value.
- the fixed taps of k_dn_doub_quad (k_denoise.cu): doub.comp samples the coarse
  levels by texture() at the normalised centre of output x of n = 2 h. In the
  kernel's IEEE single operations and the sampler's 8-bit sub-texel rounding
  that is texel x/2 - 1 at fraction 0.75 for even x and texel x/2 at 0.25 for
  odd x. The library checks this on the host per row and column size
  (doub_taps_fixed in graph.cpp) before it takes the quad kernel; here it is
  shown for the sizes of the tests and benchmarks and a spread of others."""
import numpy as np
import pytest

f32 = np.float32


def test_unorm16_exact_equals_the_ieee_quotient_on_every_code():
    v = np.arange(65536, dtype=np.float64)
    y = np.float64(f32(1.0) / f32(65535.0))                 # RN(1/65535) in float32
    q = (v * y).astype(f32).astype(np.float64)               # RN(v y)
    r = v - q * 65535.0                                      # exact
    got = (q + r * y).astype(f32)                            # the fma: one rounding
    want = (v.astype(f32) / f32(65535.0)).astype(f32)       # IEEE single quotient
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _doub_taps_fixed(n, h):
    if n != 2 * h:
        return False
    x = np.arange(n, dtype=f32)
    u = (x + f32(0.5)) / f32(n)
    t = u * f32(h)
    s = (t - f32(0.5)) * f32(256.0) + f32(0.5)               # (t - 0.5) 256 exact, then + 0.5 rounded
    xs = np.floor(s) * f32(0.00390625)
    fx = np.floor(xs)
    ax = xs - fx
    xi = np.arange(n)
    want = np.where(xi & 1, xi // 2, xi // 2 - 1)
    return bool(np.array_equal(fx.astype(np.int64), want) and np.array_equal(ax, np.where(xi & 1, f32(0.25), f32(0.75))))


@pytest.mark.parametrize("n", [16, 96, 128, 742, 1000, 1536, 2048, 4000, 4024, 6000, 6048, 6336, 8256, 9504,
                               12000, 16384, 30000, 60000])
def test_doub_taps_at_fixed_places(n):
    assert _doub_taps_fixed(n, n // 2)


def test_doub_taps_need_twice_the_half_size():
    # an odd or unequal size takes the per-pixel kernel
    assert not _doub_taps_fixed(101, 50)
