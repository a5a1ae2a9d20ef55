"""Ingestion of packed raw video on the device.

The uncompressed magic lantern frame (i-mlv/video_mlv.c:254-274, unpacked on
the host in the reference; vkdt_cuda_unpack_mlv): CPU tests pin the layout of
the oracle restatement (its inverse packs random frames that unpack to
themselves; known bit positions); GPU tests check the kernel against the
oracle bit for bit on random bytes, and that a packed frame unpacked into a
graph's source develops to the same image as the u16 mosaic uploaded as it is.

The motioncam frame (i-mcraw/prefix.comp + decode.comp;
vkdt_cuda_mcraw_decode): the oracle restatement equals the reference's own
decode shader (compiled for the CPU) on random streams of every bit count,
here and through committed fixtures; the device decoder equals the oracle
bit for bit; the test encoder's frames decode to themselves."""
import numpy as np
import pytest

import oracle
import vkdt_gb300 as v


@pytest.mark.parametrize("bpp", [10, 12, 14, 16])
@pytest.mark.parametrize("npix", [8, 16, 4096 + 8, 99992])
def test_mlv_round_trip(bpp, npix):
    # frames hold whole 16-bit words (sample counts in multiples of 8, as the sensor widths are)
    rng = np.random.default_rng(bpp * 1000 + npix)
    vals = rng.integers(0, 1 << bpp, npix).astype(np.uint16)
    packed = oracle.pack_mlv(vals, bpp)
    assert packed.size == npix * bpp // 8
    assert np.array_equal(oracle.unpack_mlv(packed, bpp, npix), vals)


def test_mlv_bit_positions():
    # samples fill the little-endian 16-bit words from their most significant bit:
    # at 14 bits sample 0 is bits 2..15 of word 0, sample 1 continues with bits 0..1
    # of word 0 (its top bits) and bits 4..15 of word 1
    one = np.zeros(8, np.uint16)
    one[0] = 1
    assert list(oracle.pack_mlv(one, 14)[:4]) == [0x04, 0x00, 0x00, 0x00]
    one[:] = 0
    one[1] = 1 << 13
    assert list(oracle.pack_mlv(one, 14)[:4]) == [0x02, 0x00, 0x00, 0x00]
    one[1] = 1
    assert list(oracle.pack_mlv(one, 14)[:4]) == [0x00, 0x00, 0x10, 0x00]
    # 16 bits: the words are the samples
    w = np.arange(8, dtype=np.uint16) * 4097
    assert np.array_equal(oracle.pack_mlv(w, 16).view(np.uint16), w)


@pytest.mark.gpu
@pytest.mark.parametrize("bpp", [10, 12, 14, 16])
@pytest.mark.parametrize("wd,ht", [(4096, 2160), (1928, 1081), (40, 5)])
def test_unpack_mlv_gpu_equals_oracle(gpu, bpp, wd, ht):
    import torch
    rng = np.random.default_rng(bpp + wd)
    nbytes = wd * ht * bpp // 8
    packed = rng.integers(0, 256, nbytes + (nbytes & 1)).astype(np.uint8)
    want = oracle.unpack_mlv(packed[:nbytes], bpp, wd * ht)
    d_in = torch.from_numpy(packed).cuda()
    for shift in (0, 1):   # 16-byte aligned output and an output 2 bytes off (scalar stores)
        d_out = torch.zeros(wd * ht + 8, dtype=torch.int16, device="cuda")
        v.unpack_mlv(d_in.data_ptr(), nbytes, bpp, wd, ht, d_out.data_ptr() + 2 * shift)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(np.uint16)[shift:shift + wd * ht]
        assert np.array_equal(got, want), (bpp, wd, ht, shift, int((got != want).sum()))


@pytest.mark.gpu
def test_unpack_mlv_rejects(gpu):
    import torch
    d = torch.zeros(1024, dtype=torch.int16, device="cuda")
    for bpp in (8, 11, 32):
        with pytest.raises(v._lib.VkdtError):
            v.unpack_mlv(d.data_ptr(), 2048, bpp, 16, 16, d.data_ptr())
    with pytest.raises(v._lib.VkdtError):   # frame too short
        v.unpack_mlv(d.data_ptr(), 100, 14, 16, 16, d.data_ptr())
    with pytest.raises(v._lib.VkdtError):   # unaligned
        v.unpack_mlv(d.data_ptr() + 1, 2000, 14, 16, 16, d.data_ptr())


@pytest.mark.gpu
def test_packed_frame_develops_like_the_mosaic(gpu):
    # a 12-bit video frame packed as magic lantern writes it and unpacked on the device
    # develops to the same image as the u16 mosaic uploaded as it is
    import torch
    wd, ht = 1920, 1080
    m = v.scene_host(v.make_scene(wd, ht, seed=31, black=256.0, white=4095.0, a=4.0, b=0.8))
    ip = v.default_img_param(wd=wd, ht=ht, black=256.0, white=4095.0)
    packed = torch.from_numpy(oracle.pack_mlv(m, 12)).cuda()
    d_plain = torch.from_numpy(m.view(np.int16).reshape(-1)).cuda()
    d_unpacked = torch.zeros(wd * ht, dtype=torch.int16, device="cuda")
    v.unpack_mlv(packed.data_ptr(), packed.numel(), 12, wd, ht, d_unpacked.data_ptr())
    out = [torch.zeros(wd * ht * 4, dtype=torch.float16, device="cuda") for _ in range(2)]
    with v.Graph() as g:
        g.set_input(wd, ht, ip)
        g.set_param("demosaic", "method", np.int32(1))
        g.alloc()
        g.develop(d_plain.data_ptr(), out[0].data_ptr())
        g.develop(d_unpacked.data_ptr(), out[1].data_ptr())
        g.wait()
    torch.cuda.synchronize()
    assert torch.equal(d_unpacked, d_plain)
    assert torch.equal(out[0].view(torch.int16), out[1].view(torch.int16))


# ---------------------------------------------------------------- motioncam (i-mcraw)
MC_BYTES = {0: 0, 1: 8, 2: 16, 3: 24, 4: 32, 5: 40, 6: 48, 7: 64, 8: 64, 9: 80, 10: 80}


def mc_random_stream(rng, rwd, ht):
    """a random frame stream: every bit count 0..15, random references and data"""
    blocks = rwd * ht // 64
    nib = rng.integers(0, 16, blocks)
    nib[:min(16, blocks)] = np.arange(min(16, blocks))
    bitcnt = np.zeros((blocks + 1) // 2, np.uint8)
    for i, n in enumerate(nib):
        bitcnt[i // 2] |= int(n) << (4 * (i & 1))
    size = sum(MC_BYTES.get(int(n), 128) for n in nib)
    refval = rng.integers(0, 20000, blocks).astype(np.uint16)
    data = rng.integers(0, 256, size).astype(np.uint8)
    return bitcnt, refval, data


@pytest.mark.parametrize("fc", [-1, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 15])
def test_mcraw_round_trip(fc):
    # the test encoder inverts the decoder for every bit count (counts 7 and 9 use the
    # 8 and 10 bit layouts, 11..15 the 16 bit one)
    rng = np.random.default_rng(fc + 20)
    rwd, ht = 256, 16
    width = {-1: 14, 7: 8, 9: 10, 15: 14}.get(fc, fc)
    img = (1000 + rng.integers(0, 1 << width, (ht, rwd))).astype(np.uint16)
    bc, rv, dt = oracle.mcraw_encode(img, fc)
    assert np.array_equal(oracle.mcraw_decode(bc, rv, dt, rwd, ht), img)


def test_mcraw_unorm_store():
    # the decoder stores (ref + delta) / 65536 into an R16_UNORM image: codes above 32768
    # come back one lower (no 10..14 bit sensor reaches them)
    rwd, ht = 64, 4
    bc = np.zeros(2, np.uint8)
    rv = np.array([100, 32768, 40000, 65535], np.uint16)
    out = oracle.mcraw_decode(bc, rv, np.zeros(0, np.uint8), rwd, ht)
    assert out[0, 0] == 100 and out[0, 1] == 32768 and out[1, 0] == 39999 and out[1, 1] == 65534


def _ref_available():
    try:
        from oracle import glsl_ref
        return glsl_ref.available()
    except Exception:
        return False


@pytest.mark.parametrize("name", ["mcraw_256x16", "mcraw_320x24_crop"])
def test_mcraw_oracle_matches_golden(name):
    import golden_cases as gc
    bitcnt, refval, data, (rwd, ht, ox, oy, _), want = gc.load_mcraw(name)
    H, W = want.shape
    assert np.array_equal(oracle.mcraw_decode(bitcnt, refval, data, rwd, ht, ox, oy, W, H), want)


@pytest.mark.skipif(not _ref_available(), reason="reference shaders not compiled here (oracle/_ref)")
@pytest.mark.parametrize("rwd,ht,ox,oy", [(256, 16, 0, 0), (320, 24, 1, 1), (128, 8, 1, 0)])
def test_mcraw_oracle_matches_reference_shader(rwd, ht, ox, oy):
    from oracle import glsl_ref as gr
    rng = np.random.default_rng(rwd + ht)
    bitcnt, refval, data = mc_random_stream(rng, rwd, ht)
    W, H = (rwd - ox) // 2 * 2, (ht - oy) // 2 * 2
    want = oracle.mcraw_decode(bitcnt, refval, data, rwd, ht, ox, oy, W, H)
    sizes = [MC_BYTES.get((int(bitcnt[i // 2]) >> (4 * (i & 1))) & 15, 128) for i in range(rwd * ht // 64)]
    offs = np.cumsum(sizes).astype(np.uint32)   # prefix.comp: the inclusive sum
    out = gr.Img(W, H, 1, gr.UNORM16)
    gr.run("i_mcraw_decode", rwd * ht // 64 * 8, 1, {0: out}, push=gr.u32(ox, oy, rwd, ht),
           buffers={1: bitcnt, 2: offs, 3: refval, 4: np.concatenate([data, np.zeros(128, np.uint8)])})
    got = np.rint(out.a[..., 0] * 65535).astype(np.uint16)
    assert np.array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("rwd,ht,ox,oy", [(4096, 2160, 0, 0), (4032, 3024, 1, 1), (256, 16, 1, 0), (64, 4, 0, 0)])
def test_mcraw_gpu_equals_oracle(gpu, rwd, ht, ox, oy):
    import torch
    rng = np.random.default_rng(rwd * 3 + ht)
    bitcnt, refval, data = mc_random_stream(rng, rwd, ht)
    W, H = (rwd - ox) // 2 * 2, (ht - oy) // 2 * 2
    want = oracle.mcraw_decode(bitcnt, refval, data, rwd, ht, ox, oy, W, H)
    d = [torch.from_numpy(a).cuda() for a in (bitcnt, refval.view(np.int16), data)]
    out = torch.zeros(W * H, dtype=torch.int16, device="cuda")
    v.mcraw_decode(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), data.size, rwd, ht, out.data_ptr(), ox, oy, W, H)
    got = out.cpu().numpy().view(np.uint16).reshape(H, W)
    assert np.array_equal(got, want), int((got != want).sum())


@pytest.mark.gpu
def test_mcraw_frame_round_trip_gpu(gpu):
    # a 12-bit video frame through the test encoder and the device decoder
    import torch
    rwd, ht = 4096, 2160
    m = v.scene_host(v.make_scene(rwd, ht, seed=41, black=256.0, white=4095.0, a=4.0, b=0.8))
    bc, rv, dt = oracle.mcraw_encode(m)
    d = [torch.from_numpy(a).cuda() for a in (bc, rv.view(np.int16), dt)]
    out = torch.zeros(rwd * ht, dtype=torch.int16, device="cuda")
    v.mcraw_decode(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), dt.size, rwd, ht, out.data_ptr())
    assert np.array_equal(out.cpu().numpy().view(np.uint16).reshape(ht, rwd), m)


@pytest.mark.gpu
def test_mcraw_rejects(gpu):
    import torch
    d = torch.zeros(4096, dtype=torch.int16, device="cuda")
    p = d.data_ptr()
    for rwd, ht in ((100, 16), (128, 6), (0, 4)):
        with pytest.raises(v._lib.VkdtError):
            v.mcraw_decode(p, p, p, 16, rwd, ht, p, d_scratch=p)
    with pytest.raises(v._lib.VkdtError):
        v.mcraw_decode(p, p + 1, p, 16, 64, 4, p, d_scratch=p)
