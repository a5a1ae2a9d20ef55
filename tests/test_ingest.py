"""Ingestion of packed raw video: the uncompressed magic lantern frame
(i-mlv/video_mlv.c:254-274) unpacked on the device (vkdt_cuda_unpack_mlv).

CPU tests pin the layout of the oracle restatement (its inverse packs random
frames that unpack to themselves; known bit positions); GPU tests check the
kernel against the oracle bit for bit on random bytes, and that a packed
frame unpacked into a graph's source develops to the same image as the u16
mosaic uploaded as it is."""
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
    d_plain = torch.from_numpy(m.view(np.int16)).cuda()
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
