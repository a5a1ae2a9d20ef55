"""vkdt_cuda_graph_develop_static: the develop on the library's fixed device
scratch (no allocation in the call) against vkdt_cuda_graph_develop on an
allocated graph. Both run the same kernels on the same input, so the results
are equal bit for bit; the call allocates no device memory. Collected last,
and independent of every other test file."""
import numpy as np
import pytest

import vkdt_gb300 as v

pytestmark = pytest.mark.gpu

NA, NB = 2.0 / (16383 - 512) ** 2, 0.4 / (16383 - 512)


def _graph(wd, ht):
    g = v.Graph()
    g.set_input(wd, ht, v.default_img_param(wd=wd, ht=ht, noise_a=NA, noise_b=NB))
    return g


def _allocated_develop(dm, wd, ht):
    import torch
    out = torch.zeros((ht, wd, 4), dtype=torch.float16, device="cuda")
    torch.cuda.synchronize()
    with _graph(wd, ht) as g:
        g.alloc()
        g.develop(dm.data_ptr(), out.data_ptr())
        g.wait()
    return out.float().cpu().numpy()


@pytest.mark.parametrize("wd,ht", [(1024, 768), (1600, 1200)])
def test_static_develop_matches_allocated_twice(gpu, wd, ht):
    import torch
    m = v.scene_host(v.make_scene(wd, ht, seed=31))
    dm = torch.from_numpy(m.view(np.int16)).cuda()
    want = _allocated_develop(dm, wd, ht)
    with _graph(wd, ht) as g:
        g.create_nodes()
        for call in range(2):   # two calls in a row on the same scratch
            out = torch.full((ht, wd, 4), float("nan"), dtype=torch.float16, device="cuda")
            torch.cuda.synchronize()
            free0, _ = torch.cuda.mem_get_info()
            used0 = torch.cuda.memory_allocated()
            g.develop_static(dm.data_ptr(), out.data_ptr())
            torch.cuda.synchronize()
            if call == 1:
                # the defining property: the call takes no device memory (the first call may
                # load the module's kernels; the second runs the same kernels again)
                # (torch may free a temporary of the test meanwhile: nothing grows)
                assert torch.cuda.mem_get_info()[0] >= free0 and torch.cuda.memory_allocated() <= used0
            got = out.float().cpu().numpy()
            assert np.isfinite(got).all(), call
            assert np.array_equal(got.astype(np.float16).view(np.uint16), want.astype(np.float16).view(np.uint16)), call


def test_static_develop_rejects_what_it_cannot_run(gpu):
    import torch
    v.init()
    dummy = torch.zeros(16, dtype=torch.float16, device="cuda")
    # beyond the scratch: a clear error, before any device work
    with _graph(1920, 1080) as g:
        g.create_nodes()
        with pytest.raises(v._lib.VkdtError) as e:
            g.develop_static(dummy.data_ptr(), dummy.data_ptr())
        assert e.value.code == v._lib.ERROR_FORMAT_NOT_SUPPORTED and "static scratch" in str(e.value)
    # no plan yet
    with _graph(256, 192) as g:
        with pytest.raises(v._lib.VkdtError) as e:
            g.develop_static(dummy.data_ptr(), dummy.data_ptr())
        assert e.value.code == v._lib.INCOMPLETE
    # an allocated graph keeps its own buffers
    with _graph(256, 192) as g:
        g.alloc()
        with pytest.raises(v._lib.VkdtError) as e:
            g.develop_static(dummy.data_ptr(), dummy.data_ptr())
        assert e.value.code == v._lib.INCOMPLETE
    # a graph changed after create_nodes (here its output size) would run a stale plan
    with _graph(256, 192) as g:
        g.create_nodes()
        g.set_output_size(64, 48)
        with pytest.raises(v._lib.VkdtError) as e:
            g.develop_static(dummy.data_ptr(), dummy.data_ptr())
        assert e.value.code == v._lib.INCOMPLETE
