"""The develop server (continuous batching): every job's result is the same
alone and in the mix (bit exact: the same kernels on its own buffers), with
device and host buffers, mixed shapes and per-image metadata; admission under
a device memory cap; errors are reported per job and the server carries on."""
import numpy as np
import pytest

import vkdt_gb300 as v

pytestmark = pytest.mark.gpu

BAYER, XTRANS = 0x94949494, 9


def _jobs():
    # (wd, ht, filters, out_wd, out_ht, seed, wb)
    return [(512, 384, BAYER, 0, 0, 1, (2.0, 1.0, 1.6)), (640, 480, BAYER, 0, 0, 2, (1.7, 1.0, 1.9)),
            (512, 384, BAYER, 0, 0, 3, (2.3, 1.0, 1.3)), (606, 402, XTRANS, 0, 0, 4, (2.0, 1.0, 1.6)),
            (1000, 742, BAYER, 250, 185, 5, (1.9, 1.0, 1.5)), (640, 480, BAYER, 0, 0, 6, (2.1, 1.0, 1.4))]


def _img_param(wd, ht, filters, wb, seed):
    rng = np.random.default_rng(seed)
    a, b = rng.uniform(1, 16), rng.uniform(0.2, 3)
    return v.default_img_param(wd=wd, ht=ht, filters=filters, wb=wb,
                               noise_a=a / (16383 - 512) ** 2, noise_b=b / (16383 - 512))


def _inputs():
    import torch
    out = []
    for wd, ht, f, ow, oh, seed, wb in _jobs():
        m = v.scene_host(v.make_scene(wd, ht, seed=seed, filters=f, wb=wb))
        out.append((m, torch.from_numpy(m.view(np.int16)).cuda(), _img_param(wd, ht, f, wb, seed), ow, oh))
    torch.cuda.synchronize()
    return out


def _alone(inputs):
    import torch
    res = []
    for m, dm, ip, ow, oh in inputs:
        ht, wd = m.shape
        with v.Graph() as g:
            g.set_input(wd, ht, ip)
            if ow:
                g.set_output_size(ow, oh)
            g.alloc()
            out = torch.zeros((g.out_ht, g.out_wd, 4), dtype=torch.float16, device="cuda")
            torch.cuda.synchronize()
            g.develop(dm.data_ptr(), out.data_ptr())
            g.wait()
            res.append(out.cpu().numpy().view(np.uint16).copy())
    return res


def _out_shape(wd, ht, ow, oh):
    return (oh, ow) if ow else (ht, wd)


def test_server_same_result_alone_and_in_the_mix(gpu):
    import torch
    inputs = _inputs()
    want = _alone(inputs)
    with v.Server(slots=4) as s:
        for rep in range(2):     # the second round reuses the pooled graphs with other metadata
            outs, ids = [], []
            for (m, dm, ip, ow, oh), w in zip(inputs, want):
                ht, wd = m.shape
                if rep == 0:     # device buffers
                    o = torch.zeros(w.shape, dtype=torch.int16, device="cuda")
                    torch.cuda.synchronize()
                    ids.append(s.submit(dm.data_ptr(), o.data_ptr(), wd, ht, ip, ow, oh))
                else:            # host buffers
                    o = np.zeros(w.shape, np.uint16)
                    ids.append(s.submit(m, o, wd, ht, ip, ow, oh))
                outs.append(o)
            for i in ids:
                s.wait(i)
            for o, w in zip(outs, want):
                got = o.cpu().numpy().view(np.uint16) if rep == 0 else o
                assert np.array_equal(got, w)
        st = s.stats()
        assert st["completed"] == 12 and st["failed"] == 0
        assert st["latency_p99_ms"] >= st["latency_p50_ms"] > 0


def test_server_admission_under_a_small_cap(gpu):
    import torch
    inputs = _inputs()[:3]
    want = _alone(inputs)
    # room for about one 640x480 graph: jobs wait for memory and graphs are recycled
    with v.Graph() as g:
        g.set_input(640, 480, v.default_img_param(wd=640, ht=480))
        g.create_nodes()
        import ctypes as C
        nb = C.c_uint64()
        v._lib.check(v._lib.lib().vkdt_cuda_graph_plan_bytes(g._g, C.byref(nb)), "plan_bytes")
    cap = int(nb.value * 1.5)
    with v.Server(slots=4, hbm_cap=cap) as s:
        outs = [(torch.zeros(w.shape, dtype=torch.int16, device="cuda"), w, x) for _ in range(3)
                for x, w in zip(inputs, want)]
        torch.cuda.synchronize()      # the server's streams do not wait for torch's
        for o, w, (m, dm, ip, ow, oh) in outs:
            ht, wd = m.shape
            s.submit(dm.data_ptr(), o.data_ptr(), wd, ht, ip, ow, oh)
        s.drain()
        for o, w, _ in outs:
            assert np.array_equal(o.cpu().numpy().view(np.uint16), w)
        st = s.stats()
        assert st["completed"] == 9 and st["peak_device_bytes"] <= cap


def test_server_reports_failed_jobs_and_carries_on(gpu):
    import torch
    inputs = _inputs()[:1]
    want = _alone(inputs)
    m, dm, ip, ow, oh = inputs[0]
    ht, wd = m.shape
    with v.Server(slots=2, hbm_cap=1 << 20) as s:     # 1 MiB: nothing fits
        o = torch.zeros(want[0].shape, dtype=torch.int16, device="cuda")
        torch.cuda.synchronize()
        j = s.submit(dm.data_ptr(), o.data_ptr(), wd, ht, ip)
        with pytest.raises(v._lib.VkdtError) as e:
            s.wait(j)
        assert e.value.code == v._lib.ERROR_OUT_OF_DEVICE_MEMORY
    with v.Server(slots=2) as s:
        bad = v.default_img_param(wd=wd - 1, ht=ht)      # odd bayer width: the graph rejects it
        o = torch.zeros(want[0].shape, dtype=torch.int16, device="cuda")
        torch.cuda.synchronize()
        j1 = s.submit(dm.data_ptr(), o.data_ptr(), wd - 1, ht, bad)
        o2 = torch.zeros(want[0].shape, dtype=torch.int16, device="cuda")
        torch.cuda.synchronize()
        j2 = s.submit(dm.data_ptr(), o2.data_ptr(), wd, ht, ip)
        with pytest.raises(v._lib.VkdtError):
            s.wait(j1)
        s.wait(j2)
        assert np.array_equal(o2.cpu().numpy().view(np.uint16), want[0])
        assert s.stats()["failed"] == 1
