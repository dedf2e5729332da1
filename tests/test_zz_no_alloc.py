"""The allocation-free batch render, called through the C ABI.

Some hosts of this library cannot let it allocate device memory while they
render: engines that reserve all GPU memory up front for their own allocator,
or that forbid allocations on their render path.  For them
sky_cuda_render_batch_noalloc() renders a small batch of jobs with the
persistent tracer while keeping the kernel's job table and work counter in a
fixed scratch area of the library instead of in allocated memory.  These
tests check it against the ordinary device-output entry point,
sky_cuda_render_device(), on two calls in a row (the scratch area is reused
by every call); that the second, warmed call allocates nothing (the
library's own count of device allocations and the GPU's free memory are
unchanged across it); and that an oversized batch and a request for the
plain kernel are refused.
"""

import ctypes

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig
from sky_cuda import _abi

pytestmark = pytest.mark.gpu


def _configs():
    common = dict(phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS, max_orders=16)
    return [
        RenderConfig(width=16, height=8, spp=32, seed=11, **common),
        RenderConfig(width=12, height=10, spp=48, seed=12, output_projection=_abi.PROJECTION_SKY_VIEW_LUT,
                     **common),
        RenderConfig(width=8, height=8, spp=16, seed=13, sample_offset=64, **common),
    ]


def _buffers(torch, cfg, bands):
    cells = cfg.pixels * bands
    return {
        "cell_sum": torch.zeros(cells, dtype=torch.float64, device="cuda"),
        "cell_sumsq": torch.zeros(cells, dtype=torch.float64, device="cuda"),
        "film": torch.zeros(cells, dtype=torch.float32, device="cuda"),
    }


def _outputs_struct(bufs, status=None, counters=None):
    o = _abi.SkyDeviceOutputs()
    o.cell_sum = bufs["cell_sum"].data_ptr()
    o.cell_sumsq = bufs["cell_sumsq"].data_ptr()
    o.film = bufs["film"].data_ptr()
    o.status = status.data_ptr() if status is not None else None
    o.counters = counters.data_ptr() if counters is not None else None
    return o


def test_noalloc_batch_matches_render_device(gpu, dome_scene):
    import torch
    lib = _abi.load_library()
    configs = _configs()
    stream = torch.cuda.current_stream().cuda_stream
    with GpuScene(dome_scene) as gs:
        bands = gs.band_count
        reference = []
        for cfg in configs:
            bufs = _buffers(torch, cfg, bands)
            status = torch.zeros(1, dtype=torch.int32, device="cuda")
            gs.render_device(cfg, {"cell_sum": bufs["cell_sum"].data_ptr(),
                                   "cell_sumsq": bufs["cell_sumsq"].data_ptr(),
                                   "film": bufs["film"].data_ptr(), "status": status.data_ptr()}, stream)
            torch.cuda.synchronize()
            assert int(status.item()) == 0
            reference.append({k: v.cpu().numpy() for k, v in bufs.items()})

        c_configs = (_abi.SkyRenderConfig * len(configs))(*[c.to_c() for c in configs])
        for call in range(2):  # the shared scratch area must serve consecutive calls
            bufs = [_buffers(torch, c, bands) for c in configs]
            status = torch.zeros(1, dtype=torch.int32, device="cuda")
            counters = torch.zeros(8, dtype=torch.int64, device="cuda")
            outs = (_abi.SkyDeviceOutputs * len(configs))(
                *[_outputs_struct(b, status if i == 0 else None, counters if i == 0 else None)
                  for i, b in enumerate(bufs)])
            torch.cuda.synchronize()
            allocs, free = lib.sky_cuda_device_allocations(), torch.cuda.mem_get_info()[0]
            st = lib.sky_cuda_render_batch_noalloc(gs.handle, c_configs, outs, len(configs),
                                                   ctypes.c_void_p(stream))
            _abi.check(st, lib)
            torch.cuda.synchronize()
            if call == 1:  # warmed: the device code is loaded, nothing may be allocated
                assert lib.sky_cuda_device_allocations() == allocs
                assert torch.cuda.mem_get_info()[0] == free
            assert int(status.item()) == 0
            chains = sum(c.pixels * bands * c.spp for c in configs)
            assert int(counters[6].item()) == chains
            for ref, got in zip(reference, bufs):
                np.testing.assert_allclose(got["cell_sum"].cpu().numpy(), ref["cell_sum"], rtol=1e-12, atol=0)
                np.testing.assert_allclose(got["cell_sumsq"].cpu().numpy(), ref["cell_sumsq"], rtol=1e-12, atol=0)
                np.testing.assert_allclose(got["film"].cpu().numpy(), ref["film"], rtol=1e-6, atol=0)


def test_noalloc_rejects_oversized_batch(gpu, dome_scene):
    import torch
    lib = _abi.load_library()
    n = _abi.NOALLOC_MAX_JOBS + 1
    cfg = RenderConfig(width=4, height=4, spp=4, tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(dome_scene) as gs:
        bufs = _buffers(torch, cfg, gs.band_count)
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        c_configs = (_abi.SkyRenderConfig * n)(*[cfg.to_c() for _ in range(n)])
        outs = (_abi.SkyDeviceOutputs * n)(*[_outputs_struct(bufs, status) for _ in range(n)])
        st = lib.sky_cuda_render_batch_noalloc(gs.handle, c_configs, outs, n, None)
        assert st == _abi.SKY_ERR_INVALID_CONFIG
        assert "SKY_NOALLOC_MAX_JOBS" in _abi.last_error(lib)
        # the call runs the wavefront kernel only: a job asking for the plain kernel is refused
        plain = (_abi.SkyRenderConfig * 1)(RenderConfig(width=4, height=4, spp=4, kernel=_abi.KERNEL_PLAIN,
                                                        tracking=_abi.TRACKING_MERGED_LAYERS).to_c())
        st = lib.sky_cuda_render_batch_noalloc(gs.handle, plain, outs, 1, None)
        assert st == _abi.SKY_ERR_INVALID_CONFIG and "wavefront kernel only" in _abi.last_error(lib)
        # the scene still renders through the allocation-free path afterwards
        st = lib.sky_cuda_render_batch_noalloc(gs.handle, c_configs, outs, 1, None)
        _abi.check(st, lib)
        torch.cuda.synchronize()
        assert int(status.item()) == 0 and np.all(np.isfinite(bufs["film"].cpu().numpy()))
