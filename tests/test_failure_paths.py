"""Failure paths on the GPU, made without faulting it.

* The wavefront kernel's loop backstop (SkyTuning.iteration_limit) set to a
  few iterations: every warp stops early, sets status bit 2, and the call
  returns SKY_ERR_WATCHDOG, as the reference maps its device watchdog flag
  to RenderError::Watchdog (integrator.rs:301-304).  The wait runs out on
  the device by design; the context stays usable.
* A device allocation failure injected on the host
  (SKY_CUDA_FAIL_DEVICE_ALLOC): the call that must allocate returns
  SKY_ERR_OUT_OF_MEMORY, and the scene renders again once the injection ends.
"""

import os

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig, RenderWatchdog, SkyCudaError
from sky_cuda import _abi

pytestmark = pytest.mark.gpu


def _cfg(**kw):
    return RenderConfig(**{**dict(width=16, height=8, spp=64, phase_sampling=_abi.PHASE_TABULATED,
                                  tracking=_abi.TRACKING_MERGED_LAYERS), **kw})


def test_iteration_limit_reports_the_watchdog(gpu, dome_scene):
    import torch
    with GpuScene(dome_scene) as gs:
        gs.set_tuning(iteration_limit=3)
        assert gs.get_tuning()["iteration_limit"] == 3
        with pytest.raises(RenderWatchdog, match="iteration limit"):
            gs.render(_cfg())
        # the device word carries bit 2 (bit 1 is the per-path depth watchdog)
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        s = torch.zeros(_cfg().pixels * gs.band_count, dtype=torch.float64, device="cuda")
        gs.render_device(_cfg(), {"cell_sum": s.data_ptr(), "status": st.data_ptr()},
                         torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert int(st.item()) & 2
        # back to the default backstop: the same render completes
        gs.set_tuning(iteration_limit=0)
        film, stats = gs.render(_cfg())
        assert stats.watchdog == 0 and np.all(np.isfinite(film.values)) and film.values.sum() > 0


def test_injected_allocation_failure(gpu, dome_scene, monkeypatch):
    lib = _abi.load_library()
    with GpuScene(dome_scene) as gs:
        gs.render(_cfg(width=4, height=4))  # workspace for 16 pixels
        before = lib.sky_cuda_device_allocations()
        monkeypatch.setenv("SKY_CUDA_FAIL_DEVICE_ALLOC", "1")
        # a larger render must grow the workspace: that allocation fails
        with pytest.raises(SkyCudaError) as e:
            gs.render(_cfg(width=32, height=16))
        assert e.value.status == _abi.SKY_ERR_OUT_OF_MEMORY
        # scene creation fails the same way and leaves nothing behind
        with pytest.raises(SkyCudaError) as e:
            GpuScene(dome_scene)
        assert e.value.status == _abi.SKY_ERR_OUT_OF_MEMORY
        # a render that fits the existing workspace needs no allocation and works
        film, _ = gs.render(_cfg(width=4, height=2))
        assert np.all(np.isfinite(film.values))
        assert lib.sky_cuda_device_allocations() == before
        monkeypatch.delenv("SKY_CUDA_FAIL_DEVICE_ALLOC")
        film, stats = gs.render(_cfg(width=32, height=16))
        assert stats.watchdog == 0 and film.values.size == 32 * 16 * gs.band_count
        assert lib.sky_cuda_device_allocations() > before
    assert os.environ.get("SKY_CUDA_FAIL_DEVICE_ALLOC") is None
