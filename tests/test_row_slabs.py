"""Pixel-row slabs on the GPU, through the C ABI: a render cut into row slabs
(SkyRenderConfig.row_begin / row_count, the unit of the multi-GPU split) and
concatenated equals the whole render, in every kernel and in the
differentiable forward render; slab outputs hold the slab's pixels only."""

from dataclasses import replace

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig, SkyCudaError
from sky_cuda import _abi
from sky_cuda.parallel import row_slabs, slab_config

pytestmark = pytest.mark.gpu


def _sums(gs, cfg):
    import torch
    cells = cfg.pixels * gs.band_count
    s = torch.zeros(cells, dtype=torch.float64, device="cuda")
    q = torch.zeros(cells, dtype=torch.float64, device="cuda")
    film = torch.zeros(cells, dtype=torch.float32, device="cuda")
    xyz = torch.zeros(cfg.pixels * 3, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    gs.render_device(cfg, {"cell_sum": s.data_ptr(), "cell_sumsq": q.data_ptr(), "film": film.data_ptr(),
                           "xyz": xyz.data_ptr(), "status": st.data_ptr()},
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    B = gs.band_count
    return (s.cpu().numpy().reshape(-1, B), q.cpu().numpy().reshape(-1, B), film.cpu().numpy().reshape(-1, B),
            xyz.cpu().numpy().reshape(-1, 3))


@pytest.mark.parametrize("kernel", [_abi.KERNEL_PLAIN, _abi.KERNEL_WAVEFRONT])
@pytest.mark.parametrize("projection", [_abi.PROJECTION_PANORAMA, _abi.PROJECTION_SKY_VIEW_LUT])
def test_slabs_concatenate_to_the_whole_render(gpu, dome_scene, kernel, projection):
    cfg = RenderConfig(width=20, height=11, spp=24, seed=5, kernel=kernel, output_projection=projection,
                       phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS,
                       rr_start_depth=8)
    with GpuScene(dome_scene) as gs:
        whole = _sums(gs, cfg)
        parts = [_sums(gs, slab_config(cfg, r, 3)) for r in range(3)]
    for k, (name, tol) in enumerate([("sum", 1e-12), ("sumsq", 1e-12), ("film", 1e-6), ("xyz", 1e-12)]):
        joined = np.concatenate([p[k] for p in parts], axis=0)
        assert joined.shape == whole[k].shape, name
        if kernel == _abi.KERNEL_PLAIN and name != "film":
            np.testing.assert_array_equal(joined, whole[k], err_msg=name)  # fixed summation order
        else:
            np.testing.assert_allclose(joined, whole[k], rtol=tol, atol=1e-300, err_msg=name)
    assert np.all(whole[0].sum(axis=1) > 0)


def test_slab_of_a_batch_and_of_the_adjoint_forward(gpu, dome_scene):
    """A batch job and the differentiable forward render honour the slab too."""
    import torch
    from sky_cuda.adjoint import AdjointRenderer, initial_layer_params
    cfg = RenderConfig(width=16, height=9, spp=16, seed=8, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS, rr_start_depth=8)
    slab = replace(cfg, row_begin=4, row_count=3)
    B = dome_scene.band_count
    lo, hi = 4 * cfg.width, 7 * cfg.width
    stream = torch.cuda.current_stream().cuda_stream
    with GpuScene(dome_scene) as gs:
        whole = _sums(gs, cfg)[0]
        s = torch.zeros(slab.pixels * B, dtype=torch.float64, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        gs.render_batch([(slab, None, {"cell_sum": s.data_ptr(), "status": st.data_ptr()})], stream)
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        np.testing.assert_allclose(s.cpu().numpy().reshape(-1, B), whole[lo:hi], rtol=1e-12, atol=0)
        theta = torch.as_tensor(initial_layer_params(dome_scene, 0.76), device="cuda")
        full = AdjointRenderer(gs, cfg).forward(theta)["cell_sum"].cpu().numpy().reshape(-1, B)
        part = AdjointRenderer(gs, slab).forward(theta)["cell_sum"].cpu().numpy().reshape(-1, B)
    assert part.shape == (slab.pixels, B)
    np.testing.assert_allclose(part, full[lo:hi], rtol=1e-12, atol=0)


def test_slab_validation(gpu, dome_scene):
    with GpuScene(dome_scene) as gs:
        with pytest.raises(SkyCudaError, match="exceed the image height"):
            gs.render(RenderConfig(width=4, height=4, spp=2, row_begin=2, row_count=3))
        with pytest.raises(SkyCudaError, match="row_begin needs a nonzero row_count"):
            gs.render(RenderConfig(width=4, height=4, spp=2, row_begin=1))
        # the host film of a slab holds the slab's pixels only
        film, stats = gs.render(RenderConfig(width=4, height=6, spp=2, row_begin=5, row_count=1))
        assert film.values.size == 4 * gs.band_count and stats.chains == 4 * gs.band_count * 2
    assert row_slabs(6, 4) == [(0, 2), (2, 2), (4, 1), (5, 1)]
