"""Host side of the differentiable renderer (no GPU): parameter layout and
the defaults that reproduce a scene."""

import numpy as np

from sky_cuda import synthetic_scene, wavelengths
from sky_cuda.adjoint import BAND_PARAMS, PARAMS_PER_LAYER, initial_layer_params, mie_albedo, param_names


def test_initial_parameters_reproduce_the_synthetic_scene(data_dir):
    scene = synthetic_scene(wavelengths(400.0, 700.0, 4), data_dir, sun_elevation_deg=10.0)
    p = initial_layer_params(scene, 0.76)
    L = scene.layer_count
    assert p.dtype == np.float32 and p.size == PARAMS_PER_LAYER * L + 2
    assert np.all(p[:PARAMS_PER_LAYER * L] == 1.0)
    assert abs(mie_albedo(scene) - 0.9) < 1e-6 and abs(p[-2] - 0.9) < 1e-6
    assert abs(p[-1] - 0.76) < 1e-7
    names = param_names(L)
    assert len(names) == p.size and names[:3] == ["rayleigh[0]", "mie[0]", "ozone[0]"]
    assert names[-2:] == ["mie_albedo", "mie_g"]
    assert BAND_PARAMS == 4
