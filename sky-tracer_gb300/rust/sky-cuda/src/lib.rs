//! `sky-cuda`: the spectral path tracer of `sky-spectral-path-tracer`
//! (integrator.rs:125-128) running on the GB300 CUDA kernels of
//! libsky_cuda.so, behind the same signature:
//!
//! ```ignore
//! pub fn render(scene: &SceneData, config: &RenderConfig) -> Result<Film, RenderError>
//! ```
//!
//! The scene is packed exactly as `PackedScene::new` packs it
//! (integrator.rs:319-418), with the library's `SkyBand` etc. in place of
//! `GpuBand` etc., and handed to the one-shot `sky_cuda_render_desc`, which
//! validates it (integrator.rs:130-163), uploads the tables, traces, reads
//! the film back, divides by spp and clamps at zero (integrator.rs:306-316)
//! and frees the device tables.  Statuses map onto `RenderError` one to one
//! for codes 1-6; the library's own out-of-memory, launch and I/O failures
//! keep their variant-appropriate kind and a message that names them.
//!
//! `sky-reference-render` switches its dependency from
//! `sky-spectral-path-tracer` to `sky-cuda` and calls `sky_cuda::render`
//! (main.rs:113); nothing else changes.
//!
//! [`Adjoint`] is the differentiable render of a resident scene as a
//! forward/backward pair (`sky_cuda_adjoint_forward` / `_backward`): the
//! film over per-layer density scales, Mie albedo and asymmetry and per-band
//! multipliers, and the path-replay gradient of a loss given dLoss/dfilm.
//! Its buffers are the caller's device memory (a fitting host keeps
//! parameters, film and gradients on the GPU between iterations).

pub mod ffi;

use std::ffi::CStr;
use std::os::raw::{c_char, c_void};

use sky_core::atmosphere::{GROUND_ALBEDO, PHASE_BINS, SceneData};
pub use sky_spectral_path_tracer::config::{OutputProjection, RenderConfig};
pub use sky_spectral_path_tracer::film::Film;
pub use sky_spectral_path_tracer::integrator::RenderError;

/// Library and ABI version, e.g. "sky_cuda 0.1.0 (abi 1, sm_103a)".
pub fn version() -> String {
    unsafe { CStr::from_ptr(ffi::sky_cuda_version()) }.to_string_lossy().into_owned()
}

/// The message of the calling thread's last failed call.
fn last_error() -> String {
    let mut buf = [0 as c_char; 1024];
    unsafe { ffi::sky_cuda_last_error(buf.as_mut_ptr(), buf.len()) };
    unsafe { CStr::from_ptr(buf.as_ptr()) }.to_string_lossy().into_owned()
}

/// `RenderError` of a nonzero status (integrator.rs:18-26 for 1-6).
pub fn render_error(status: i32, message: String) -> RenderError {
    match status {
        ffi::SKY_ERR_INVALID_CONFIG => RenderError::InvalidConfig(message),
        ffi::SKY_ERR_NO_DEVICE => RenderError::NoAdapter(message),
        ffi::SKY_ERR_DEVICE_INIT => RenderError::RequestDevice(message),
        ffi::SKY_ERR_COPY => RenderError::BufferMap(message),
        ffi::SKY_ERR_SYNC => RenderError::Poll(message),
        ffi::SKY_ERR_WATCHDOG => RenderError::Watchdog,
        ffi::SKY_ERR_OUT_OF_MEMORY => RenderError::RequestDevice(format!("out of device memory: {message}")),
        ffi::SKY_ERR_LAUNCH => RenderError::Poll(format!("kernel launch failed: {message}")),
        ffi::SKY_ERR_IO => RenderError::InvalidConfig(format!("table input failed: {message}")),
        other => RenderError::Poll(format!("unknown status {other}: {message}")),
    }
}

/// The reference's tables of `scene`, owned, in the library's row layouts.
pub struct PackedTables {
    pub bands: Vec<ffi::SkyBand>,
    pub atmosphere: Vec<ffi::SkyAtmospherePoint>,
    pub aerosol: Vec<ffi::SkyAerosolPoint>,
    pub aerosol_optics: Vec<ffi::SkyAerosolOptics>,
}

impl PackedTables {
    /// PackedScene::new (integrator.rs:319-418), table by table.
    pub fn new(scene: &SceneData) -> Self {
        let bands = scene
            .bands
            .iter()
            .enumerate()
            .map(|(band, value)| ffi::SkyBand {
                center_nm: value.center_nm,
                lower_nm: value.lower_nm,
                upper_nm: value.upper_nm,
                ozone_cross_section_cm2: value.ozone_cross_section_cm2,
                solar_radiance_w_m2_sr: scene.solar_radiance_w_m2_sr(band),
                rayleigh_cross_section_m2: scene.rayleigh_cross_sections_m2[band],
            })
            .collect();
        let atmosphere = scene
            .atmospheric_profile
            .iter()
            .map(|p| ffi::SkyAtmospherePoint {
                altitude_km: p.altitude_km,
                temperature_k: p.temperature_k,
                air_cm3: p.air_cm3,
                ozone_cm3: p.ozone_cm3,
            })
            .collect();
        let aerosol = scene
            .aerosol_profile
            .iter()
            .map(|p| ffi::SkyAerosolPoint { altitude_km: p.altitude_km, mass_g_m3: p.mass_g_m3, _pad: [0.0; 3] })
            .collect();
        let aerosol_optics = scene
            .aerosol_optics
            .iter()
            .flat_map(|band| {
                band.iter().map(|o| ffi::SkyAerosolOptics {
                    scattering_km_inv_per_g_m3: o.scattering_km_inv_per_g_m3,
                    absorption_km_inv_per_g_m3: o.absorption_km_inv_per_g_m3,
                })
            })
            .collect();
        Self { bands, atmosphere, aerosol, aerosol_optics }
    }

    /// The scene descriptor over these tables and `scene`'s grid, phase table
    /// and sun; it borrows both, so it must not outlive them.
    pub fn desc(&self, scene: &SceneData) -> ffi::SkySceneDesc {
        ffi::SkySceneDesc {
            band_count: self.bands.len() as u32,
            atmosphere_len: self.atmosphere.len() as u32,
            aerosol_len: self.aerosol.len() as u32,
            majorant_layers: scene.majorant_grid.layer_count as u32,
            phase_bins: PHASE_BINS as u32,
            _reserved0: 0,
            ground_radius_km: scene.planet.ground_radius_km,
            atmosphere_radius_km: scene.planet.atmosphere_radius_km,
            top_altitude_km: scene.majorant_grid.top_altitude_km,
            sun_direction: [scene.sun.direction.x, scene.sun.direction.y, scene.sun.direction.z],
            sun_angular_radius_rad: scene.sun.angular_radius_rad,
            sun_solid_angle_sr: scene.sun.solid_angle_sr,
            ground_albedo: GROUND_ALBEDO,
            _reserved1: 0.0,
            bands: self.bands.as_ptr(),
            atmosphere: self.atmosphere.as_ptr(),
            aerosol: self.aerosol.as_ptr(),
            aerosol_optics: self.aerosol_optics.as_ptr(),
            majorants_km_inv: scene.majorant_grid.values_km_inv.as_ptr(),
            phase_values: scene.phase_table.values().as_ptr(),
            band_xyz_weights: std::ptr::null(),
        }
    }
}

/// The reference's RenderConfig as the library's; the extension fields stay
/// zero, which renders what the reference shader renders.
pub fn render_config(config: &RenderConfig) -> ffi::SkyRenderConfig {
    ffi::SkyRenderConfig {
        width: config.width as u32,
        height: config.height as u32,
        spp: config.spp as u32,
        direct_light_samples: config.direct_light_samples as u32,
        seed: config.seed,
        sun_elevation_deg: config.sun_elevation_deg,
        sun_azimuth_deg: config.sun_azimuth_deg,
        observer_altitude_km: config.observer_altitude_km,
        output_projection: config.output_projection.as_gpu_u32(),
        ..Default::default()
    }
}

/// render (integrator.rs:125-128) on the GPU: synchronous, the device tables
/// created and freed inside the call, like the reference.
pub fn render(scene: &SceneData, config: &RenderConfig) -> Result<Film, RenderError> {
    // usize dimensions that do not fit the C ABI are the reference's InvalidConfig
    for (name, v) in [("width", config.width), ("height", config.height), ("spp", config.spp)] {
        if v > u32::MAX as usize {
            return Err(RenderError::InvalidConfig(format!("{name} does not fit 32 bits")));
        }
    }
    let tables = PackedTables::new(scene);
    let desc = tables.desc(scene);
    let cfg = render_config(config);
    let bands = tables.bands.len();
    let mut film = vec![0.0_f32; config.width * config.height * bands];
    let status =
        unsafe { ffi::sky_cuda_render_desc(&desc, &cfg, film.as_mut_ptr(), film.len(), std::ptr::null_mut()) };
    if status != ffi::SKY_OK {
        return Err(render_error(status, last_error()));
    }
    Ok(Film::from_values(config.width, config.height, bands, film))
}

/// A scene kept on the device between renders (sky_cuda_scene_create).
pub struct GpuScene {
    handle: *mut ffi::SkyScene,
    bands: usize,
}

impl GpuScene {
    pub fn new(scene: &SceneData) -> Result<Self, RenderError> {
        let tables = PackedTables::new(scene);
        let desc = tables.desc(scene);
        let mut handle = std::ptr::null_mut();
        let status = unsafe { ffi::sky_cuda_scene_create(&desc, &mut handle) };
        if status != ffi::SKY_OK {
            return Err(render_error(status, last_error()));
        }
        Ok(Self { handle, bands: tables.bands.len() })
    }

    /// One render of the resident scene; the film as `render` returns it.
    pub fn render(&self, config: &RenderConfig) -> Result<Film, RenderError> {
        let cfg = render_config(config);
        let mut film = vec![0.0_f32; config.width * config.height * self.bands];
        let status = unsafe {
            ffi::sky_cuda_render(self.handle, &cfg, film.as_mut_ptr(), film.len(), std::ptr::null_mut())
        };
        if status != ffi::SKY_OK {
            return Err(render_error(status, last_error()));
        }
        Ok(Film::from_values(config.width, config.height, self.bands, film))
    }
}

impl Drop for GpuScene {
    fn drop(&mut self) {
        unsafe { ffi::sky_cuda_scene_destroy(self.handle) };
    }
}

/// Device-side parameters of a differentiable render (SkyAdjointParams).
#[derive(Clone, Copy, Debug)]
pub struct AdjointParams {
    /// [3 * layers + 2]: (Rayleigh, Mie, ozone) density scale per majorant
    /// layer, then the Mie albedo and HG asymmetry.
    pub layer_params: *const f32,
    /// [bands][4] multipliers (Rayleigh, Mie, ozone, solar) or null for ones.
    pub band_params: *const f32,
    /// Unit sun direction, or all zero for the scene's own sun.
    pub sun_direction: [f32; 3],
    /// `ffi::SKY_ADJOINT_SEGMENT_INTEGRALS` or `ffi::SKY_ADJOINT_NULL_COLLISIONS`.
    pub estimator: u32,
    /// Optional [pixels][bands][spp] buffer: the forward writes each chain's
    /// radiance, a backward at the same parameters and sun replays each chain
    /// once instead of twice.
    pub chain_radiance: *mut f32,
    /// Floats in `chain_radiance` (the library refuses a shorter buffer).
    pub chain_radiance_len: u64,
}

impl AdjointParams {
    fn ffi(&self) -> ffi::SkyAdjointParams {
        ffi::SkyAdjointParams {
            layer_params: self.layer_params,
            band_params: self.band_params,
            sun_direction: self.sun_direction,
            estimator: self.estimator,
            chain_radiance: self.chain_radiance,
            chain_radiance_len: self.chain_radiance_len,
            ..Default::default()
        }
    }
}

/// The forward/backward pair of the differentiable render of one config on
/// a resident scene.  Tracking is merged-layer (residual carry over the
/// merged grid) and phase sampling tabulated unless the config is changed
/// through `config_mut`; the reference's segment-restart tracking is not
/// differentiable here.
pub struct Adjoint<'a> {
    scene: &'a GpuScene,
    config: ffi::SkyRenderConfig,
}

impl<'a> Adjoint<'a> {
    pub fn new(scene: &'a GpuScene, config: &RenderConfig) -> Self {
        let mut c = render_config(config);
        c.tracking = ffi::SKY_TRACKING_MERGED_LAYERS;
        c.phase_sampling = ffi::SKY_PHASE_TABULATED;
        Self { scene, config: c }
    }

    /// The render config (the starting point of a batch's `SkyAdjointJob`s).
    pub fn config(&self) -> ffi::SkyRenderConfig {
        self.config
    }

    pub fn config_mut(&mut self) -> &mut ffi::SkyRenderConfig {
        &mut self.config
    }

    /// Length of `AdjointParams::layer_params`: 3 * majorant layers + 2.
    pub fn param_count(&self) -> usize {
        unsafe { ffi::sky_cuda_adjoint_param_count(self.scene.handle) as usize }
    }

    /// Film, cell sums and status of the render at `params`, queued on
    /// `stream` (null: the default stream).
    ///
    /// # Safety
    /// Every pointer in `params` and `outputs` is device memory of the
    /// scene's GPU with the sizes include/sky_cuda.h gives (cell_sum and
    /// status required), live until the stream has run the call.
    pub unsafe fn forward(&self, params: &AdjointParams, outputs: &ffi::SkyDeviceOutputs,
                          stream: *mut c_void) -> Result<(), RenderError> {
        let p = params.ffi();
        let status = unsafe { ffi::sky_cuda_adjoint_forward(self.scene.handle, &self.config, &p, outputs, stream) };
        if status != ffi::SKY_OK {
            return Err(render_error(status, last_error()));
        }
        Ok(())
    }

    /// Forward renders of this config at several suns and views in one launch
    /// per 32 renders (`jobs[i].config`, `.sun_direction`, `.outputs`,
    /// `.chain_radiance`; `params.chain_radiance` is not read).
    ///
    /// # Safety
    /// As for `forward`, for every job.
    pub unsafe fn forward_batch(&self, params: &AdjointParams, jobs: &[ffi::SkyAdjointJob],
                                stream: *mut c_void) -> Result<(), RenderError> {
        let p = params.ffi();
        let status = unsafe {
            ffi::sky_cuda_adjoint_forward_batch(self.scene.handle, jobs.as_ptr(), jobs.len() as u32, &p, stream)
        };
        if status != ffi::SKY_OK {
            return Err(render_error(status, last_error()));
        }
        Ok(())
    }

    /// The gradient of the summed loss of a batch (`jobs[i].dloss_dfilm`),
    /// added to `grads.layer_grad` / `grads.band_grad` in one launch per 32
    /// renders.
    ///
    /// # Safety
    /// As for `backward`, for every job.
    pub unsafe fn backward_batch(&self, params: &AdjointParams, jobs: &[ffi::SkyAdjointJob],
                                 grads: &ffi::SkyAdjointGrads, stream: *mut c_void) -> Result<(), RenderError> {
        let p = params.ffi();
        let status = unsafe {
            ffi::sky_cuda_adjoint_backward_batch(self.scene.handle, jobs.as_ptr(), jobs.len() as u32, &p, grads,
                                                 stream)
        };
        if status != ffi::SKY_OK {
            return Err(render_error(status, last_error()));
        }
        Ok(())
    }

    /// Adds the gradient of the loss whose film derivative is
    /// `grads.dloss_dfilm` to `grads.layer_grad` / `grads.band_grad`, queued
    /// on `stream`.  The watchdog lands in `*grads.status` (read it after the
    /// stream has run the call).
    ///
    /// # Safety
    /// As for `forward`; `params.chain_radiance`, when set, holds what a
    /// forward at the same parameters, sun and config wrote.
    pub unsafe fn backward(&self, params: &AdjointParams, grads: &ffi::SkyAdjointGrads,
                           stream: *mut c_void) -> Result<(), RenderError> {
        let p = params.ffi();
        let status = unsafe { ffi::sky_cuda_adjoint_backward(self.scene.handle, &self.config, &p, grads, stream) };
        if status != ffi::SKY_OK {
            return Err(render_error(status, last_error()));
        }
        Ok(())
    }
}

#[cfg(test)]
mod tests {
    use super::*;

    #[test]
    fn statuses_map_to_distinct_render_errors() {
        assert!(matches!(render_error(1, "m".into()), RenderError::InvalidConfig(_)));
        assert!(matches!(render_error(2, "m".into()), RenderError::NoAdapter(_)));
        assert!(matches!(render_error(3, "m".into()), RenderError::RequestDevice(_)));
        assert!(matches!(render_error(4, "m".into()), RenderError::BufferMap(_)));
        assert!(matches!(render_error(5, "m".into()), RenderError::Poll(_)));
        assert!(matches!(render_error(6, "m".into()), RenderError::Watchdog));
        let text = |s| render_error(s, "m".into()).to_string();
        assert!(text(7).contains("out of device memory"));
        assert!(text(8).contains("kernel launch failed"));
        assert!(text(9).contains("table input failed"));
    }
}
