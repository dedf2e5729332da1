//! Declarations of include/sky_cuda.h used by this crate.  Every struct is
//! `#[repr(C)]` with the header's field order; the table rows have the byte
//! layout of the reference's GPU structs (integrator.rs:77-112).

use std::os::raw::{c_char, c_int, c_void};

pub const SKY_OK: c_int = 0;
pub const SKY_ERR_INVALID_CONFIG: c_int = 1;
pub const SKY_ERR_NO_DEVICE: c_int = 2;
pub const SKY_ERR_DEVICE_INIT: c_int = 3;
pub const SKY_ERR_COPY: c_int = 4;
pub const SKY_ERR_SYNC: c_int = 5;
pub const SKY_ERR_WATCHDOG: c_int = 6;
pub const SKY_ERR_OUT_OF_MEMORY: c_int = 7;
pub const SKY_ERR_LAUNCH: c_int = 8;
pub const SKY_ERR_IO: c_int = 9;

/// SkyRenderConfig.flags bits.
pub const SKY_FLAG_ACCUMULATE: u32 = 1;
pub const SKY_FLAG_COUNT_EVENTS: u32 = 2;

/// SkyRenderConfig.phase_sampling and .tracking values.
pub const SKY_PHASE_ISOTROPIC: u32 = 0;
pub const SKY_PHASE_TABULATED: u32 = 1;
pub const SKY_TRACKING_SEGMENT_RESTART: u32 = 0;
pub const SKY_TRACKING_RESIDUAL_CARRY: u32 = 1;
pub const SKY_TRACKING_MERGED_LAYERS: u32 = 2;

/// Differentiable rendering: band multipliers per band, and the estimators
/// of the backward pass (SkyAdjointEstimator).
pub const SKY_ADJOINT_BAND_PARAMS: u32 = 4;
pub const SKY_ADJOINT_SEGMENT_INTEGRALS: u32 = 0;
pub const SKY_ADJOINT_NULL_COLLISIONS: u32 = 1;

/// = GpuBand (integrator.rs:79-86), 24 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct SkyBand {
    pub center_nm: f32,
    pub lower_nm: f32,
    pub upper_nm: f32,
    pub ozone_cross_section_cm2: f32,
    pub solar_radiance_w_m2_sr: f32,
    pub rayleigh_cross_section_m2: f32,
}

/// = GpuAtmospherePoint (integrator.rs:90-95), 16 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct SkyAtmospherePoint {
    pub altitude_km: f32,
    pub temperature_k: f32,
    pub air_cm3: f32,
    pub ozone_cm3: f32,
}

/// = GpuAerosolPoint (integrator.rs:99-105), 32 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct SkyAerosolPoint {
    pub altitude_km: f32,
    pub mass_g_m3: [f32; 4],
    pub _pad: [f32; 3],
}

/// = GpuAerosolOptics (integrator.rs:109-112), 8 bytes.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct SkyAerosolOptics {
    pub scattering_km_inv_per_g_m3: f32,
    pub absorption_km_inv_per_g_m3: f32,
}

#[repr(C)]
pub struct SkySceneDesc {
    pub band_count: u32,
    pub atmosphere_len: u32,
    pub aerosol_len: u32,
    pub majorant_layers: u32,
    pub phase_bins: u32,
    pub _reserved0: u32,
    pub ground_radius_km: f32,
    pub atmosphere_radius_km: f32,
    pub top_altitude_km: f32,
    pub sun_direction: [f32; 3],
    pub sun_angular_radius_rad: f32,
    pub sun_solid_angle_sr: f32,
    pub ground_albedo: f32,
    pub _reserved1: f32,
    pub bands: *const SkyBand,
    pub atmosphere: *const SkyAtmospherePoint,
    pub aerosol: *const SkyAerosolPoint,
    pub aerosol_optics: *const SkyAerosolOptics,
    pub majorants_km_inv: *const f32,
    pub phase_values: *const f32,
    pub band_xyz_weights: *const f32,
}

/// = RenderConfig (config.rs:2-12) followed by the extensions; all-zero
/// extensions render what the reference shader renders.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct SkyRenderConfig {
    pub width: u32,
    pub height: u32,
    pub spp: u32,
    pub direct_light_samples: u32,
    pub seed: u64,
    pub sun_elevation_deg: f32,
    pub sun_azimuth_deg: f32,
    pub observer_altitude_km: f32,
    pub output_projection: u32,
    pub sample_offset: u32,
    pub phase_sampling: u32,
    pub rr_start_depth: u32,
    pub max_orders: u32,
    pub watchdog_limit: u32,
    pub kernel: u32,
    pub flags: u32,
    pub tracking: u32,
    pub row_begin: u32,
    pub row_count: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct SkyRenderStats {
    pub kernel_ms: f64,
    pub total_ms: f64,
    pub chains: u64,
    pub events: [u64; 8],
    pub watchdog: u32,
    pub kernel_used: u32,
}

/// Device buffers of one render (SkyDeviceOutputs); null where not wanted.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct SkyDeviceOutputs {
    pub cell_sum: *mut f64,
    pub cell_sumsq: *mut f64,
    pub film: *mut f32,
    pub xyz: *mut f64,
    pub xyz_var: *mut f64,
    pub counters: *mut u64,
    pub status: *mut u32,
    pub rgb: *mut f32,
}

impl Default for SkyDeviceOutputs {
    fn default() -> Self {
        let n = std::ptr::null_mut();
        Self { cell_sum: n, cell_sumsq: n, film: std::ptr::null_mut(), xyz: n, xyz_var: n,
               counters: std::ptr::null_mut(), status: std::ptr::null_mut(), rgb: std::ptr::null_mut() }
    }
}

/// Parameters of a differentiable render (SkyAdjointParams); device pointers.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct SkyAdjointParams {
    pub layer_params: *const f32,
    pub band_params: *const f32,
    pub sample_layer_params: *const f32,
    pub sample_band_params: *const f32,
    pub sun_direction: [f32; 3],
    pub estimator: u32,
    pub chain_radiance: *mut f32,
    pub chain_radiance_len: u64,
}

impl Default for SkyAdjointParams {
    fn default() -> Self {
        Self { layer_params: std::ptr::null(), band_params: std::ptr::null(), sample_layer_params: std::ptr::null(),
               sample_band_params: std::ptr::null(), sun_direction: [0.0; 3], estimator: SKY_ADJOINT_SEGMENT_INTEGRALS,
               chain_radiance: std::ptr::null_mut(), chain_radiance_len: 0 }
    }
}

/// Gradient request of a backward call (SkyAdjointGrads); device pointers.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct SkyAdjointGrads {
    pub dloss_dfilm: *const f32,
    pub layer_grad: *mut f64,
    pub band_grad: *mut f64,
    pub counters: *mut u64,
    pub status: *mut u32,
}

/// One render of a differentiable batch (SkyAdjointJob).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct SkyAdjointJob {
    pub config: SkyRenderConfig,
    pub sun_direction: [f32; 3],
    pub _reserved: f32,
    pub outputs: SkyDeviceOutputs,
    pub dloss_dfilm: *const f32,
    pub chain_radiance: *mut f32,
    pub chain_radiance_len: u64,
}

/// Opaque scene handle (device tables owned by the library).
#[repr(C)]
pub struct SkyScene {
    _opaque: [u8; 0],
}

unsafe extern "C" {
    pub fn sky_cuda_version() -> *const c_char;
    pub fn sky_cuda_last_error(buf: *mut c_char, buf_len: usize) -> c_int;
    pub fn sky_cuda_scene_create(desc: *const SkySceneDesc, out_scene: *mut *mut SkyScene) -> c_int;
    pub fn sky_cuda_scene_destroy(scene: *mut SkyScene);
    pub fn sky_cuda_render(scene: *const SkyScene, config: *const SkyRenderConfig, film_out: *mut f32,
                           film_len: usize, stats: *mut SkyRenderStats) -> c_int;
    pub fn sky_cuda_render_desc(desc: *const SkySceneDesc, config: *const SkyRenderConfig, film_out: *mut f32,
                                film_len: usize, stats: *mut SkyRenderStats) -> c_int;
    pub fn sky_cuda_render_device(scene: *const SkyScene, config: *const SkyRenderConfig,
                                  outputs: *const SkyDeviceOutputs, cuda_stream: *mut c_void) -> c_int;
    pub fn sky_cuda_adjoint_param_count(scene: *const SkyScene) -> u32;
    pub fn sky_cuda_adjoint_forward(scene: *const SkyScene, config: *const SkyRenderConfig,
                                    params: *const SkyAdjointParams, outputs: *const SkyDeviceOutputs,
                                    cuda_stream: *mut c_void) -> c_int;
    pub fn sky_cuda_adjoint_backward(scene: *const SkyScene, config: *const SkyRenderConfig,
                                     params: *const SkyAdjointParams, grads: *const SkyAdjointGrads,
                                     cuda_stream: *mut c_void) -> c_int;
    pub fn sky_cuda_adjoint_forward_batch(scene: *const SkyScene, jobs: *const SkyAdjointJob, job_count: u32,
                                          params: *const SkyAdjointParams, cuda_stream: *mut c_void) -> c_int;
    pub fn sky_cuda_adjoint_backward_batch(scene: *const SkyScene, jobs: *const SkyAdjointJob, job_count: u32,
                                           params: *const SkyAdjointParams, grads: *const SkyAdjointGrads,
                                           cuda_stream: *mut c_void) -> c_int;
}

#[cfg(test)]
mod layout {
    use super::*;
    use std::mem::size_of;

    #[test]
    fn rows_have_the_reference_gpu_layouts() {
        // integrator.rs:479-510 checks the same sizes for GpuBand and friends
        assert_eq!(size_of::<SkyBand>(), 24);
        assert_eq!(size_of::<SkyAtmospherePoint>(), 16);
        assert_eq!(size_of::<SkyAerosolPoint>(), 32);
        assert_eq!(size_of::<SkyAerosolOptics>(), 8);
        assert_eq!(size_of::<SkySceneDesc>(), 120);
        assert_eq!(size_of::<SkyRenderConfig>(), 80);
        assert_eq!(size_of::<SkyRenderStats>(), 96);
        assert_eq!(size_of::<SkyDeviceOutputs>(), 64);
        assert_eq!(size_of::<SkyAdjointParams>(), 64);
        assert_eq!(size_of::<SkyAdjointGrads>(), 40);
        assert_eq!(size_of::<SkyAdjointJob>(), 184);
    }
}
