//! The reference's smoke test (crates/sky-spectral-path-tracer/tests/smoke.rs)
//! against `sky_cuda::render`: a tiny render returns a finite, non-negative,
//! non-zero spectral film; a machine without a CUDA device skips, as the
//! reference skips without a wgpu adapter.

use std::path::Path;

use sky_core::data::load_scene_data;
use sky_cuda::{RenderConfig, RenderError, render};

#[test]
fn tiny_render_returns_finite_spectral_film() -> Result<(), Box<dyn std::error::Error>> {
    let config = RenderConfig { width: 32, height: 16, spp: 2, ..RenderConfig::default() };
    let scene = load_scene_data(&repository_data_dir(), 0.0, 0.0).expect("scene data");
    let film = match render(&scene, &config) {
        Ok(film) => film,
        Err(RenderError::NoAdapter(_)) => return Ok(()),
        Err(err) => return Err(err.into()),
    };
    assert!(film.values().iter().all(|x| x.is_finite() && *x >= 0.0));
    assert!(film.values().iter().any(|x| *x > 0.0));
    Ok(())
}

#[test]
fn invalid_config_is_reported_like_the_reference() {
    let scene = load_scene_data(&repository_data_dir(), 0.0, 0.0).expect("scene data");
    let config = RenderConfig { width: 0, height: 16, spp: 2, ..RenderConfig::default() };
    match render(&scene, &config) {
        Err(RenderError::InvalidConfig(message)) => assert!(message.contains("greater than zero")),
        Err(RenderError::NoAdapter(_)) => {}
        other => panic!("expected InvalidConfig, got {other:?}"),
    }
}

fn repository_data_dir() -> std::path::PathBuf {
    Path::new(env!("CARGO_MANIFEST_DIR")).join("..").join("..").join("data")
}
