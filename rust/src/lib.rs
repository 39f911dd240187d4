//! Renderer entry point of the crate on top of the raw binding: render a
//! scene JSON with an integrator JSON into a linear RGB image. The image
//! size is the scene camera's `res` (`scenes/cbox.json:518-521`); every
//! handle is released on every path.

pub mod ffi;

use std::ffi::{CStr, CString};
use crate::ffi::*;

unsafe fn check(status: aqua_status, ctx: *const aqua_ctx) -> Result<(), String> {
    if status == AQUA_OK {
        return Ok(());
    }
    // aqua_create failures are reported by aqua_last_error(NULL)
    Err(CStr::from_ptr(aqua_last_error(ctx)).to_string_lossy().into_owned())
}

/// (width, height, width*height*3 linear RGB floats, row 0 at the top)
pub fn render(scene: &str, integrator: &str) -> Result<(u32, u32, Vec<f32>), String> {
    let scene = CString::new(scene).map_err(|e| e.to_string())?;
    let integrator = CString::new(integrator).map_err(|e| e.to_string())?;
    unsafe {
        let mut ctx = std::ptr::null_mut();
        let opt = aqua_options { device: -1, ..Default::default() };
        check(aqua_create(&mut ctx, &opt), std::ptr::null())?;
        let image = render_on(ctx, &scene, &integrator);
        aqua_destroy(ctx);
        image
    }
}

unsafe fn render_on(ctx: *mut aqua_ctx, scene: &CStr, integrator: &CStr)
        -> Result<(u32, u32, Vec<f32>), String> {
    let mut cfg = aqua_integrator_cfg::default();
    check(aqua_load_integrator_json(ctx, integrator.as_ptr(), &mut cfg), ctx)?;
    let mut s = std::ptr::null_mut();
    check(aqua_load_scene_json(ctx, scene.as_ptr(), 0, &mut s), ctx)?;
    let mut info = aqua_scene_info::default();
    let mut status = aqua_scene_get_info(ctx, s, &mut info);
    let (w, h) = (info.width.max(0) as u32, info.height.max(0) as u32);
    let mut rgb = vec![0f32; w as usize * h as usize * 3];
    if status == AQUA_OK {
        status = aqua_render(ctx, s, &cfg, std::ptr::null(), rgb.as_mut_ptr(), 0, std::ptr::null_mut());
    }
    let result = check(status, ctx).map(|_| (w, h, rgb));
    aqua_scene_free(ctx, s);
    result
}
