//! Raw FFI bindings to libgvs: the C ABI of include/gvs.h, declaration for
//! declaration (tests/test_rust_ffi_cpu.py checks that every function and
//! argument here matches the header).  libgvs is the GB300 (CUDA sm_103a)
//! engine for sim-core's force calculation and time integration: BruteForce,
//! BarnesHut, LeapfrogKDK and the SPH solver, plus mixed precision, adjoint
//! gradients and batched ensembles.  build.rs compiles it from source with nvcc.
//!
//! Conventions (see include/gvs.h): every function returns a gvs_status and
//! never unwinds; host arrays are the f64 Vec fields of sim-core's Particles in
//! the caller's order, borrowed for one call; "accumulate" entry points add to
//! the caller's (zeroed) acceleration arrays, as GravitySolver requires.  One
//! context is used by one thread at a time.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_longlong, c_uint, c_void};

pub type gvs_status = c_int;
pub const GVS_OK: gvs_status = 0;
pub const GVS_ERR_INVALID_ARG: gvs_status = 1;
pub const GVS_ERR_OOM: gvs_status = 2;
pub const GVS_ERR_LAUNCH: gvs_status = 3;
pub const GVS_ERR_DEVICE: gvs_status = 4;
pub const GVS_ERR_TIMEOUT: gvs_status = 5;
pub const GVS_ERR_INJECTED: gvs_status = 6;
pub const GVS_ERR_NO_DEVICE: gvs_status = 7;
pub const GVS_ERR_STATE: gvs_status = 8;

pub const GVS_PREC_FP64_EXACT: c_int = 0;
pub const GVS_PREC_FP64: c_int = 1;
pub const GVS_PREC_FP32: c_int = 2;
pub const GVS_PREC_MIXED: c_int = 3;

pub const GVS_ALGO_NONE: c_int = 0;
pub const GVS_ALGO_DIRECT: c_int = 1;
pub const GVS_ALGO_BH: c_int = 2;

/// Opaque engine context (one CUDA stream, the device-resident state, scratch).
#[repr(C)]
pub struct gvs_ctx {
    _private: [u8; 0],
}

/// Diagnostics::compute (crates/sim-core/src/diagnostics.rs:37-148).
#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct gvs_diag {
    pub kinetic_energy: f64,
    pub potential_energy: f64,
    pub thermal_energy: f64,
    pub total_energy: f64,
    pub momentum: [f64; 3],
    pub angular_momentum: [f64; 3],
    pub center_of_mass: [f64; 3],
    pub center_of_mass_velocity: [f64; 3],
    pub virial_ratio: f64,
}

/// SphSolver::new + ForceParams::default (crates/sim-core/src/sph/solver.rs:40-49,
/// crates/sim-core/src/sph/forces.rs:30-41); fill with gvs_sph_params_default.
#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct gvs_sph_params {
    pub gamma: f64,
    pub eta: f64,
    pub cfl_factor: f64,
    pub force_factor: f64,
    pub h_max: f64,
    pub beta_visc: f64,
    pub alpha_min: f64,
    pub alpha_max: f64,
    pub alpha_cond: f64,
    pub sigma_visc: f64,
    pub precision: c_int,
}

/// Kernel-time counters of one context.
#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct gvs_profile {
    pub force_ms: f64,
    pub force_launches: c_longlong,
    pub launches: c_longlong,
    pub force_flops: f64,
    pub force_bytes: f64,
    pub tile_visits: f64,
    pub near_tile_visits: f64,
    pub vjp_ms: f64,
    pub vjp_launches: c_longlong,
    pub sph_f64_redo: c_longlong,
    pub bh_groups: c_longlong,
    pub bh_group_fallbacks: c_longlong,
    pub bh_group_iterations: c_longlong,
    pub bh_group_interactions: c_longlong,
    pub bh_walk_terms: c_longlong,
}

unsafe extern "C" {
    pub fn gvs_version() -> *const c_char;
    pub fn gvs_create(out: *mut *mut gvs_ctx, device: c_int) -> gvs_status;
    pub fn gvs_destroy(ctx: *mut gvs_ctx) -> gvs_status;
    pub fn gvs_last_error(ctx: *const gvs_ctx, buf: *mut c_char, len: usize) -> gvs_status;
    pub fn gvs_set_fault(ctx: *mut gvs_ctx, spec: *const c_char) -> gvs_status;
    pub fn gvs_sync(ctx: *mut gvs_ctx) -> gvs_status;
    pub fn gvs_device_errors(ctx: *mut gvs_ctx, flags: *mut c_uint) -> gvs_status;
    pub fn gvs_set_state(ctx: *mut gvs_ctx, n: usize, x: *const f64, y: *const f64, z: *const f64,
        vx: *const f64, vy: *const f64, vz: *const f64, mass: *const f64, ptype: *const u8, u: *const f64,
        h: *const f64, alpha: *const f64) -> gvs_status;
    pub fn gvs_get_state(ctx: *mut gvs_ctx, x: *mut f64, y: *mut f64, z: *mut f64, vx: *mut f64, vy: *mut f64,
        vz: *mut f64, ax: *mut f64, ay: *mut f64, az: *mut f64) -> gvs_status;
    pub fn gvs_set_accelerations(ctx: *mut gvs_ctx, ax: *const f64, ay: *const f64,
        az: *const f64) -> gvs_status;
    pub fn gvs_get_gas(ctx: *mut gvs_ctx, density: *mut f64, pressure: *mut f64, u: *mut f64, du_dt: *mut f64,
        h: *mut f64, sound_speed: *mut f64, alpha: *mut f64) -> gvs_status;
    pub fn gvs_set_gas(ctx: *mut gvs_ctx, density: *const f64, pressure: *const f64, u: *const f64,
        du_dt: *const f64, h: *const f64, sound_speed: *const f64, alpha: *const f64) -> gvs_status;
    pub fn gvs_count(ctx: *const gvs_ctx) -> usize;
    pub fn gvs_gravity_direct(ctx: *mut gvs_ctx, n: usize, x: *const f64, y: *const f64, z: *const f64,
        mass: *const f64, softening: f64, precision: c_int, ax: *mut f64, ay: *mut f64,
        az: *mut f64) -> gvs_status;
    pub fn gvs_gravity_bh(ctx: *mut gvs_ctx, n: usize, x: *const f64, y: *const f64, z: *const f64,
        mass: *const f64, softening: f64, theta: f64, precision: c_int, ax: *mut f64, ay: *mut f64,
        az: *mut f64) -> gvs_status;
    pub fn gvs_tree_export(ctx: *mut gvs_ctx, cap: usize, nnodes: *mut usize, level: *mut u8, first: *mut u32,
        count: *mut u32, skip: *mut u32, mass: *mut f64, com: *mut f64, order: *mut u32,
        keys: *mut u64) -> gvs_status;
    pub fn gvs_compute_forces(ctx: *mut gvs_ctx, algo: c_int, precision: c_int, softening: f64,
        theta: f64) -> gvs_status;
    pub fn gvs_kdk_steps(ctx: *mut gvs_ctx, algo: c_int, precision: c_int, softening: f64, theta: f64,
        dt: f64, nsteps: c_longlong) -> gvs_status;
    pub fn gvs_kdk_step_host(ctx: *mut gvs_ctx, n: usize, x: *mut f64, y: *mut f64, z: *mut f64, vx: *mut f64,
        vy: *mut f64, vz: *mut f64, ax: *mut f64, ay: *mut f64, az: *mut f64, mass: *const f64, algo: c_int,
        precision: c_int, softening: f64, theta: f64, dt: f64) -> gvs_status;
    pub fn gvs_diagnostics(ctx: *mut gvs_ctx, softening: f64, with_potential: c_int,
        out: *mut gvs_diag) -> gvs_status;
    pub fn gvs_adjoint_forward(ctx: *mut gvs_ctx, precision: c_int, softening: f64, dt: f64,
        nsteps: c_longlong, checkpoint_every: c_longlong) -> gvs_status;
    pub fn gvs_adjoint_backward(ctx: *mut gvs_ctx, dl_dx: *const f64, dl_dy: *const f64, dl_dz: *const f64,
        dl_dvx: *const f64, dl_dvy: *const f64, dl_dvz: *const f64, g_x: *mut f64, g_y: *mut f64,
        g_z: *mut f64, g_vx: *mut f64, g_vy: *mut f64, g_vz: *mut f64, g_m: *mut f64) -> gvs_status;
    pub fn gvs_adjoint_checkpoints(ctx: *mut gvs_ctx, cap: c_longlong, count: *mut c_longlong,
        steps: *mut c_longlong) -> gvs_status;
    pub fn gvs_adjoint_checkpoint_read(ctx: *mut gvs_ctx, k: c_longlong, x: *mut f64, y: *mut f64, z: *mut f64,
        vx: *mut f64, vy: *mut f64, vz: *mut f64) -> gvs_status;
    pub fn gvs_adjoint_prepare(ctx: *mut gvs_ctx, precision: c_int, softening: f64, dt: f64,
        nsteps: c_longlong, checkpoint_every: c_longlong) -> gvs_status;
    pub fn gvs_adjoint_checkpoint_write(ctx: *mut gvs_ctx, k: c_longlong, x: *const f64, y: *const f64,
        z: *const f64, vx: *const f64, vy: *const f64, vz: *const f64) -> gvs_status;
    pub fn gvs_ensemble_setup(ctx: *mut gvs_ctx, nsys: c_int, sizes: *const i64,
        softening: f64) -> gvs_status;
    pub fn gvs_ensemble_forces(ctx: *mut gvs_ctx) -> gvs_status;
    pub fn gvs_ensemble_kdk_steps(ctx: *mut gvs_ctx, dt: f64, nsteps: c_longlong,
        use_graph: c_int) -> gvs_status;
    pub fn gvs_sph_params_default(out: *mut gvs_sph_params) -> gvs_status;
    pub fn gvs_sph_compute(ctx: *mut gvs_ctx, params: *const gvs_sph_params, omega: *mut f64, div_v: *mut f64,
        max_mu: *mut f64, dalpha_dt: *mut f64) -> gvs_status;
    pub fn gvs_sph_timestep(ctx: *mut gvs_ctx, params: *const gvs_sph_params, dt: *mut f64) -> gvs_status;
    pub fn gvs_sph_step(ctx: *mut gvs_ctx, params: *const gvs_sph_params, algo: c_int, precision: c_int,
        softening: f64, theta: f64, dt: f64, dt_next: *mut f64) -> gvs_status;
    pub fn gvs_sph_neighbors(ctx: *mut gvs_ctx, cap: usize, total: *mut usize, start: *mut u32,
        count: *mut u32, idx: *mut u32) -> gvs_status;
    pub fn gvs_diagnostics_noalloc(device: c_int, stream: *mut c_void, n: usize, x: *const f64, y: *const f64,
        z: *const f64, vx: *const f64, vy: *const f64, vz: *const f64, mass: *const f64, ptype: *const u8,
        u: *const f64, softening: f64, with_potential: c_int, out: *mut gvs_diag) -> gvs_status;
    pub fn gvs_direct_subset(ctx: *mut gvs_ctx, precision: c_int, softening: f64, idx: *const i64,
        nidx: usize, out_ax: *mut f64, out_ay: *mut f64, out_az: *mut f64) -> gvs_status;
    pub fn gvs_autotune_direct(ctx: *mut gvs_ctx, precision: c_int, softening: f64, nthreads: *mut c_int,
        ipt: *mut c_int, ms: *mut f64) -> gvs_status;
    pub fn gvs_set_direct_shape(ctx: *mut gvs_ctx, nthreads: c_int, ipt: c_int, min_blocks: c_int,
        unroll: c_int) -> gvs_status;
    pub fn gvs_set_bh_walk(ctx: *mut gvs_ctx, group_size: c_int, budget: c_int) -> gvs_status;
    pub fn gvs_autotune_report(ctx: *mut gvs_ctx, cap: c_int, count: *mut c_int, nthreads: *mut c_int,
        ipt: *mut c_int, min_blocks: *mut c_int, unroll: *mut c_int, ms: *mut f64) -> gvs_status;
    pub fn gvs_ic_plummer(n: usize, seed: u64, scale_radius: f64, total_mass: f64, x: *mut f64, y: *mut f64,
        z: *mut f64, vx: *mut f64, vy: *mut f64, vz: *mut f64, mass: *mut f64) -> gvs_status;
    pub fn gvs_ic_plummer_device(ctx: *mut gvs_ctx, n: usize, seed: u64, scale_radius: f64,
        total_mass: f64) -> gvs_status;
    pub fn gvs_ic_collision_device(ctx: *mut gvs_ctx, n: usize, seed: u64, separation: f64) -> gvs_status;
    pub fn gvs_ic_two_body(mass_ratio: f64, e: f64, a: f64, x: *mut f64, y: *mut f64, z: *mut f64,
        vx: *mut f64, vy: *mut f64, vz: *mut f64, mass: *mut f64) -> gvs_status;
    pub fn gvs_ic_evrard(n: usize, seed: u64, total_mass: f64, radius: f64, u0: f64, x: *mut f64, y: *mut f64,
        z: *mut f64, mass: *mut f64, u: *mut f64, h: *mut f64) -> gvs_status;
    pub fn gvs_ic_cold_collapse(n: usize, seed: u64, radius: f64, total_mass: f64, sph: c_int, x: *mut f64,
        y: *mut f64, z: *mut f64, vx: *mut f64, vy: *mut f64, vz: *mut f64, mass: *mut f64, u: *mut f64,
        h: *mut f64) -> gvs_status;
    pub fn gvs_ic_collision(n: usize, seed: u64, separation: f64, x: *mut f64, y: *mut f64, z: *mut f64,
        vx: *mut f64, vy: *mut f64, vz: *mut f64, mass: *mut f64) -> gvs_status;
    pub fn gvs_ic_gas_sphere_1r(n: usize, total_mass: f64, radius: f64, u0: f64, eta: f64, x: *mut f64,
        y: *mut f64, z: *mut f64, mass: *mut f64, u: *mut f64, h: *mut f64) -> gvs_status;
    pub fn gvs_ic_ensemble_sizes(count: usize, seed: u64, lo: f64, hi: f64, sizes: *mut i64) -> gvs_status;
    pub fn gvs_profile_enable(ctx: *mut gvs_ctx, on: c_int) -> gvs_status;
    pub fn gvs_profile_read(ctx: *mut gvs_ctx, out: *mut gvs_profile) -> gvs_status;
    pub fn gvs_event_record(ctx: *mut gvs_ctx, slot: c_int) -> gvs_status;
    pub fn gvs_event_elapsed(ctx: *mut gvs_ctx, slot_a: c_int, slot_b: c_int, ms: *mut f32) -> gvs_status;
    pub fn gvs_stream(ctx: *mut gvs_ctx, stream: *mut *mut c_void) -> gvs_status;
    pub fn gvs_l2_flush(ctx: *mut gvs_ctx) -> gvs_status;
    pub fn gvs_check_bounded_wait(ctx: *mut gvs_ctx, polls: c_uint) -> gvs_status;
    pub fn gvs_measure_fp32_peak(ctx: *mut gvs_ctx, tflops: *mut f64) -> gvs_status;
    pub fn gvs_fp32_peak_variants(ctx: *mut gvs_ctx, scalar: *mut f64, packed: *mut f64,
        mixed: *mut f64) -> gvs_status;
}
