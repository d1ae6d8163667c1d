//! GB300 drop-ins for gravis sim-core's force and integration interfaces.
//!
//! - [`GpuGravity`] implements `GravitySolver` (crates/sim-core/src/gravity.rs:6-10) for the
//!   direct sum (BruteForce, gravity.rs:47-80) and Barnes-Hut (barnes_hut.rs:139-192), with
//!   the same accumulate contract: the caller zeroes the accelerations, the solver adds.
//!   With `Precision::Fp64Exact` the direct sum returns BruteForce's bits.
//! - [`GpuLeapfrog`] implements `Integrator` (integrator.rs:5-8, LeapfrogKDK 42-76) with the
//!   whole kick-drift-force-kick step on the GPU.
//! - [`GpuSph`] has SphSolver's surface (sph/solver.rs:61-131): `compute`,
//!   `compute_timestep`, and `step_with_sph` (solver.rs:145-212).
//! - [`gravity_for`] maps headless `--algorithm gpu-direct|gpu-bh` names to a solver
//!   (the wiring point is crates/headless/src/main.rs:114-121).
//!
//! Every libgvs status other than OK becomes an [`Error`] with libgvs' message; the trait
//! methods, which return `()`, panic with it, as the reference's `.expect` calls do.
use std::ffi::CStr;
use std::os::raw::c_int;
use std::sync::{Arc, Mutex};

use gvs_sys as sys;
use sim_core::gravity::GravitySolver;
use sim_core::integrator::Integrator;
use sim_core::particle::Particles;
use sim_core::sph::forces::ForceIntermediates;

/// A libgvs failure: its status code and message.
#[derive(Debug, Clone)]
pub struct Error {
    pub status: i32,
    pub message: String,
}

impl std::fmt::Display for Error {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        write!(f, "libgvs status {}: {}", self.status, self.message)
    }
}

impl std::error::Error for Error {}

pub type Result<T> = std::result::Result<T, Error>;

/// Force arithmetic (include/gvs.h GVS_PREC_*).
#[derive(Debug, Clone, Copy, PartialEq, Eq)]
pub enum Precision {
    /// f64 with the reference's operation order: BruteForce's bits.
    Fp64Exact,
    /// f64 tiled kernel (FMA).
    Fp64,
    /// f32 pairs on absolute positions.
    Fp32,
    /// f32 pairs on f64 tile centres with compensated sums (force error ~1e-7).
    Mixed,
}

impl Precision {
    fn raw(self) -> c_int {
        match self {
            Precision::Fp64Exact => sys::GVS_PREC_FP64_EXACT,
            Precision::Fp64 => sys::GVS_PREC_FP64,
            Precision::Fp32 => sys::GVS_PREC_FP32,
            Precision::Mixed => sys::GVS_PREC_MIXED,
        }
    }

    /// Parses the headless `--precision` names: fp64-exact, fp64, fp32, mixed.
    pub fn parse(name: &str) -> Option<Self> {
        match name {
            "fp64-exact" | "exact" => Some(Precision::Fp64Exact),
            "fp64" => Some(Precision::Fp64),
            "fp32" => Some(Precision::Fp32),
            "mixed" => Some(Precision::Mixed),
            _ => None,
        }
    }
}

/// The force a solver or integrator computes.
#[derive(Debug, Clone, Copy, PartialEq)]
pub enum Force {
    Direct,
    BarnesHut { theta: f64 },
}

impl Force {
    fn algo(self) -> c_int {
        match self {
            Force::Direct => sys::GVS_ALGO_DIRECT,
            Force::BarnesHut { .. } => sys::GVS_ALGO_BH,
        }
    }

    fn theta(self) -> f64 {
        match self {
            Force::Direct => 0.0,
            Force::BarnesHut { theta } => theta,
        }
    }
}

struct Raw(*mut sys::gvs_ctx);

// The context is only touched under the Mutex of `Context`, one thread at a time, which is
// what libgvs requires of a gvs_ctx.
unsafe impl Send for Raw {}

impl Drop for Raw {
    fn drop(&mut self) {
        unsafe {
            sys::gvs_destroy(self.0);
        }
    }
}

/// One libgvs context on one GPU (a CUDA stream, the device-resident particle state and
/// its scratch).  Clones share the context; calls serialise on a mutex, the pattern of
/// BarnesHut's tree cache (barnes_hut.rs:27,146), so solvers built on it are Send + Sync.
#[derive(Clone)]
pub struct Context {
    inner: Arc<Mutex<Raw>>,
}

fn message(ctx: *const sys::gvs_ctx) -> String {
    let mut buf = vec![0 as std::os::raw::c_char; 512];
    unsafe {
        sys::gvs_last_error(ctx, buf.as_mut_ptr(), buf.len());
        CStr::from_ptr(buf.as_ptr()).to_string_lossy().into_owned()
    }
}

fn check(ctx: *const sys::gvs_ctx, status: sys::gvs_status) -> Result<()> {
    if status == sys::GVS_OK {
        Ok(())
    } else {
        Err(Error { status, message: message(ctx) })
    }
}

fn ptr_or_null(v: &[f64], use_it: bool) -> *const f64 {
    if use_it { v.as_ptr() } else { std::ptr::null() }
}

impl Context {
    /// Creates a context on CUDA device `device`.
    pub fn new(device: i32) -> Result<Self> {
        let mut c: *mut sys::gvs_ctx = std::ptr::null_mut();
        check(std::ptr::null(), unsafe { sys::gvs_create(&mut c, device) })?;
        Ok(Context { inner: Arc::new(Mutex::new(Raw(c))) })
    }

    fn with<T>(&self, f: impl FnOnce(*mut sys::gvs_ctx) -> Result<T>) -> Result<T> {
        let g = self.inner.lock().unwrap_or_else(|e| e.into_inner());
        f(g.0)
    }

    /// Uploads every Particles field the engine uses (particle.rs:22-64); accelerations
    /// are uploaded too, so a KDK step can start from them.
    pub fn set_state(&self, p: &Particles) -> Result<()> {
        let gas = p.has_gas();
        self.with(|c| unsafe {
            check(c, sys::gvs_set_state(c, p.count, p.x.as_ptr(), p.y.as_ptr(), p.z.as_ptr(), p.vx.as_ptr(),
                p.vy.as_ptr(), p.vz.as_ptr(), p.mass.as_ptr(),
                if gas { p.particle_type.as_ptr() } else { std::ptr::null() },
                ptr_or_null(&p.internal_energy, gas), ptr_or_null(&p.smoothing_length, gas),
                ptr_or_null(&p.alpha_visc, gas)))?;
            check(c, sys::gvs_set_accelerations(c, p.ax.as_ptr(), p.ay.as_ptr(), p.az.as_ptr()))?;
            if gas {
                check(c, sys::gvs_set_gas(c, p.density.as_ptr(), p.pressure.as_ptr(), p.internal_energy.as_ptr(),
                    p.du_dt.as_ptr(), p.smoothing_length.as_ptr(), p.sound_speed.as_ptr(),
                    p.alpha_visc.as_ptr()))?;
            }
            Ok(())
        })
    }

    /// Downloads positions, velocities, accelerations and (for a gas system) the gas fields.
    pub fn get_state(&self, p: &mut Particles) -> Result<()> {
        let gas = p.has_gas();
        self.with(|c| unsafe {
            check(c, sys::gvs_get_state(c, p.x.as_mut_ptr(), p.y.as_mut_ptr(), p.z.as_mut_ptr(),
                p.vx.as_mut_ptr(), p.vy.as_mut_ptr(), p.vz.as_mut_ptr(), p.ax.as_mut_ptr(), p.ay.as_mut_ptr(),
                p.az.as_mut_ptr()))?;
            if gas {
                check(c, sys::gvs_get_gas(c, p.density.as_mut_ptr(), p.pressure.as_mut_ptr(),
                    p.internal_energy.as_mut_ptr(), p.du_dt.as_mut_ptr(), p.smoothing_length.as_mut_ptr(),
                    p.sound_speed.as_mut_ptr(), p.alpha_visc.as_mut_ptr()))?;
            }
            Ok(())
        })
    }

    /// clear_accelerations + compute_accelerations on the resident state.
    pub fn compute_forces(&self, force: Force, precision: Precision, softening: f64) -> Result<()> {
        self.with(|c| unsafe {
            check(c, sys::gvs_compute_forces(c, force.algo(), precision.raw(), softening, force.theta()))
        })
    }

    /// `nsteps` LeapfrogKDK steps on the resident state (no host copies; direct-sum steps
    /// replay one captured CUDA graph).  Needs valid resident accelerations.
    pub fn kdk_steps(&self, force: Force, precision: Precision, softening: f64, dt: f64, nsteps: i64) -> Result<()> {
        self.with(|c| unsafe {
            check(c, sys::gvs_kdk_steps(c, force.algo(), precision.raw(), softening, force.theta(), dt, nsteps))
        })
    }

    /// Diagnostics::compute of the resident state (diagnostics.rs:37-148).
    pub fn diagnostics(&self, softening: f64, with_potential: bool) -> Result<sys::gvs_diag> {
        let mut d = sys::gvs_diag::default();
        self.with(|c| unsafe { check(c, sys::gvs_diagnostics(c, softening, with_potential as c_int, &mut d)) })?;
        Ok(d)
    }

    /// `PlummerSphere::generate` (plummer_sphere.rs:106-133) on the GPU, into the resident
    /// state: the reference's stream and draws, within a few ulps of the host sampler.
    pub fn plummer_on_device(&self, n: usize, seed: u64, scale_radius: f64, total_mass: f64) -> Result<()> {
        self.with(|c| unsafe { check(c, sys::gvs_ic_plummer_device(c, n, seed, scale_radius, total_mass)) })
    }

    /// Two Plummer spheres from one stream on a head-on orbit (the Barnes-Hut workload's
    /// initial conditions) on the GPU, into the resident state.
    pub fn collision_on_device(&self, n: usize, seed: u64, separation: f64) -> Result<()> {
        self.with(|c| unsafe { check(c, sys::gvs_ic_collision_device(c, n, seed, separation)) })
    }
}

/// `GravitySolver` on the GPU: BruteForce or BarnesHut.
pub struct GpuGravity {
    ctx: Context,
    softening: f64,
    force: Force,
    precision: Precision,
}

impl GpuGravity {
    /// BruteForce::new(softening) on device 0.
    pub fn direct(softening: f64, precision: Precision) -> Result<Self> {
        Ok(Self::on(Context::new(0)?, softening, Force::Direct, precision))
    }

    /// BarnesHut::new(softening, theta) on device 0.
    pub fn barnes_hut(softening: f64, theta: f64, precision: Precision) -> Result<Self> {
        Ok(Self::on(Context::new(0)?, softening, Force::BarnesHut { theta }, precision))
    }

    pub fn on(ctx: Context, softening: f64, force: Force, precision: Precision) -> Self {
        GpuGravity { ctx, softening, force, precision }
    }

    pub fn context(&self) -> &Context {
        &self.ctx
    }

    /// The integrator that runs whole KDK steps with this solver's force on its context.
    pub fn leapfrog(&self) -> GpuLeapfrog {
        GpuLeapfrog { ctx: self.ctx.clone(), softening: self.softening, force: self.force, precision: self.precision }
    }

    /// Adds this solver's accelerations to p.ax..az.
    pub fn try_compute(&self, p: &mut Particles) -> Result<()> {
        self.ctx.with(|c| unsafe {
            let st = match self.force {
                Force::Direct => sys::gvs_gravity_direct(c, p.count, p.x.as_ptr(), p.y.as_ptr(), p.z.as_ptr(),
                    p.mass.as_ptr(), self.softening, self.precision.raw(), p.ax.as_mut_ptr(), p.ay.as_mut_ptr(),
                    p.az.as_mut_ptr()),
                Force::BarnesHut { theta } => sys::gvs_gravity_bh(c, p.count, p.x.as_ptr(), p.y.as_ptr(),
                    p.z.as_ptr(), p.mass.as_ptr(), self.softening, theta, self.precision.raw(), p.ax.as_mut_ptr(),
                    p.ay.as_mut_ptr(), p.az.as_mut_ptr()),
            };
            check(c, st)
        })
    }
}

impl GravitySolver for GpuGravity {
    fn compute_accelerations(&self, particles: &mut Particles) {
        if let Err(e) = self.try_compute(particles) {
            panic!("{e}");
        }
    }
}

/// `Integrator` on the GPU: one call is one LeapfrogKDK step (half-kick, drift, forces,
/// half-kick) through gvs_kdk_step_host, with the force it was built with.  The whole step
/// runs on the GPU, so the `gravity` argument of `step` is not called: build this
/// integrator from the solver the caller would pass ([`GpuGravity::leapfrog`]).
pub struct GpuLeapfrog {
    ctx: Context,
    softening: f64,
    force: Force,
    precision: Precision,
}

impl GpuLeapfrog {
    pub fn try_step(&self, p: &mut Particles, dt: f64) -> Result<()> {
        self.ctx.with(|c| unsafe {
            check(c, sys::gvs_kdk_step_host(c, p.count, p.x.as_mut_ptr(), p.y.as_mut_ptr(), p.z.as_mut_ptr(),
                p.vx.as_mut_ptr(), p.vy.as_mut_ptr(), p.vz.as_mut_ptr(), p.ax.as_mut_ptr(), p.ay.as_mut_ptr(),
                p.az.as_mut_ptr(), p.mass.as_ptr(), self.force.algo(), self.precision.raw(), self.softening,
                self.force.theta(), dt))
        })
    }
}

impl Integrator for GpuLeapfrog {
    fn step(&self, particles: &mut Particles, _gravity: &dyn GravitySolver, dt: f64) {
        if let Err(e) = self.try_step(particles, dt) {
            panic!("{e}");
        }
    }
}

/// SphSolver's surface on the GPU (sph/solver.rs:20-131, step_with_sph 145-212).  The
/// parameters default to SphSolver::new and ForceParams::default.
pub struct GpuSph {
    ctx: Context,
    pub params: sys::gvs_sph_params,
}

impl GpuSph {
    pub fn new(ctx: Context) -> Result<Self> {
        let mut params = sys::gvs_sph_params::default();
        check(std::ptr::null(), unsafe { sys::gvs_sph_params_default(&mut params) })?;
        Ok(GpuSph { ctx, params })
    }

    /// SphSolver::compute: a and du/dt ACCUMULATE into p (call after gravity).
    pub fn compute(&mut self, p: &mut Particles) -> Result<ForceIntermediates> {
        self.ctx.set_state(p)?;
        let n = p.count;
        let (mut div_v, mut max_mu, mut dalpha_dt) = (vec![0.0; n], vec![0.0; n], vec![0.0; n]);
        let params = self.params;
        self.ctx.with(|c| unsafe {
            check(c, sys::gvs_sph_compute(c, &params, std::ptr::null_mut(), div_v.as_mut_ptr(), max_mu.as_mut_ptr(),
                dalpha_dt.as_mut_ptr()))
        })?;
        self.ctx.get_state(p)?;
        Ok(ForceIntermediates { div_v, max_mu, dalpha_dt })
    }

    /// SphSolver::compute_timestep for the state of the last `compute` (the intermediates
    /// of that call are kept on the GPU).
    pub fn compute_timestep(&self, _p: &Particles, _intermediates: &ForceIntermediates) -> Result<f64> {
        let mut dt = 0.0;
        let params = self.params;
        self.ctx.with(|c| unsafe { check(c, sys::gvs_sph_timestep(c, &params, &mut dt)) })?;
        Ok(dt)
    }

    /// step_with_sph with `gravity`'s force on the GPU; returns dt_next.
    pub fn step_with_sph(&mut self, p: &mut Particles, gravity: &GpuGravity, dt: f64) -> Result<f64> {
        self.ctx.set_state(p)?;
        let mut dt_next = 0.0;
        let params = self.params;
        self.ctx.with(|c| unsafe {
            check(c, sys::gvs_sph_step(c, &params, gravity.force.algo(), gravity.precision.raw(), gravity.softening,
                gravity.force.theta(), dt, &mut dt_next))
        })?;
        self.ctx.get_state(p)?;
        Ok(dt_next)
    }
}

/// The headless `--algorithm` names this crate adds: "gpu-direct" and "gpu-bh" (with
/// `--precision fp64-exact|fp64|fp32|mixed`).  None for any other name.
pub fn gravity_for(algorithm: &str, softening: f64, theta: f64, precision: &str)
    -> Option<Result<Box<dyn GravitySolver + Send + Sync>>> {
    let prec = Precision::parse(precision)?;
    let g = match algorithm {
        "gpu-direct" => GpuGravity::direct(softening, prec),
        "gpu-bh" => GpuGravity::barnes_hut(softening, theta, prec),
        _ => return None,
    };
    Some(g.map(|g| Box::new(g) as Box<dyn GravitySolver + Send + Sync>))
}

#[cfg(test)]
mod tests {
    use super::*;
    use sim_core::gravity::BruteForce;
    use sim_core::scenario::Scenario;
    use sim_core::scenarios::plummer_sphere::PlummerSphere;

    /// With the exact f64 form the GPU direct sum returns BruteForce's bits
    /// (needs a GB300; the engine has no CPU fallback).
    #[test]
    fn exact_direct_sum_equals_brute_force() {
        let sc = PlummerSphere { n: 1000, seed: 42, ..Default::default() };
        let mut a = sc.generate();
        let mut b = a.clone();
        let eps = sc.suggested_softening();
        a.clear_accelerations();
        b.clear_accelerations();
        BruteForce::new(eps).compute_accelerations(&mut a);
        GpuGravity::direct(eps, Precision::Fp64Exact).unwrap().compute_accelerations(&mut b);
        assert_eq!(a.ax, b.ax);
        assert_eq!(a.ay, b.ay);
        assert_eq!(a.az, b.az);
    }
}
