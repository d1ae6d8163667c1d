"""Host-side mirror of gravis sim-core's hot-path interfaces, backed by libgvs.so.

Names, argument meanings and accumulate semantics follow sim-core:

  Particles                   crates/sim-core/src/particle.rs:22-227
  GravitySolver / NoGravity   crates/sim-core/src/gravity.rs:6-19
  BruteForce                  crates/sim-core/src/gravity.rs:47-80
  BarnesHut                   crates/sim-core/src/barnes_hut.rs:21-192
  LeapfrogKDK                 crates/sim-core/src/integrator.rs:5-76
  SphSolver / step_with_sph   crates/sim-core/src/sph/solver.rs:20-212
  diagnostics.compute         crates/sim-core/src/diagnostics.rs:37-148
  PlummerSphere, TwoBody,     crates/sim-core/src/scenarios/{plummer_sphere,two_body,
  EvrardCollapse                evrard_collapse}.rs

Every numeric operation runs on the GPU through the C ABI (include/gvs.h);
this module only moves numpy arrays across it.  There is no CPU fallback: if
libgvs.so is missing or no GB300 is visible, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from ._lib import check

GAS = 4
_F64 = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass", "density", "pressure", "internal_energy",
        "du_dt", "smoothing_length", "sound_speed", "alpha_visc")


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data


class Particles:
    """Structure-of-arrays particle store (particle.rs:22-64), f64 numpy arrays."""

    def __init__(self, n: int = 0):
        self.count = int(n)
        for f in _F64:
            setattr(self, f, np.zeros(self.count, dtype=np.float64))
        self.particle_type = np.zeros(self.count, dtype=np.uint8)

    @classmethod
    def from_arrays(cls, x, y, z, vx, vy, vz, mass, **gas) -> "Particles":
        p = cls(len(x))
        p.x[:], p.y[:], p.z[:] = x, y, z
        p.vx[:], p.vy[:], p.vz[:] = vx, vy, vz
        p.mass[:] = mass
        for k, v in gas.items():
            getattr(p, k)[:] = v
        return p

    def add(self, x, y, z, vx, vy, vz, mass, ptype: int = 0) -> int:
        """Particles::add / add_typed (particle.rs:94-132)."""
        i = self.count
        self.count += 1
        for f in _F64:
            setattr(self, f, np.append(getattr(self, f), 0.0))
        self.particle_type = np.append(self.particle_type, np.uint8(ptype))
        self.x[i], self.y[i], self.z[i], self.vx[i], self.vy[i], self.vz[i], self.mass[i] = x, y, z, vx, vy, vz, mass
        return i

    def add_gas(self, x, y, z, vx, vy, vz, mass, internal_energy, smoothing_length) -> int:
        """Particles::add_gas (particle.rs:136-154): alpha starts at 1."""
        i = self.add(x, y, z, vx, vy, vz, mass, GAS)
        self.internal_energy[i] = internal_energy
        self.smoothing_length[i] = smoothing_length
        self.alpha_visc[i] = 1.0
        return i

    def is_gas(self, i: int) -> bool:
        return self.particle_type[i] == GAS

    def has_gas(self) -> bool:
        return bool(np.any(self.particle_type == GAS))

    def total_mass(self) -> float:
        return float(np.sum(self.mass))

    def clear_accelerations(self):
        self.ax[:] = 0.0
        self.ay[:] = 0.0
        self.az[:] = 0.0

    def clear_sph_rates(self):
        self.du_dt[:] = 0.0

    def shift_to_com_frame(self):
        """particle.rs:189-226 (sequential sums, as the reference)."""
        mt = 0.0
        for m in self.mass:
            mt += m
        if mt == 0.0:
            return
        c = [0.0] * 6
        for i in range(self.count):
            m = self.mass[i]
            c[0] += m * self.x[i]; c[1] += m * self.y[i]; c[2] += m * self.z[i]
            c[3] += m * self.vx[i]; c[4] += m * self.vy[i]; c[5] += m * self.vz[i]
        c = [v / mt for v in c]
        self.x -= c[0]; self.y -= c[1]; self.z -= c[2]
        self.vx -= c[3]; self.vy -= c[4]; self.vz -= c[5]

    def copy(self) -> "Particles":
        q = Particles(self.count)
        for f in _F64 + ("particle_type",):
            getattr(q, f)[:] = getattr(self, f)
        return q

    def acc(self) -> np.ndarray:
        return np.stack([self.ax, self.ay, self.az], axis=1)


class Context:
    """One engine context: a CUDA stream on `device` plus device-resident state."""

    def __init__(self, device: int = 0):
        self._lib = L.load()
        h = C.c_void_p()
        st = self._lib.gvs_create(C.byref(h), device)
        if st != L.OK:
            raise L.GvsError(st, L.last_error(None))
        self.h = h.value
        self._adj_run = None  # (softening, dt) of the last adjoint forward run

    def close(self):
        if getattr(self, "h", None):
            self._lib.gvs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st):
        check(st, self.h)

    # ---- state ---------------------------------------------------------------
    def set_state(self, p: Particles):
        gas = p.has_gas()
        self._ck(self._lib.gvs_set_state(
            self.h, p.count, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy), _ptr(p.vz), _ptr(p.mass),
            _ptr(p.particle_type) if gas else None, _ptr(p.internal_energy) if gas else None,
            _ptr(p.smoothing_length) if gas else None, _ptr(p.alpha_visc) if gas else None))

    def set_accelerations(self, p: Particles):
        self._ck(self._lib.gvs_set_accelerations(self.h, _ptr(p.ax), _ptr(p.ay), _ptr(p.az)))

    def get_state(self, p: Particles):
        self._ck(self._lib.gvs_get_state(self.h, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy),
                                         _ptr(p.vz), _ptr(p.ax), _ptr(p.ay), _ptr(p.az)))

    def get_gas(self, p: Particles):
        self._ck(self._lib.gvs_get_gas(self.h, _ptr(p.density), _ptr(p.pressure), _ptr(p.internal_energy),
                                       _ptr(p.du_dt), _ptr(p.smoothing_length), _ptr(p.sound_speed),
                                       _ptr(p.alpha_visc)))

    # ---- device-resident operations -------------------------------------------
    def compute_forces(self, algo: int, precision: int, softening: float, theta: float = 0.5):
        self._ck(self._lib.gvs_compute_forces(self.h, algo, precision, softening, theta))

    def kdk_steps(self, algo: int, precision: int, softening: float, theta: float, dt: float, nsteps: int):
        self._ck(self._lib.gvs_kdk_steps(self.h, algo, precision, softening, theta, dt, nsteps))

    def diagnostics(self, softening: float, with_potential: bool = True) -> "Diagnostics":
        d = L.Diag()
        self._ck(self._lib.gvs_diagnostics(self.h, softening, 1 if with_potential else 0, C.byref(d)))
        return Diagnostics.from_c(d)

    def direct_subset(self, idx, softening: float, precision: int = L.PREC_FP64_EXACT) -> np.ndarray:
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        out = np.zeros((3, len(idx)))
        self._ck(self._lib.gvs_direct_subset(self.h, precision, softening, _ptr(idx), len(idx), _ptr(out[0]),
                                             _ptr(out[1]), _ptr(out[2])))
        return out.T.copy()

    def tree_export(self) -> dict:
        """The octree of the resident positions (depth-first pre-order)."""
        nn = C.c_size_t()
        self._ck(self._lib.gvs_tree_export(self.h, 0, C.byref(nn), None, None, None, None, None, None, None, None))
        k, n = nn.value, self._lib.gvs_count(self.h)
        out = {"level": np.zeros(k, np.uint8), "first": np.zeros(k, np.uint32), "count": np.zeros(k, np.uint32),
               "skip": np.zeros(k, np.uint32), "mass": np.zeros(k), "com": np.zeros((3, k)),
               "order": np.zeros(n, np.uint32), "keys": np.zeros((2, n), np.uint64)}
        self._ck(self._lib.gvs_tree_export(self.h, k, C.byref(nn), *(_ptr(out[f]) for f in
                                                                      ("level", "first", "count", "skip", "mass",
                                                                       "com", "order", "keys"))))
        out["nnodes"] = k
        return out

    def ensemble_setup(self, sizes, softening: float):
        """The resident state holds len(sizes) independent systems back to back."""
        self._ens_sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        self._ck(self._lib.gvs_ensemble_setup(self.h, len(self._ens_sizes), _ptr(self._ens_sizes), softening))

    def ensemble_forces(self):
        self._ck(self._lib.gvs_ensemble_forces(self.h))

    def ensemble_kdk_steps(self, dt: float, nsteps: int, use_graph: bool = True):
        self._ck(self._lib.gvs_ensemble_kdk_steps(self.h, dt, nsteps, 1 if use_graph else 0))

    def ic_plummer_device(self, n: int, seed: int = 42, scale_radius: float = 1.0, total_mass: float = 1.0):
        """PlummerSphere(n, scale_radius, total_mass, seed).generate() on the GPU, into the
        resident state: the host generator's stream and draws, values within a few ulps."""
        self._ck(self._lib.gvs_ic_plummer_device(self.h, n, seed, scale_radius, total_mass))

    def ic_collision_device(self, n: int, seed: int = 7, separation: float = 20.0):
        """collision(n, seed, separation) on the GPU, into the resident state."""
        self._ck(self._lib.gvs_ic_collision_device(self.h, n, seed, separation))

    def adjoint_forward(self, precision: int, softening: float, dt: float, nsteps: int, checkpoint_every: int = 100):
        self._ck(self._lib.gvs_adjoint_forward(self.h, precision, softening, dt, nsteps, checkpoint_every))
        self._adj_run = (softening, dt)

    def adjoint_checkpoint_steps(self) -> list:
        """Step index of every checkpoint of the last forward run: 0, every, ..., nsteps."""
        count = C.c_longlong()
        self._ck(self._lib.gvs_adjoint_checkpoints(self.h, 0, C.byref(count), None))
        steps = np.zeros(count.value, dtype=np.int64)
        self._ck(self._lib.gvs_adjoint_checkpoints(self.h, count.value, C.byref(count), _ptr(steps)))
        return [int(s) for s in steps]

    def adjoint_checkpoint(self, k: int) -> tuple:
        """Checkpoint k's f64 positions and velocities, (n, 3) arrays in caller order."""
        n = self._lib.gvs_count(self.h)
        a = np.zeros((6, n))
        self._ck(self._lib.gvs_adjoint_checkpoint_read(self.h, k, *(_ptr(a[f]) for f in range(6))))
        return a[:3].T.copy(), a[3:].T.copy()

    def adjoint_save_checkpoints(self, directory: str, particles: Particles) -> list:
        """Writes every checkpoint of the last forward run as an NBODY003 snapshot
        (snapshot.rs:40-65), directory/checkpoint_<step>.nbody: time = step * dt, the
        run's softening and dt, the checkpoint's positions and velocities, and the masses,
        particle types and gas fields of `particles` (the state the run started from).
        Returns the paths in step order."""
        import os
        if self._adj_run is None:
            raise L.GvsError(L.ERR_STATE, "adjoint_save_checkpoints needs adjoint_forward")
        softening, dt = self._adj_run
        paths = []
        for k, step in enumerate(self.adjoint_checkpoint_steps()):
            x, v = self.adjoint_checkpoint(k)
            p = particles.copy()
            p.x, p.y, p.z = (np.ascontiguousarray(x[:, d]) for d in range(3))
            p.vx, p.vy, p.vz = (np.ascontiguousarray(v[:, d]) for d in range(3))
            path = os.path.join(directory, f"checkpoint_{step:09d}.nbody")
            with open(path, "wb") as fh:
                Snapshot.capture(p, step * dt, step, softening, dt).write_to(fh)
            paths.append(path)
        return paths

    def adjoint_load_checkpoints(self, paths, precision: int):
        """Reads the NBODY003 checkpoints of one forward run (any order), makes the first
        (step 0) the resident state and fills the backward sweep's checkpoints with them,
        so that adjoint_backward gives the gradients of that run bit for bit."""
        snaps = []
        for path in paths:
            with open(path, "rb") as fh:
                snaps.append(Snapshot.read_from(fh))
        snaps.sort(key=lambda s: s.step)
        nsteps, every = checkpoint_plan([s.step for s in snaps])
        s0 = snaps[0]
        for s in snaps[1:]:
            if (s.softening, s.dt, s.particles.count) != (s0.softening, s0.dt, s0.particles.count) or \
                    not np.array_equal(s.particles.mass, s0.particles.mass):
                raise ValueError(f"adjoint checkpoints: step {s.step} is not from the run of step 0")
        self.set_state(s0.particles)
        self._ck(self._lib.gvs_adjoint_prepare(self.h, precision, s0.softening, s0.dt, nsteps, every))
        self._adj_run = (s0.softening, s0.dt)
        for k, s in enumerate(snaps):
            q = s.particles
            arrs = [np.ascontiguousarray(getattr(q, f), dtype=np.float64) for f in ("x", "y", "z", "vx", "vy", "vz")]
            self._ck(self._lib.gvs_adjoint_checkpoint_write(self.h, k, *(_ptr(a) for a in arrs)))

    def adjoint_backward(self, dl_dx: np.ndarray, dl_dv: np.ndarray | None = None) -> dict:
        """dl_dx, dl_dv: (n, 3) arrays.  Returns dL/dx0, dL/dv0 (n, 3) and dL/dm (n,) through the dynamics."""
        n = self._lib.gvs_count(self.h)
        lx = np.ascontiguousarray(np.asarray(dl_dx, dtype=np.float64).T)
        lv = None if dl_dv is None else np.ascontiguousarray(np.asarray(dl_dv, dtype=np.float64).T)
        gx, gv, gm = np.zeros((3, n)), np.zeros((3, n)), np.zeros(n)
        self._ck(self._lib.gvs_adjoint_backward(
            self.h, _ptr(lx[0]), _ptr(lx[1]), _ptr(lx[2]), *((_ptr(lv[0]), _ptr(lv[1]), _ptr(lv[2])) if lv is not None
                                                            else (None, None, None)),
            _ptr(gx[0]), _ptr(gx[1]), _ptr(gx[2]), _ptr(gv[0]), _ptr(gv[1]), _ptr(gv[2]), _ptr(gm)))
        return {"x": gx.T.copy(), "v": gv.T.copy(), "m": gm}

    def autotune(self, precision: int, softening: float) -> dict:
        nt, ipt, ms = C.c_int(), C.c_int(), C.c_double()
        self._ck(self._lib.gvs_autotune_direct(self.h, precision, softening, C.byref(nt), C.byref(ipt),
                                               C.byref(ms)))
        return {"nthreads": nt.value, "ipt": ipt.value, "ms": ms.value}

    def set_direct_shape(self, nthreads: int, ipt: int, min_blocks: int, unroll: int):
        """Fixes the pair-kernel shape (one of autotune_report's candidates)."""
        self._ck(self._lib.gvs_set_direct_shape(self.h, nthreads, ipt, min_blocks, unroll))

    def set_bh_walk(self, group_size: int, budget: int = 0):
        """FP32 Barnes-Hut walk: 32, 64 or 128 particles per warp group (a refinement of
        each particle's Barnes-Hut sum), -1 for the automatic size (128 from 2^21
        particles, else 64), or 0 for the per-particle walk.  Groups whose walk exceeds
        `budget` iterations (0: 1024) are walked per particle."""
        self._ck(self._lib.gvs_set_bh_walk(self.h, group_size, budget))

    def autotune_report(self) -> list:
        """Every candidate of the last autotune: block size, targets per thread, minimum
        resident blocks per SM and ms per force evaluation."""
        cnt = C.c_int()
        self._ck(self._lib.gvs_autotune_report(self.h, 0, C.byref(cnt), None, None, None, None, None))
        k = cnt.value
        nt, ipt, mb, un = ((C.c_int * max(k, 1))() for _ in range(4))
        ms = (C.c_double * max(k, 1))()
        self._ck(self._lib.gvs_autotune_report(self.h, k, C.byref(cnt), nt, ipt, mb, un, ms))
        return [{"nthreads": nt[i], "ipt": ipt[i], "min_blocks": mb[i], "unroll": un[i], "ms": ms[i]}
                for i in range(k)]

    def sync(self):
        self._ck(self._lib.gvs_sync(self.h))

    def set_fault(self, spec: str):
        self._ck(self._lib.gvs_set_fault(self.h, spec.encode()))

    def device_errors(self) -> int:
        f = C.c_uint()
        self._ck(self._lib.gvs_device_errors(self.h, C.byref(f)))
        return f.value

    # ---- timing -------------------------------------------------------------------
    def profile(self, on: bool):
        self._ck(self._lib.gvs_profile_enable(self.h, 1 if on else 0))

    def profile_read(self) -> dict:
        pr = L.Profile()
        self._ck(self._lib.gvs_profile_read(self.h, C.byref(pr)))
        return {"force_ms": pr.force_ms, "force_launches": pr.force_launches, "launches": pr.launches,
                "force_flops": pr.force_flops, "force_bytes": pr.force_bytes, "tile_visits": pr.tile_visits,
                "near_tile_visits": pr.near_tile_visits, "vjp_ms": pr.vjp_ms, "vjp_launches": pr.vjp_launches,
                "sph_f64_redo": pr.sph_f64_redo, "bh_groups": pr.bh_groups,
                "bh_group_fallbacks": pr.bh_group_fallbacks, "bh_group_iterations": pr.bh_group_iterations,
                "bh_group_interactions": pr.bh_group_interactions, "bh_walk_terms": pr.bh_walk_terms}

    def event(self, slot: int):
        self._ck(self._lib.gvs_event_record(self.h, slot))

    def elapsed(self, a: int, b: int) -> float:
        ms = C.c_float()
        self._ck(self._lib.gvs_event_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value

    def l2_flush(self):
        self._ck(self._lib.gvs_l2_flush(self.h))

    def stream(self) -> int:
        """The context's cudaStream_t (as an integer), for ordering other CUDA work against it."""
        s = C.c_void_p()
        self._ck(self._lib.gvs_stream(self.h, C.byref(s)))
        return s.value or 0

    def fp32_peak_tflops(self) -> float:
        v = C.c_double()
        self._ck(self._lib.gvs_measure_fp32_peak(self.h, C.byref(v)))
        return v.value

    def fp32_peak_variants(self) -> dict:
        """TFLOP/s of the probe's scalar, packed and interleaved forms (after fp32_peak_tflops)."""
        v = [C.c_double() for _ in range(3)]
        self._ck(self._lib.gvs_fp32_peak_variants(self.h, *(C.byref(x) for x in v)))
        return {"scalar": v[0].value, "packed": v[1].value, "mixed": v[2].value}


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---- gravity solvers ------------------------------------------------------------
class GravitySolver:
    """gravity.rs:6-10: compute_accelerations ACCUMULATES into ax/ay/az."""
    algo = L.ALGO_NONE
    softening = 0.0
    theta = 0.5
    precision = L.PREC_FP64_EXACT

    def compute_accelerations(self, p: Particles):
        raise NotImplementedError

    def context(self) -> Context:
        return getattr(self, "ctx", None) or default_context()


class NoGravity(GravitySolver):
    """gravity.rs:13-19."""

    def compute_accelerations(self, p: Particles):
        return None


class BruteForce(GravitySolver):
    """gravity.rs:47-80 on the GPU.  precision=PREC_FP64_EXACT reproduces the
    reference bit for bit; PREC_MIXED is the fast f32-pair path."""
    algo = L.ALGO_DIRECT

    def __init__(self, softening: float, precision: int = L.PREC_FP64_EXACT, ctx: Context | None = None):
        self.softening = float(softening)
        self.precision = precision
        self.ctx = ctx

    def compute_accelerations(self, p: Particles):
        c = self.context()
        c._ck(c._lib.gvs_gravity_direct(c.h, p.count, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.mass),
                                        self.softening, self.precision, _ptr(p.ax), _ptr(p.ay), _ptr(p.az)))


class BarnesHut(GravitySolver):
    """barnes_hut.rs:21-192 on the GPU (octree from sorted octant-path keys)."""
    algo = L.ALGO_BH

    def __init__(self, softening: float, theta: float = 0.5, precision: int = L.PREC_FP64,
                 ctx: Context | None = None):
        self.softening = float(softening)
        self.theta = float(theta)
        self.precision = precision
        self.ctx = ctx

    def compute_accelerations(self, p: Particles):
        c = self.context()
        c._ck(c._lib.gvs_gravity_bh(c.h, p.count, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.mass), self.softening,
                                    self.theta, self.precision, _ptr(p.ax), _ptr(p.ay), _ptr(p.az)))


class LeapfrogKDK:
    """integrator.rs:42-76: one KDK step on the GPU (x, v, a round-trip through the ABI)."""

    def step(self, p: Particles, gravity: GravitySolver, dt: float):
        c = gravity.context()
        c._ck(c._lib.gvs_kdk_step_host(c.h, p.count, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy),
                                       _ptr(p.vz), _ptr(p.ax), _ptr(p.ay), _ptr(p.az), _ptr(p.mass), gravity.algo,
                                       gravity.precision, gravity.softening, gravity.theta, dt))


# ---- SPH ----------------------------------------------------------------------------
@dataclass
class ForceIntermediates:
    """forces.rs:45-52 (plus Omega from density.rs:19-25)."""
    div_v: np.ndarray
    max_mu: np.ndarray
    dalpha_dt: np.ndarray
    omega: np.ndarray


class SphSolver:
    """sph/solver.rs:20-131 on the GPU.  Parameters default to SphSolver::new and
    ForceParams::default; change them through the attributes of `params`."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx
        self.params = L.SphParams()
        check(L.load().gvs_sph_params_default(C.byref(self.params)))
        self._last = None

    def context(self) -> Context:
        return self.ctx or default_context()

    def _upload(self, p: Particles):
        c = self.context()
        c.set_state(p)
        c.set_accelerations(p)
        c._ck(c._lib.gvs_set_gas(c.h, _ptr(p.density), _ptr(p.pressure), _ptr(p.internal_energy), _ptr(p.du_dt),
                                 _ptr(p.smoothing_length), _ptr(p.sound_speed), _ptr(p.alpha_visc)))

    def _download(self, p: Particles):
        c = self.context()
        c._ck(c._lib.gvs_get_state(c.h, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy), _ptr(p.vz),
                                   _ptr(p.ax), _ptr(p.ay), _ptr(p.az)))
        c.get_gas(p)

    def compute(self, p: Particles) -> ForceIntermediates:
        """SphSolver::compute (solver.rs:61-80): a and du/dt accumulate into p."""
        c = self.context()
        self._upload(p)
        out = [np.zeros(p.count) for _ in range(4)]
        c._ck(c._lib.gvs_sph_compute(c.h, C.byref(self.params), *(_ptr(a) for a in out)))
        self._download(p)
        self._last = ForceIntermediates(div_v=out[1], max_mu=out[2], dalpha_dt=out[3], omega=out[0])
        return self._last

    def compute_timestep(self, p: Particles, intermediates: ForceIntermediates | None = None) -> float:
        """SphSolver::compute_timestep (solver.rs:90-131) for the state of the last compute."""
        c = self.context()
        dt = C.c_double()
        c._ck(c._lib.gvs_sph_timestep(c.h, C.byref(self.params), C.byref(dt)))
        return dt.value

    def neighbors(self) -> tuple:
        """NeighborList of the last compute, in caller indices: (start, count, indices)."""
        c = self.context()
        total = C.c_size_t()
        c._ck(c._lib.gvs_sph_neighbors(c.h, 0, C.byref(total), None, None, None))
        n = c._lib.gvs_count(c.h)
        start, count = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        idx = np.zeros(max(1, total.value), np.uint32)
        c._ck(c._lib.gvs_sph_neighbors(c.h, total.value, C.byref(total), _ptr(start), _ptr(count), _ptr(idx)))
        return start, count, idx[: total.value]


def step_with_sph(p: Particles, gravity: GravitySolver, sph: SphSolver, dt: float) -> float:
    """step_with_sph (sph/solver.rs:145-212) on the GPU; returns the next timestep."""
    c = sph.context()
    sph._upload(p)
    dtn = C.c_double()
    c._ck(c._lib.gvs_sph_step(c.h, C.byref(sph.params), gravity.algo, gravity.precision, gravity.softening,
                              gravity.theta, dt, C.byref(dtn)))
    sph._download(p)
    return dtn.value


# ---- diagnostics ------------------------------------------------------------------
@dataclass
class Diagnostics:
    kinetic_energy: float = 0.0
    potential_energy: float = 0.0
    thermal_energy: float = 0.0
    total_energy: float = 0.0
    momentum: np.ndarray = field(default_factory=lambda: np.zeros(3))
    angular_momentum: np.ndarray = field(default_factory=lambda: np.zeros(3))
    center_of_mass: np.ndarray = field(default_factory=lambda: np.zeros(3))
    center_of_mass_velocity: np.ndarray = field(default_factory=lambda: np.zeros(3))
    virial_ratio: float = 0.0
    time: float = 0.0
    step: int = 0

    @classmethod
    def from_c(cls, d: L.Diag) -> "Diagnostics":
        return cls(d.kinetic_energy, d.potential_energy, d.thermal_energy, d.total_energy,
                   np.array(d.momentum[:]), np.array(d.angular_momentum[:]), np.array(d.center_of_mass[:]),
                   np.array(d.center_of_mass_velocity[:]), d.virial_ratio)

    def momentum_magnitude(self) -> float:
        return float(np.sqrt(self.momentum @ self.momentum))

    def angular_momentum_magnitude(self) -> float:
        return float(np.sqrt(self.angular_momentum @ self.angular_momentum))

    def com_drift(self) -> float:
        return float(np.sqrt(self.center_of_mass @ self.center_of_mass))

    @staticmethod
    def csv_header() -> str:
        """diagnostics.rs:170-172."""
        return ("step,time,kinetic_energy,potential_energy,thermal_energy,total_energy,momentum_mag,"
                "angular_momentum_mag,com_drift,virial_ratio")

    def to_csv_row(self) -> str:
        """diagnostics.rs:175-189 ({:.6e} / {:.10e} in Rust's exponent style)."""
        def e(v, prec):
            s = f"{v:.{prec}e}"
            mant, ex = s.split("e")
            return f"{mant}e{int(ex)}"
        vals = [e(self.kinetic_energy, 10), e(self.potential_energy, 10), e(self.thermal_energy, 10),
                e(self.total_energy, 10), e(self.momentum_magnitude(), 10), e(self.angular_momentum_magnitude(), 10),
                e(self.com_drift(), 10)]
        return f"{self.step},{e(self.time, 6)}," + ",".join(vals) + f",{self.virial_ratio:.6f}"


def compute_diagnostics(p: Particles, softening: float, time: float = 0.0, step: int = 0,
                        ctx: Context | None = None, with_potential: bool = True) -> Diagnostics:
    """diagnostics::compute (diagnostics.rs:37-39) on the GPU for a host Particles."""
    c = ctx or default_context()
    c.set_state(p)
    d = c.diagnostics(softening, with_potential)
    d.time, d.step = time, step
    return d


def checkpoint_plan(steps) -> tuple:
    """(nsteps, every) of the forward run whose checkpoints sit at `steps` (sorted):
    0, every, 2 every, ..., and nsteps, the last one.  Raises ValueError for any other set."""
    steps = [int(s) for s in steps]
    if len(steps) < 2 or steps[0] != 0:
        raise ValueError("adjoint checkpoints: need step 0 and at least one later step")
    nsteps, every = steps[-1], steps[1]
    if every < 1 or steps != list(range(0, nsteps, every)) + [nsteps]:
        raise ValueError(f"adjoint checkpoints: steps {steps} are not 0, {every}, ..., {nsteps}")
    return nsteps, every


# ---- snapshots ----------------------------------------------------------------------
_MAGIC = {b"NBODY001": 1, b"NBODY002": 2, b"NBODY003": 3}


@dataclass
class Snapshot:
    """snapshot.rs:1-170: the NBODY003 binary format (little-endian): magic, time, step,
    softening, dt, count, x y z vx vy vz mass (f64), particle_type (u8), then
    internal_energy, smoothing_length, density (f64).  NBODY001/002 are read too.
    Accelerations are not stored: initialize() recomputes them."""
    time: float
    step: int
    softening: float
    dt: float
    particles: Particles

    @classmethod
    def capture(cls, p: Particles, time: float, step: int, softening: float, dt: float) -> "Snapshot":
        return cls(time, step, softening, dt, p.copy())

    def write_to(self, fh):
        p = self.particles
        fh.write(b"NBODY003")
        fh.write(np.array([self.time], "<f8").tobytes() + np.array([self.step], "<u8").tobytes())
        fh.write(np.array([self.softening, self.dt], "<f8").tobytes() + np.array([p.count], "<u8").tobytes())
        for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
            fh.write(np.asarray(getattr(p, f), "<f8").tobytes())
        fh.write(np.asarray(p.particle_type, np.uint8).tobytes())
        for f in ("internal_energy", "smoothing_length", "density"):
            fh.write(np.asarray(getattr(p, f), "<f8").tobytes())

    @classmethod
    def read_from(cls, fh) -> "Snapshot":
        magic = fh.read(8)
        if magic not in _MAGIC:
            raise ValueError("Invalid snapshot magic bytes")
        ver = _MAGIC[magic]
        time, = np.frombuffer(fh.read(8), "<f8")
        step, = np.frombuffer(fh.read(8), "<u8")
        softening, dt = np.frombuffer(fh.read(16), "<f8")
        n, = np.frombuffer(fh.read(8), "<u8")
        n = int(n)
        p = Particles(n)

        def vec(dtype, size):
            b = fh.read(size * np.dtype(dtype).itemsize)
            if len(b) != size * np.dtype(dtype).itemsize:
                raise ValueError("snapshot: truncated")
            return np.frombuffer(b, dtype).copy()

        for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
            setattr(p, f, vec("<f8", n))
        if ver >= 2:
            p.particle_type = vec(np.uint8, n)
        if ver >= 3:
            for f in ("internal_energy", "smoothing_length", "density"):
                setattr(p, f, vec("<f8", n))
        return cls(float(time), int(step), float(softening), float(dt), p)

    def initialize(self, gravity: "GravitySolver"):
        """Snapshot::initialize (snapshot.rs:152-158): recompute a before stepping."""
        self.particles.clear_accelerations()
        gravity.compute_accelerations(self.particles)


# ---- scenarios ----------------------------------------------------------------------
class PlummerSphere:
    """scenarios/plummer_sphere.rs:79-153."""

    def __init__(self, n: int = 1000, scale_radius: float = 1.0, total_mass: float = 1.0, seed: int = 42):
        self.n, self.scale_radius, self.total_mass, self.seed = n, scale_radius, total_mass, seed

    def name(self) -> str:
        return "Plummer Sphere"

    def generate(self) -> Particles:
        p = Particles(self.n)
        check(L.load().gvs_ic_plummer(self.n, self.seed, self.scale_radius, self.total_mass, _ptr(p.x), _ptr(p.y),
                                      _ptr(p.z), _ptr(p.vx), _ptr(p.vy), _ptr(p.vz), _ptr(p.mass)))
        return p

    def suggested_dt(self) -> float:
        return math.sqrt(self.scale_radius ** 3 / (1.0 * self.total_mass)) / 100.0

    def suggested_softening(self) -> float:
        r_h = 1.305 * self.scale_radius
        return (4.0 / 3.0 * math.pi * (r_h * r_h * r_h) / self.n) ** (1.0 / 3.0) * 0.5


class TwoBody:
    """scenarios/two_body.rs:17-106."""

    def __init__(self, mass_ratio: float = 0.5, eccentricity: float = 0.5, semi_major_axis: float = 1.0):
        self.mass_ratio, self.eccentricity, self.semi_major_axis = mass_ratio, eccentricity, semi_major_axis

    def period(self) -> float:
        return 2.0 * math.pi * math.sqrt(self.semi_major_axis ** 3 / 1.0)

    def generate(self) -> Particles:
        p = Particles(2)
        check(L.load().gvs_ic_two_body(self.mass_ratio, self.eccentricity, self.semi_major_axis, _ptr(p.x),
                                       _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy), _ptr(p.vz), _ptr(p.mass)))
        return p

    def suggested_dt(self) -> float:
        return self.period() / 10000.0

    def suggested_softening(self) -> float:
        return self.semi_major_axis * (1.0 - self.eccentricity) * 0.001


class EvrardCollapse:
    """scenarios/evrard_collapse.rs:15-71 (uniform gas sphere)."""

    def __init__(self, n_particles: int = 5000, total_mass: float = 1.0, radius: float = 1.0, u_0: float = 0.05,
                 seed: int = 42):
        self.n, self.total_mass, self.radius, self.u_0, self.seed = n_particles, total_mass, radius, u_0, seed

    def generate(self) -> Particles:
        p = Particles(self.n)
        check(L.load().gvs_ic_evrard(self.n, self.seed, self.total_mass, self.radius, self.u_0, _ptr(p.x),
                                     _ptr(p.y), _ptr(p.z), _ptr(p.mass), _ptr(p.internal_energy),
                                     _ptr(p.smoothing_length)))
        p.particle_type[:] = GAS
        p.alpha_visc[:] = 1.0
        return p

    def suggested_softening(self) -> float:
        vol = 4.0 / 3.0 * math.pi * self.radius ** 3
        return 0.3 * (vol / self.n) ** (1.0 / 3.0)

    def suggested_dt(self) -> float:
        return math.pi / 2 * math.sqrt(self.radius ** 3 / (2.0 * self.total_mass)) / 500.0


class ColdCollapse:
    """scenarios/cold_collapse.rs:26-123: particles at rest, uniform in a sphere (gas if sph)."""

    def __init__(self, n: int = 5000, radius: float = 1.0, total_mass: float = 1.0, seed: int = 42,
                 sph: bool = False):
        self.n, self.radius, self.total_mass, self.seed, self.sph = n, radius, total_mass, seed, sph

    def name(self) -> str:
        return "Cold Collapse (Gas)" if self.sph else "Cold Collapse"

    def generate(self) -> Particles:
        p = Particles(self.n)
        check(L.load().gvs_ic_cold_collapse(self.n, self.seed, self.radius, self.total_mass, 1 if self.sph else 0,
                                            _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy), _ptr(p.vz),
                                            _ptr(p.mass), _ptr(p.internal_energy), _ptr(p.smoothing_length)))
        if self.sph:
            p.particle_type[:] = GAS
            p.alpha_visc[:] = 1.0
        return p

    def suggested_dt(self) -> float:
        """Free-fall time pi/2 sqrt(R^3 / (2 G M)) over 200 (gas: 500)."""
        t_ff = (math.pi / 2) * math.sqrt((self.radius * self.radius * self.radius) / (2.0 * 1.0 * self.total_mass))
        return t_ff / 500.0 if self.sph else t_ff / 200.0

    def suggested_softening(self) -> float:
        """0.3 x the mean spacing (4/3 pi R^3 / n)^(1/3)."""
        r3 = self.radius * self.radius * self.radius
        return (4.0 / 3.0 * math.pi * r3 / self.n) ** (1.0 / 3.0) * 0.3


def collision(n: int, seed: int = 7, separation: float = 20.0) -> Particles:
    """Two Plummer spheres on a parabolic head-on orbit (see gvs_ic_collision)."""
    p = Particles(n)
    check(L.load().gvs_ic_collision(n, seed, separation, _ptr(p.x), _ptr(p.y), _ptr(p.z), _ptr(p.vx), _ptr(p.vy),
                                    _ptr(p.vz), _ptr(p.mass)))
    return p


def gas_sphere_1r(n: int, total_mass: float = 1.0, radius: float = 1.0, u0: float = 0.05,
                  eta: float = 1.2) -> Particles:
    """Seedless rho ~ 1/r gas sphere (see gvs_ic_gas_sphere_1r)."""
    p = Particles(n)
    check(L.load().gvs_ic_gas_sphere_1r(n, total_mass, radius, u0, eta, _ptr(p.x), _ptr(p.y), _ptr(p.z),
                                        _ptr(p.mass), _ptr(p.internal_energy), _ptr(p.smoothing_length)))
    p.particle_type[:] = GAS
    p.alpha_visc[:] = 1.0
    return p


def ensemble_sizes(count: int, seed: int, lo: float = 256, hi: float = 16384) -> np.ndarray:
    out = np.zeros(count, dtype=np.int64)
    check(L.load().gvs_ic_ensemble_sizes(count, seed, lo, hi, _ptr(out)))
    return out


def plummer_ensemble(sizes, seed0: int = 1000) -> Particles:
    """Plummer spheres with N = sizes[i] and seed seed0 + i, concatenated (each in its own COM frame)."""
    parts = [PlummerSphere(int(n), seed=seed0 + i).generate() for i, n in enumerate(sizes)]
    p = Particles(int(np.sum(sizes)))
    o = 0
    for q in parts:
        for f in _F64 + ("particle_type",):
            getattr(p, f)[o:o + q.count] = getattr(q, f)
        o += q.count
    return p
