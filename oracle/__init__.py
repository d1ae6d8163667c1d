"""ctypes binding to liboracle.so, the CPU restatement of gravis sim-core.

TEST INFRASTRUCTURE ONLY.  The GPU engine (package ``gravis_gb300``) never
imports this module; only the tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use it, and only as the checker.

Parity status: pinned against the reference's committed diagnostics and
Barnes-Hut accuracy files (tests/test_oracle_pins.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

GAS = 4
GRAV_NONE, GRAV_BF, GRAV_BF_GATHER, GRAV_BH = 0, 1, 2, 3

_F64_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass")
_GAS_FIELDS = ("density", "pressure", "u", "du_dt", "h", "cs", "alpha")


class _CParticles(C.Structure):
    _fields_ = ([("n", C.c_int64)] + [(f, C.POINTER(C.c_double)) for f in _F64_FIELDS]
                + [("ptype", C.POINTER(C.c_uint8))]
                + [(f, C.POINTER(C.c_double)) for f in _GAS_FIELDS])


class _CGravity(C.Structure):
    _fields_ = [("kind", C.c_int), ("softening", C.c_double), ("theta", C.c_double), ("nthreads", C.c_int)]


class _CDiag(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("potential", C.c_double), ("thermal", C.c_double),
                ("total", C.c_double), ("momentum", C.c_double * 3), ("angular_momentum", C.c_double * 3),
                ("com", C.c_double * 3), ("com_vel", C.c_double * 3), ("virial", C.c_double)]


class _CSph(C.Structure):
    _fields_ = [("gamma", C.c_double), ("eta", C.c_double), ("cfl_factor", C.c_double),
                ("force_factor", C.c_double), ("h_max", C.c_double), ("beta_visc", C.c_double),
                ("alpha_min", C.c_double), ("alpha_max", C.c_double), ("alpha_cond", C.c_double),
                ("sigma_visc", C.c_double), ("nthreads", C.c_int),
                ("tree_nodes", C.c_void_p), ("tree_count", C.c_int64), ("tree_cap", C.c_int64),
                ("n", C.c_int64), ("nl_idx", C.POINTER(C.c_uint32)), ("nl_len", C.c_int64),
                ("nl_cap", C.c_int64), ("nl_start", C.POINTER(C.c_uint32)), ("nl_end", C.POINTER(C.c_uint32)),
                ("omega", C.POINTER(C.c_double)), ("div_v", C.POINTER(C.c_double)),
                ("max_mu", C.POINTER(C.c_double)), ("dalpha_dt", C.POINTER(C.c_double))]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    src = os.path.join(_HERE, "gvs_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        P = C.POINTER(_CParticles)
        G = C.POINTER(_CGravity)
        d, i64, u64, i32 = C.c_double, C.c_int64, C.c_uint64, C.c_int
        sig = {
            "orc_plummer_generate": (None, [P, i64, d, d, u64]),
            "orc_plummer_suggested_dt": (d, [d, d]),
            "orc_plummer_suggested_softening": (d, [i64, d]),
            "orc_two_body_generate": (None, [P, d, d, d]),
            "orc_two_body_period": (d, [d]),
            "orc_two_body_suggested_softening": (d, [d, d]),
            "orc_evrard_generate": (None, [P, i64, d, d, d, u64]),
            "orc_evrard_suggested_softening": (d, [i64, d]),
            "orc_cold_collapse_generate": (None, [P, i64, d, d, u64, C.c_int]),
            "orc_cold_collapse_suggested_dt": (d, [d, d, C.c_int]),
            "orc_cold_collapse_suggested_softening": (d, [i64, d]),
            "orc_shift_to_com_frame": (None, [P]),
            "orc_bf_serial": (None, [P, d]),
            "orc_bf_gather": (None, [P, d, i32]),
            "orc_bf_gather_subset": (None, [P, d, C.c_void_p, i64, C.c_void_p, C.c_void_p, C.c_void_p, i32]),
            "orc_bh": (None, [P, d, d, i32]),
            "orc_bh_subset": (None, [P, d, d, C.c_void_p, i64, C.c_void_p, C.c_void_p, C.c_void_p, i32]),
            "orc_gravity_apply": (None, [G, P]),
            "orc_kdk_step": (None, [P, G, d]),
            "orc_kdk_steps": (None, [P, G, d, i64]),
            "orc_diagnostics": (None, [P, d, i32, C.POINTER(_CDiag)]),
            "orc_octant": (i32, [C.POINTER(C.c_double), d, d, d]),
            "orc_bbox_containing": (None, [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "orc_sph_w": (d, [d, d]),
            "orc_sph_grad_w": (None, [d, d, d, d, d, C.POINTER(C.c_double)]),
            "orc_sph_dw_dh": (d, [d, d]),
            "orc_sph_abs_grad_w": (d, [d, d]),
            "orc_sph_new": (C.POINTER(_CSph), [i32]),
            "orc_sph_free": (None, [C.POINTER(_CSph)]),
            "orc_sph_neighbors_only": (None, [C.POINTER(_CSph), P, d]),
            "orc_sph_density": (None, [C.POINTER(_CSph), P]),
            "orc_sph_forces": (None, [C.POINTER(_CSph), P]),
            "orc_sph_compute": (None, [C.POINTER(_CSph), P]),
            "orc_sph_timestep": (d, [C.POINTER(_CSph), P]),
            "orc_sph_step": (d, [P, G, C.POINTER(_CSph), d]),
            "orc_max_threads": (i32, []),
            "orc_octree_build_leaves": (i64, [P, C.POINTER(i64), C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, i64]),
            "orc_rng_seed_u64": (None, [C.c_void_p, u64]),
            "orc_rng_next_u64": (u64, [C.c_void_p]),
            "orc_rng_f64": (d, [C.c_void_p]),
            "orc_rng_range": (d, [C.c_void_p, d, d]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class Particles:
    """numpy SoA mirror of particle.rs:22-64, shareable with the C oracle."""

    def __init__(self, n: int):
        self.n = int(n)
        for f in _F64_FIELDS + _GAS_FIELDS:
            setattr(self, f, np.zeros(self.n, dtype=np.float64))
        self.ptype = np.zeros(self.n, dtype=np.uint8)
        self._c = None

    def c(self):
        cp = _CParticles()
        cp.n = self.n
        for f in _F64_FIELDS + _GAS_FIELDS:
            a = getattr(self, f)
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == (self.n,)
            setattr(cp, f, a.ctypes.data_as(C.POINTER(C.c_double)))
        cp.ptype = self.ptype.ctypes.data_as(C.POINTER(C.c_uint8))
        self._c = cp
        return C.byref(cp)

    def copy(self) -> "Particles":
        q = Particles(self.n)
        for f in _F64_FIELDS + _GAS_FIELDS + ("ptype",):
            getattr(q, f)[:] = getattr(self, f)
        return q

    def subset(self, idx) -> "Particles":
        idx = np.asarray(idx)
        q = Particles(len(idx))
        for f in _F64_FIELDS + _GAS_FIELDS + ("ptype",):
            getattr(q, f)[:] = getattr(self, f)[idx]
        return q

    def clear_accelerations(self):
        self.ax[:] = 0.0
        self.ay[:] = 0.0
        self.az[:] = 0.0

    def acc(self) -> np.ndarray:
        return np.stack([self.ax, self.ay, self.az], axis=1)


# ---- scenarios ---------------------------------------------------------------
def plummer(n: int, seed: int = 42, scale_radius: float = 1.0, total_mass: float = 1.0) -> Particles:
    p = Particles(n)
    lib().orc_plummer_generate(p.c(), n, scale_radius, total_mass, seed)
    return p


def plummer_suggested_softening(n: int, scale_radius: float = 1.0) -> float:
    return lib().orc_plummer_suggested_softening(n, scale_radius)


def plummer_suggested_dt(scale_radius: float = 1.0, total_mass: float = 1.0) -> float:
    return lib().orc_plummer_suggested_dt(scale_radius, total_mass)


def two_body(mass_ratio: float = 0.5, e: float = 0.5, a: float = 1.0) -> Particles:
    p = Particles(2)
    lib().orc_two_body_generate(p.c(), mass_ratio, e, a)
    return p


def evrard(n: int, seed: int = 42, total_mass: float = 1.0, radius: float = 1.0, u0: float = 0.05) -> Particles:
    p = Particles(n)
    lib().orc_evrard_generate(p.c(), n, total_mass, radius, u0, seed)
    return p


def cold_collapse(n: int, seed: int = 42, radius: float = 1.0, total_mass: float = 1.0, sph: bool = False) -> Particles:
    p = Particles(n)
    lib().orc_cold_collapse_generate(p.c(), n, radius, total_mass, seed, 1 if sph else 0)
    return p


def cold_collapse_suggested_dt(radius: float = 1.0, total_mass: float = 1.0, sph: bool = False) -> float:
    return lib().orc_cold_collapse_suggested_dt(radius, total_mass, 1 if sph else 0)


def cold_collapse_suggested_softening(n: int, radius: float = 1.0) -> float:
    return lib().orc_cold_collapse_suggested_softening(n, radius)


# ---- solvers -----------------------------------------------------------------
def gravity(kind: int, softening: float, theta: float = 0.5, nthreads: int = 0) -> _CGravity:
    g = _CGravity()
    g.kind, g.softening, g.theta, g.nthreads = kind, softening, theta, nthreads
    return g


def bf_serial(p: Particles, softening: float):
    lib().orc_bf_serial(p.c(), softening)


def bf_gather(p: Particles, softening: float, nthreads: int = 0):
    lib().orc_bf_gather(p.c(), softening, nthreads)


def bf_subset(p: Particles, softening: float, idx, nthreads: int = 0) -> np.ndarray:
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.zeros((3, len(idx)), dtype=np.float64)
    lib().orc_bf_gather_subset(p.c(), softening, idx.ctypes.data, len(idx), out[0].ctypes.data,
                               out[1].ctypes.data, out[2].ctypes.data, nthreads)
    return out.T.copy()


def bh(p: Particles, softening: float, theta: float, nthreads: int = 0):
    lib().orc_bh(p.c(), softening, theta, nthreads)


def bh_subset(p: Particles, softening: float, theta: float, idx, nthreads: int = 0) -> np.ndarray:
    """BarnesHut accelerations of the targets idx (the reference tree of all of p)."""
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.zeros((3, len(idx)), dtype=np.float64)
    lib().orc_bh_subset(p.c(), softening, theta, idx.ctypes.data, len(idx), out[0].ctypes.data,
                        out[1].ctypes.data, out[2].ctypes.data, nthreads)
    return out.T.copy()


def kdk_step(p: Particles, g: _CGravity, dt: float):
    lib().orc_kdk_step(p.c(), C.byref(g), dt)


def kdk_steps(p: Particles, g: _CGravity, dt: float, nsteps: int):
    lib().orc_kdk_steps(p.c(), C.byref(g), dt, nsteps)


def diagnostics(p: Particles, softening: float, compute_potential: bool = True) -> dict:
    d = _CDiag()
    lib().orc_diagnostics(p.c(), softening, 1 if compute_potential else 0, C.byref(d))
    mom = np.array(d.momentum[:])
    am = np.array(d.angular_momentum[:])
    com = np.array(d.com[:])
    return {"kinetic_energy": d.kinetic, "potential_energy": d.potential, "thermal_energy": d.thermal,
            "total_energy": d.total, "momentum": mom, "angular_momentum": am, "com": com,
            "com_velocity": np.array(d.com_vel[:]), "virial_ratio": d.virial,
            "momentum_mag": float(np.sqrt(mom @ mom)), "angular_momentum_mag": float(np.sqrt(am @ am)),
            "com_drift": float(np.sqrt(com @ com))}


def octant(center, x, y, z) -> int:
    c = (C.c_double * 3)(*center)
    return lib().orc_octant(c, x, y, z)


def octree_leaves(p: Particles) -> dict:
    """Reference octree of p: node count and leaves in DFS pre-order (children 0..7)
    with their depth and octant path (126-bit, left-aligned, truncated at the leaf)."""
    nn = C.c_int64()
    cap = p.n
    pidx = np.zeros(cap, np.uint32)
    depth = np.zeros(cap, np.int32)
    hi = np.zeros(cap, np.uint64)
    lo = np.zeros(cap, np.uint64)
    nl = lib().orc_octree_build_leaves(p.c(), C.byref(nn), pidx.ctypes.data, depth.ctypes.data, hi.ctypes.data,
                                       lo.ctypes.data, cap)
    return {"nnodes": nn.value, "nleaves": nl, "order": pidx[:nl], "depth": depth[:nl], "path_hi": hi[:nl],
            "path_lo": lo[:nl]}


def bbox_containing(p: Particles):
    c = (C.c_double * 3)()
    hw = C.c_double()
    lib().orc_bbox_containing(p.c(), c, C.byref(hw))
    return np.array(c[:]), hw.value


class Sph:
    """Handle on an orc_sph solver (SphSolver::new defaults, solver.rs:40-49)."""

    def __init__(self, nthreads: int = 0):
        self._s = lib().orc_sph_new(nthreads)

    def __del__(self):
        if getattr(self, "_s", None):
            lib().orc_sph_free(self._s)
            self._s = None

    @property
    def params(self):
        return self._s.contents

    def neighbors_only(self, p: Particles, factor: float):
        lib().orc_sph_neighbors_only(self._s, p.c(), factor)

    def density(self, p: Particles):
        lib().orc_sph_density(self._s, p.c())

    def compute(self, p: Particles):
        lib().orc_sph_compute(self._s, p.c())

    def timestep(self, p: Particles) -> float:
        return lib().orc_sph_timestep(self._s, p.c())

    def step(self, p: Particles, g: _CGravity, dt: float) -> float:
        return lib().orc_sph_step(p.c(), C.byref(g), self._s, dt)

    def neighbors(self, i: int) -> np.ndarray:
        s = self._s.contents
        a, b = s.nl_start[i], s.nl_end[i]
        return np.array([s.nl_idx[k] for k in range(a, b)], dtype=np.uint32)

    def neighbor_lists(self, n: int):
        s = self._s.contents
        start = np.ctypeslib.as_array(s.nl_start, shape=(n,)).copy()
        end = np.ctypeslib.as_array(s.nl_end, shape=(n,)).copy()
        idx = np.ctypeslib.as_array(s.nl_idx, shape=(max(s.nl_len, 1),))[: s.nl_len].copy() \
            if s.nl_len else np.zeros(0, np.uint32)
        return start, end, idx

    def array(self, name: str, n: int) -> np.ndarray:
        return np.ctypeslib.as_array(getattr(self._s.contents, name), shape=(n,)).copy()


class Rng:
    """ChaCha20Rng::seed_from_u64 + rand 0.9 sampling (for known-answer tests)."""

    def __init__(self, seed: int):
        self._buf = C.create_string_buffer(128)
        lib().orc_rng_seed_u64(self._buf, seed)

    def next_u64(self) -> int:
        return lib().orc_rng_next_u64(self._buf)

    def f64(self) -> float:
        return lib().orc_rng_f64(self._buf)

    def range(self, lo: float, hi: float) -> float:
        return lib().orc_rng_range(self._buf, lo, hi)
