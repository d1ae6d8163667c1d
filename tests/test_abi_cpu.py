"""CPU-only checks of the C ABI: the library loads, exports every symbol the
header declares, validates arguments without a device, and its host-side
initial-condition generators reproduce the oracle's arrays exactly."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from gravis_gb300 import _lib as L
import gravis_gb300 as G


@pytest.fixture(scope="module")
def lib():
    from gravis_gb300 import build
    build.build()
    return L.load()


def test_exports_every_declared_symbol(lib):
    syms = L.header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # and the binding knows every one of them
    assert not [s for s in syms if s not in L.SIGNATURES], [s for s in syms if s not in L.SIGNATURES]


def test_version(lib):
    assert b"sm_103a" in lib.gvs_version()


def test_null_context_is_invalid_arg(lib):
    assert lib.gvs_sync(None) == L.ERR_INVALID_ARG
    assert lib.gvs_compute_forces(None, 1, 3, 0.01, 0.5) == L.ERR_INVALID_ARG
    d = L.Diag()
    assert lib.gvs_diagnostics(None, 0.01, 1, C.byref(d)) == L.ERR_INVALID_ARG
    assert lib.gvs_create(None, 0) == L.ERR_INVALID_ARG
    assert lib.gvs_set_bh_walk(None, 64, 0) == L.ERR_INVALID_ARG
    assert lib.gvs_set_direct_shape(None, 256, 4, 2, 2) == L.ERR_INVALID_ARG
    n = C.c_longlong()
    assert lib.gvs_adjoint_checkpoints(None, 0, C.byref(n), None) == L.ERR_INVALID_ARG
    assert lib.gvs_adjoint_prepare(None, 3, 0.01, 1e-3, 10, 5) == L.ERR_INVALID_ARG
    assert lib.gvs_adjoint_checkpoint_read(None, 0, *([None] * 6)) == L.ERR_INVALID_ARG
    assert lib.gvs_adjoint_checkpoint_write(None, 0, *([None] * 6)) == L.ERR_INVALID_ARG
    assert lib.gvs_ic_plummer_device(None, 10, 1, 1.0, 1.0) == L.ERR_INVALID_ARG


def test_ic_args_validated(lib):
    x = np.zeros(4)
    assert lib.gvs_ic_plummer(0, 1, 1.0, 1.0, *(x.ctypes.data,) * 7) == L.ERR_INVALID_ARG
    assert lib.gvs_ic_plummer(4, 1, -1.0, 1.0, *(x.ctypes.data,) * 7) == L.ERR_INVALID_ARG
    assert lib.gvs_ic_two_body(0.5, 1.0, 1.0, *(x.ctypes.data,) * 7) == L.ERR_INVALID_ARG


@pytest.mark.parametrize("n,seed", [(1, 3), (2, 42), (1000, 42), (4097, 1)])
def test_plummer_ics_match_oracle(lib, n, seed):
    p = G.PlummerSphere(n, seed=seed).generate()
    q = O.plummer(n, seed)
    for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
        assert np.array_equal(getattr(p, f), getattr(q, f)), f


def test_two_body_and_evrard_ics_match_oracle(lib):
    p = G.TwoBody(0.5, 0.5, 1.0).generate()
    q = O.two_body(0.5, 0.5, 1.0)
    assert np.array_equal(p.x, q.x) and np.array_equal(p.vy, q.vy) and np.array_equal(p.mass, q.mass)
    e = G.EvrardCollapse(777, seed=9).generate()
    f = O.evrard(777, 9)
    assert np.array_equal(e.x, f.x) and np.array_equal(e.z, f.z)
    assert np.array_equal(e.smoothing_length, f.h) and np.array_equal(e.internal_energy, f.u)


@pytest.mark.parametrize("n,seed,sph", [(1, 5, False), (1000, 42, False), (777, 9, True), (5000, 42, True)])
def test_cold_collapse_ics_match_oracle(lib, n, seed, sph):
    """ColdCollapse (cold_collapse.rs:60-123): the library's arrays and suggested values equal
    the oracle's restatement, for the gravity-only and the gas variant."""
    s = G.ColdCollapse(n, radius=1.5, total_mass=2.0, seed=seed, sph=sph)
    p = s.generate()
    q = O.cold_collapse(n, seed, 1.5, 2.0, sph)
    for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
        assert np.array_equal(getattr(p, f), getattr(q, f)), f
    if sph:
        assert np.array_equal(p.smoothing_length, q.h) and np.array_equal(p.internal_energy, q.u)
        assert (p.particle_type == G.engine.GAS).all()
    assert not (p.vx.any() or p.vy.any() or p.vz.any())  # at rest; the COM velocity removed is zero
    assert s.suggested_dt() == O.cold_collapse_suggested_dt(1.5, 2.0, sph)
    assert s.suggested_softening() == O.cold_collapse_suggested_softening(n, 1.5)
    # uniform sphere of radius 1.5 about the centre of mass
    r = np.sqrt(p.x ** 2 + p.y ** 2 + p.z ** 2)
    assert r.max() <= 2 * 1.5
    assert s.name() == ("Cold Collapse (Gas)" if sph else "Cold Collapse")


def test_cold_collapse_args_validated(lib):
    x = np.zeros(4)
    assert lib.gvs_ic_cold_collapse(4, 1, 1.0, 1.0, 1, *(x.ctypes.data,) * 7, None, None) == L.ERR_INVALID_ARG
    assert lib.gvs_ic_cold_collapse(4, 1, -1.0, 1.0, 0, *(x.ctypes.data,) * 9) == L.ERR_INVALID_ARG
    assert lib.gvs_ic_cold_collapse(4, 1, 1.0, 1.0, 0, *(x.ctypes.data,) * 7, None, None) == L.OK


def test_collision_and_gas_sphere_ics(lib):
    p = G.collision(1000, seed=7)
    assert abs(p.total_mass() - 1.0) < 1e-12
    m = p.mass
    assert abs((m * p.x).sum()) < 1e-12 and abs((m * p.vx).sum()) < 1e-12
    # the two halves start ~20 apart and approach each other
    assert p.x[:500].mean() < -5 and p.x[500:].mean() > 5
    assert p.vx[:500].mean() > 0 > p.vx[500:].mean()
    g = G.gas_sphere_1r(4000)
    r = np.sqrt(g.x ** 2 + g.y ** 2 + g.z ** 2)
    assert r.max() <= 1.0 + 1e-12
    # M(<r) ~ r^2: half the particles inside r = 1/sqrt(2)
    assert abs(np.mean(r < 2 ** -0.5) - 0.5) < 0.02
    assert np.all(g.particle_type == G.engine.GAS)


def test_ensemble_sizes(lib):
    s = G.ensemble_sizes(512, seed=2024)
    assert s.min() >= 256 and s.max() <= 16384 and len(set(s.tolist())) > 300


def test_no_device_reported(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    h = C.c_void_p()
    assert lib.gvs_create(C.byref(h), 0) == L.ERR_NO_DEVICE
    with pytest.raises(G.GvsError):
        G.Context(0)


def test_adjoint_checkpoint_plan():
    """The checkpoint steps a forward run leaves (0, every, ..., nsteps) and the sets a
    restart refuses."""
    from gravis_gb300.engine import checkpoint_plan
    assert checkpoint_plan([0, 100, 200, 250]) == (250, 100)
    assert checkpoint_plan([0, 100, 200]) == (200, 100)
    assert checkpoint_plan([0, 7]) == (7, 7)
    for bad in ([0], [100, 200], [0, 100, 250], [0, 100, 200, 200], [0, 0, 100]):
        with pytest.raises(ValueError):
            checkpoint_plan(bad)


def test_cold_collapse_ic_properties(lib):
    """galaxy.rs:11-56: the requested count, particles at rest, and every particle within
    the sphere plus a 10 % margin for the COM shift."""
    p = G.ColdCollapse(500).generate()
    assert p.count == 500
    q = G.ColdCollapse(100).generate()
    assert not q.vx.any() and not q.vy.any() and not q.vz.any()
    radius = 2.0
    r = G.ColdCollapse(1000, radius=radius).generate()
    margin = radius * 0.1
    assert (r.x ** 2 + r.y ** 2 + r.z ** 2 <= (radius + margin) ** 2).all()
