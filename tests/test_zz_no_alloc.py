"""gvs_diagnostics_noalloc: the diagnostics entry point that allocates nothing.

It exists for callers that cannot allocate device memory themselves -- hosts
whose allocator owns all device memory, code running under CUDA graph
capture, real-time loops -- and therefore hand the library device arrays they
already own.  Its scratch is a fixed array inside the library.  This test
calls it through the C ABI on device arrays and checks it against the
allocating gvs_diagnostics on the same state, twice in a row (the fixed
scratch keeps the previous call's contents, which must not leak into the
next result).  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

import gravis_gb300 as G
from gravis_gb300 import _lib as L

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, as the diagnostics parity tests use


def _dev(t):
    return C.c_void_p(t.data_ptr())


def _close(a, b):
    return abs(a - b) <= TOL * max(abs(b), 1e-300)


def _check(d, e):
    for f in ("kinetic_energy", "potential_energy", "thermal_energy", "total_energy", "virial_ratio"):
        assert _close(getattr(d, f), getattr(e, f)), (f, getattr(d, f), getattr(e, f))
    for f in ("momentum", "angular_momentum", "center_of_mass", "center_of_mass_velocity"):
        a, b = np.array(getattr(d, f)[:]), np.array(getattr(e, f)[:])
        assert np.allclose(a, b, rtol=TOL, atol=1e-18), (f, a, b)


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = L.load()
    ctx = G.Context(0)
    try:
        for p, eps, gas in ((G.PlummerSphere(20000, seed=4).generate(), 0.01, False),
                            (G.EvrardCollapse(3000, seed=2).generate(), 0.02, True)):
            ctx.set_state(p)
            want = L.Diag()
            L.check(lib.gvs_diagnostics(ctx.h, eps, 1, C.byref(want)), ctx.h)
            dev = {f: torch.from_numpy(getattr(p, f).copy()).cuda() for f in
                   ("x", "y", "z", "vx", "vy", "vz", "mass", "internal_energy")}
            ptype = torch.from_numpy(p.particle_type.copy()).cuda() if gas else None
            torch.cuda.synchronize()
            for _ in range(2):  # two calls in a row share the fixed scratch
                got = L.Diag()
                st = lib.gvs_diagnostics_noalloc(
                    0, None, p.count, _dev(dev["x"]), _dev(dev["y"]), _dev(dev["z"]), _dev(dev["vx"]),
                    _dev(dev["vy"]), _dev(dev["vz"]), _dev(dev["mass"]), _dev(ptype) if gas else None,
                    _dev(dev["internal_energy"]) if gas else None, eps, 1, C.byref(got))
                L.check(st)
                _check(got, want)
            if gas:
                assert got.thermal_energy > 0.0
    finally:
        ctx.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = L.load()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    d = L.Diag()
    st = lib.gvs_diagnostics_noalloc(0, None, (1 << 22) + 1, *([_dev(x)] * 7), None, None, 0.01, 1, C.byref(d))
    assert st == L.ERR_INVALID_ARG
    assert "scratch limit" in L.last_error(None)
