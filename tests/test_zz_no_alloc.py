"""gvs_diagnostics_noalloc: the diagnostics entry point that allocates nothing.

It exists for callers that cannot allocate device memory themselves -- hosts
whose own allocator owns all device memory, real-time loops that cannot
afford an allocation's device synchronisation -- and therefore hand the
library device arrays they already own.  Its scratch is a fixed array inside
the library.  This test calls it through the C ABI on device arrays and checks
it against the allocating gvs_diagnostics on the same state, two calls in a
row per state, first on a larger system and then on a smaller one (the fixed
scratch keeps the previous call's contents, which must not leak into the next
result), once without the potential and once on a non-default stream.  It
lives in its own file, collected last.
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


def _check(d, e, with_potential=True):
    fields = ["kinetic_energy", "thermal_energy"]
    if with_potential:
        fields += ["potential_energy", "total_energy", "virial_ratio"]
    for f in fields:
        assert _close(getattr(d, f), getattr(e, f)), (f, getattr(d, f), getattr(e, f))
    for f in ("momentum", "angular_momentum", "center_of_mass", "center_of_mass_velocity"):
        a, b = np.array(getattr(d, f)[:]), np.array(getattr(e, f)[:])
        assert np.allclose(a, b, rtol=TOL, atol=1e-18), (f, a, b)


def _noalloc(lib, p, dev, gas, eps, with_potential, stream=None):
    got = L.Diag()
    st = lib.gvs_diagnostics_noalloc(
        0, stream, p.count, _dev(dev["x"]), _dev(dev["y"]), _dev(dev["z"]), _dev(dev["vx"]),
        _dev(dev["vy"]), _dev(dev["vz"]), _dev(dev["mass"]), _dev(dev["ptype"]) if gas else None,
        _dev(dev["internal_energy"]) if gas else None, eps, with_potential, C.byref(got))
    L.check(st)
    return got


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = L.load()
    ctx = G.Context(0)
    try:
        # the larger system first, so the smaller one runs over its leftover partial sums
        for p, eps, gas in ((G.PlummerSphere(20000, seed=4).generate(), 0.01, False),
                            (G.EvrardCollapse(3000, seed=2).generate(), 0.02, True)):
            ctx.set_state(p)
            want = L.Diag()
            L.check(lib.gvs_diagnostics(ctx.h, eps, 1, C.byref(want)), ctx.h)
            dev = {f: torch.from_numpy(getattr(p, f).copy()).cuda() for f in
                   ("x", "y", "z", "vx", "vy", "vz", "mass", "internal_energy")}
            dev["ptype"] = torch.from_numpy(p.particle_type.copy()).cuda()
            torch.cuda.synchronize()
            for _ in range(2):  # two calls in a row share the fixed scratch
                got = _noalloc(lib, p, dev, gas, eps, 1)
                _check(got, want)
            if gas:
                assert got.thermal_energy > 0.0
            # without the potential, on a stream of the caller's own
            s = torch.cuda.Stream()
            got = _noalloc(lib, p, dev, gas, eps, 0, stream=C.c_void_p(s.cuda_stream))
            assert got.potential_energy == 0.0
            _check(got, want, with_potential=False)
            assert _close(got.total_energy, want.kinetic_energy + want.thermal_energy)
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
