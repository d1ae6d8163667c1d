"""The C++ host layer (gravis_gb300/host/): the headless runner gvs_headless and
the drop-in class check gvs_host_check.

CPU: the runner validates its arguments the way crates/headless/src/main.rs:66-95
does, before touching a GPU.  GPU: the runner reproduces the reference's own
diagnostics artifacts (m1_plummer_1k_diag.csv: N=1000 seed 42, suggested eps and
dt, 1000 steps, a row every 100; m1_kepler_diag.csv: the e=0.5 two-body orbit, a
row every 10^4 steps) to 1e-10 relative, and the per-call GravitySolver /
Integrator / SphSolver classes give the device-resident path's results bit for bit.
"""
import csv
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADLESS = os.path.join(ROOT, "gravis_gb300", "gvs_headless")
CHECK = os.path.join(ROOT, "gravis_gb300", "gvs_host_check")


@pytest.fixture(scope="module")
def built():
    from gravis_gb300 import build
    build.build()
    assert os.path.exists(HEADLESS) and os.path.exists(CHECK)


def run(*args, timeout=600):
    return subprocess.run([HEADLESS, *args], capture_output=True, text=True, timeout=timeout)


@pytest.mark.parametrize("args,msg", [
    (["--eccentricity", "1.0"], "--eccentricity must be in [0, 1)"),
    (["--particles", "0"], "--particles must be > 0"),
    (["--dt", "-1e-3"], "--dt must be positive"),
    (["--softening", "-0.1"], "--softening must be non-negative"),
    (["--algorithm", "fmm"], "--algorithm must be brute-force or barnes-hut"),
])
def test_headless_validates_arguments(built, args, msg):
    r = run(*args)
    assert r.returncode == 1
    assert msg in r.stderr


def test_headless_help(built):
    r = run("--help")
    assert r.returncode == 0 and "--diag-csv" in r.stdout


def read_csv(path):
    with open(path) as fh:
        rows = list(csv.DictReader(fh))
    return rows


@pytest.mark.gpu
def test_headless_reproduces_plummer_artifact(built, golden, tmp_path):
    out = tmp_path / "diag.csv"
    r = run("--scenario", "plummer", "-n", "1000", "--seed", "42", "--steps", "1000", "--diag-interval", "100",
            "--diag-csv", str(out))
    assert r.returncode == 0, r.stderr
    rows = read_csv(out)
    ref = golden["m1_plummer_1k_diag.csv"]["rows"]  # step, time, K, U, E, |p|, |L|, com, virial
    assert [int(x["step"]) for x in rows] == [int(v[0]) for v in ref]
    for got, want in zip(rows, ref):
        for col, k in (("kinetic_energy", 2), ("potential_energy", 3), ("total_energy", 4)):
            assert abs(float(got[col]) - want[k]) <= 1e-10 * abs(want[k]), (got["step"], col, got[col], want[k])


@pytest.mark.gpu
def test_headless_reproduces_kepler_rows(built, golden, tmp_path):
    out = tmp_path / "kepler.csv"
    r = run("--scenario", "two-body", "--steps", "20000", "--diag-interval", "10000", "--diag-csv", str(out))
    assert r.returncode == 0, r.stderr
    rows = read_csv(out)
    ref = golden["m1_kepler_diag.csv"]["rows"]
    for got, want in zip(rows, ref[:3]):
        assert int(got["step"]) == int(want[0])
        for col, k in (("kinetic_energy", 2), ("total_energy", 4)):
            assert abs(float(got[col]) - want[k]) <= 1e-10 * abs(want[k]), (got["step"], col)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64-exact", "mixed"])
def test_headless_evrard_sph(built, tmp_path, precision):
    out = tmp_path / "evrard.csv"
    r = run("--scenario", "evrard-collapse", "-n", "1000", "--steps", "20", "--diag-interval", "10",
            "--precision", precision, "--diag-csv", str(out))
    assert r.returncode == 0, r.stderr
    rows = read_csv(out)
    assert [int(x["step"]) for x in rows] == [0, 10, 20]
    e0, e1 = float(rows[0]["total_energy"]), float(rows[-1]["total_energy"])
    assert float(rows[0]["thermal_energy"]) > 0.0
    assert abs((e1 - e0) / e0) < 1e-2


@pytest.mark.gpu
@pytest.mark.parametrize("scenario,steps", [("cold-collapse", 100), ("cold-collapse-gas", 20)])
def test_headless_cold_collapse(built, tmp_path, scenario, steps):
    """scenario_builder's cold-collapse names run through the headless mirror: particles
    start at rest (K = 0) and fall inward, conserving energy over the first steps."""
    out = tmp_path / "cold.csv"
    r = run("--scenario", scenario, "-n", "2000", "--steps", str(steps), "--diag-interval", str(steps // 2),
            "--diag-csv", str(out))
    assert r.returncode == 0, r.stderr
    rows = read_csv(out)
    assert [int(x["step"]) for x in rows] == [0, steps // 2, steps]
    assert float(rows[0]["kinetic_energy"]) == 0.0
    assert float(rows[-1]["kinetic_energy"]) > 0.0
    e0, e1 = float(rows[0]["total_energy"]), float(rows[-1]["total_energy"])
    assert abs((e1 - e0) / e0) < 1e-2
    assert (float(rows[0]["thermal_energy"]) > 0.0) == (scenario == "cold-collapse-gas")


@pytest.mark.gpu
def test_drop_in_classes_match_resident_path(built):
    r = subprocess.run([CHECK], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok  ") == 5


# ---- snapshots (snapshot.rs: NBODY001..003) --------------------------------------------
def test_snapshot_round_trip_and_old_versions(tmp_path):
    """snapshot.rs:187-258 on the Python mirror: NBODY003 round trip; NBODY001/002
    files read with zero types / gas fields."""
    import io
    import numpy as np
    import gravis_gb300 as G
    p = G.Particles(5)
    rng = np.random.default_rng(3)
    for f in ("x", "y", "z", "vx", "vy", "vz", "mass", "internal_energy", "smoothing_length", "density"):
        getattr(p, f)[:] = rng.random(5)
    p.particle_type[:] = [0, 4, 4, 1, 0]
    buf = io.BytesIO()
    G.Snapshot.capture(p, 1.25, 77, 0.01, 1e-3).write_to(buf)
    raw = buf.getvalue()
    assert raw[:8] == b"NBODY003" and len(raw) == 8 + 5 * 8 + 7 * 5 * 8 + 5 + 3 * 5 * 8
    s = G.Snapshot.read_from(io.BytesIO(raw))
    assert (s.time, s.step, s.softening, s.dt) == (1.25, 77, 0.01, 1e-3)
    for f in ("x", "vz", "mass", "internal_energy", "density"):
        assert np.array_equal(getattr(s.particles, f), getattr(p, f))
    assert np.array_equal(s.particles.particle_type, p.particle_type)
    assert np.all(s.particles.ax == 0.0)
    v1 = b"NBODY001" + raw[8:8 + 40 + 7 * 40]
    s1 = G.Snapshot.read_from(io.BytesIO(v1))
    assert np.all(s1.particles.particle_type == 0) and np.all(s1.particles.internal_energy == 0.0)
    assert np.array_equal(s1.particles.y, p.y)
    with pytest.raises(ValueError):
        G.Snapshot.read_from(io.BytesIO(b"NBODY999" + raw[8:]))


@pytest.mark.gpu
def test_headless_snapshot_restart_is_seamless(built, tmp_path):
    """Run 200 steps writing snapshots every 100; restart from step 100 and run 100
    more: the step-200 snapshots are identical (FP64_EXACT, accelerations recomputed
    on restart as Snapshot::initialize does), and Python reads the C++ files."""
    import numpy as np
    import gravis_gb300 as G
    a, b = tmp_path / "a", tmp_path / "b"
    r = run("--scenario", "plummer", "-n", "2000", "--steps", "200", "--diag-interval", "0",
            "--snapshot-interval", "100", "--snapshot-dir", str(a))
    assert r.returncode == 0, r.stderr
    r = run("--restart", str(a / "snap_00000100.bin"), "--steps", "100", "--diag-interval", "0",
            "--snapshot-interval", "100", "--snapshot-dir", str(b))
    assert r.returncode == 0, r.stderr
    with open(a / "snap_00000200.bin", "rb") as fa, open(b / "snap_00000200.bin", "rb") as fb:
        sa, sb = G.Snapshot.read_from(fa), G.Snapshot.read_from(fb)
    assert sa.step == sb.step == 200 and sa.time == sb.time
    for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
        assert np.array_equal(getattr(sa.particles, f), getattr(sb.particles, f)), f
