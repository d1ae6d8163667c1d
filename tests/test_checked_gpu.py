"""The bounds-checked build (libgvs_checked.so, compiled with -DGVS_CHECKED):
every path on small cases, in a child process that loads the checked library,
with results against the oracle and the device error word zero after each step
(no computed index left its array, the tree kept its invariants)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_runs_every_path_clean():
    env = dict(os.environ, GVS_CHECKED="1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "checked_paths.py")], capture_output=True, text=True,
                       env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert "checked" in out["version"]
    assert len(out["steps"]) >= 20
    for name, st in out["steps"].items():
        assert st["flags"] == 0, (name, st)
        if st["bar"] is not None:
            assert st["err"] <= st["bar"], (name, st)
