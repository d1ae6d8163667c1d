"""bench.py's command line (no GPU): the defaults the run contract relies on."""
import sys

import pytest

import bench


def parse(*argv):
    old = sys.argv
    sys.argv = ["bench.py", *argv]
    try:
        return bench.parse()
    finally:
        sys.argv = old


def test_default_is_the_headline_direct_sum():
    a = parse()
    assert a.workload == "direct" and a.n == 1 << 20 and a.gpus == 1 and a.impl == "gvs"
    assert a.warmup >= 3 and a.precision == "mixed"


@pytest.mark.parametrize("workload,n", [("bh", 1 << 22), ("sph", 1 << 18), ("plummer1k", 1 << 20)])
def test_workload_sizes(workload, n):
    assert parse("--workload", workload).n == n
    assert parse("--workload", workload, "--n", "4096").n == 4096


def test_adjoint_configuration():
    a = parse("--workload", "adjoint", "--adjoint-steps", "1000")
    assert a.adjoint_n == 16384 and a.adjoint_steps == 1000


def test_reference_arm_flag():
    assert parse("--impl", "reference").impl == "reference"
