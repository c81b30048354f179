"""Host-side planners of libpof (csrc/pof_plan.h, csrc/pof_bplan.h) under
random shapes: workspace regions aligned, disjoint and inside the reported
size; level counts; batch chunk and group tables that cover every problem's
steps exactly once and never span two problems.  The checks are C++
(tests/plan_props.cpp), built here with the host compiler; no GPU."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "parallel-in-time-ode-filters_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "plan_props.cpp")


@pytest.fixture(scope="module")
def plan_props(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("plan") / "plan_props")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", CSRC, SRC, "-o", exe], check=True,
                   capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_plans_hold_their_invariants(plan_props, seed):
    r = subprocess.run([plan_props, "3000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok 3000"
