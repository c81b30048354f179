"""Host-side logic of libpof under random inputs, no GPU:
- the planners (csrc/pof_plan.h, csrc/pof_bplan.h): workspace regions
  aligned, disjoint and inside the reported size; level counts; batch chunk
  and group tables that cover every problem's steps exactly once and never
  span two problems (tests/plan_props.cpp);
- the serving engine's first-fit arena (csrc/pof_arena.h): free list sorted,
  coalesced and equal to the unowned grid points, first-fit placement
  (tests/arena_props.cpp).
The checks are C++, built here with the host compiler."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "parallel-in-time-ode-filters_gb300", "csrc")


def _build(tmp_path_factory, name):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp(name) / name)
    src = os.path.join(ROOT, "tests", name + ".cpp")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", CSRC, src, "-o", exe], check=True,
                   capture_output=True, text=True)
    return exe


@pytest.fixture(scope="module")
def plan_props(tmp_path_factory):
    return _build(tmp_path_factory, "plan_props")


@pytest.fixture(scope="module")
def arena_props(tmp_path_factory):
    return _build(tmp_path_factory, "arena_props")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_plans_hold_their_invariants(plan_props, seed):
    r = subprocess.run([plan_props, "3000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok 3000"


@pytest.mark.parametrize("seed", [1, 2])
def test_arena_keeps_a_coalesced_first_fit_free_list(arena_props, seed):
    r = subprocess.run([arena_props, "300", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok 300"
