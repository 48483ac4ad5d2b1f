"""The host thread pool of the driver (csrc/host_pool.hpp) under stress, on the CPU.

Idle workers poll for the next call before they park, so calls, joins and
parking race by design; the stress program checks that every index runs
exactly once, that exceptions reach the caller and that two callers take
turns, and ThreadSanitizer (where the compiler has it) checks the memory
ordering.
"""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "native" / "host_pool_stress.cpp"
CSRC = ROOT / "greenpeas_gb300" / "csrc"


def _build_and_run(tmp_path, flags, name):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / name
    r = subprocess.run([cxx, "-std=c++17", *flags, f"-I{CSRC}", str(SRC), "-o", str(exe), "-pthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        return None, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    return out, None


def test_host_pool_stress(tmp_path):
    out, err = _build_and_run(tmp_path, ["-O2"], "pool_o2")
    assert err is None, err
    assert out.returncode == 0 and "pool stress ok" in out.stdout, out.stdout + out.stderr


def test_host_pool_under_thread_sanitizer(tmp_path):
    out, err = _build_and_run(tmp_path, ["-O1", "-g", "-fsanitize=thread"], "pool_tsan")
    if err is not None:
        pytest.skip("ThreadSanitizer is not available: " + err.splitlines()[-1] if err else "")
    assert out.returncode == 0 and "pool stress ok" in out.stdout, out.stdout + out.stderr
    assert "WARNING: ThreadSanitizer" not in out.stderr, out.stderr
