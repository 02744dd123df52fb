"""The C++ host surface on the GPU: the reference's state, preparation, QFT,
teleportation, phase-estimation and superdense tests written in C++ against everett.hpp and run through
the engine (tests/cpp/test_everett.cpp, group "gpu")."""
import subprocess

import pytest

from cpp_build import build_test_program, run_group

pytestmark = pytest.mark.gpu


def test_cpp_gpu_cases(gpu, tmp_path_factory):
    try:
        exe = build_test_program(tmp_path_factory.mktemp("cppgpu"))
    except subprocess.CalledProcessError as e:
        pytest.fail(f"C++ test program failed to build:\n{e.stderr}")
    r = run_group(exe, "gpu")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "17 run, 0 failed" in r.stdout, r.stdout
