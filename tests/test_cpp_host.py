"""The C++ host surface (everett_gb300/cpp/everett.hpp): circuit building,
validation errors, OpenQASM round trips, the seeded Rng and gate identities,
run as a compiled C++ program against the engine library without a GPU."""
import subprocess

import pytest

from cpp_build import build_test_program, run_group


@pytest.fixture(scope="module")
def program(engine, tmp_path_factory):
    try:
        return build_test_program(tmp_path_factory.mktemp("cpp"))
    except subprocess.CalledProcessError as e:
        pytest.fail(f"C++ test program failed to build:\n{e.stderr}")


def test_cpp_host_cases(program):
    r = run_group(program, "host")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "16 run, 0 failed" in r.stdout, r.stdout


@pytest.mark.parametrize("seed", [0, 1, 42, 2**64 - 1])
def test_cpp_rng_matches_oracle(program, seed):
    """The header's Rng draws rng.rs's stream, bit for bit."""
    import oracle
    r = subprocess.run([str(program), "rng", str(seed), "64"], capture_output=True,
                       text=True, timeout=60, check=True)
    lines = r.stdout.split()
    u64 = [int(v) for v in lines[:64]]
    f64 = [float.fromhex(v) for v in lines[64:]]
    assert u64 == [int(v) for v in oracle.rng_u64(seed, 64)]
    assert f64 == [float(v) for v in oracle.rng_f64(seed, 64)]


def test_integer_pipe_product_host(tmp_path):
    """The integer-pipe double product and add (everett_gb300/csrc/
    ev_softfp.cuh), compiled for the host, equal the host's IEEE
    multiplication and addition on 2*10^7 operand pairs each from families
    that reach every rounding case (sums: also cancellation and exponent gaps
    at the alignment's edges)."""
    import shutil
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    gxx = shutil.which("g++")
    assert gxx, "g++ is required"
    exe = tmp_path / "test_softfp"
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
                    "-I", str(root / "everett_gb300" / "csrc"),
                    str(root / "tests" / "cpp" / "test_softfp.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    for seed in ("3", "4"):
        r = subprocess.run([str(exe), "10000000", seed], capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert ", 0 mismatches" in r.stdout, r.stdout
        assert ", 0 sum mismatches" in r.stdout, r.stdout
