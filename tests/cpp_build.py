"""Builds tests/cpp/test_everett.cpp, the C++ host surface's test program,
against the engine library (g++, C++17, rpath to the in-tree library)."""
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "test_everett.cpp"
LIBDIR = ROOT / "everett_gb300"


def build_test_program(out_dir: Path) -> Path:
    gxx = shutil.which("g++")
    if gxx is None:
        raise RuntimeError("g++ is required to build the C++ host tests")
    exe = out_dir / "test_everett"
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", str(LIBDIR / "cpp"), str(SRC), "-o", str(exe),
           "-L", str(LIBDIR), "-leverett_gb300", f"-Wl,-rpath,{LIBDIR}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def run_group(exe: Path, group: str) -> subprocess.CompletedProcess:
    return subprocess.run([str(exe), group], capture_output=True, text=True, timeout=600)
