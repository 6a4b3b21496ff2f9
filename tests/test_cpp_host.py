"""The C++ host surface over the C ABI (include/knc.hpp): knc::advance moves a
knc::State through the GPU the way scheme::advance (src/scheme.rs:212-240)
moves the reference's State. tests/cpp/test_advance.cpp compares it with the
CPU oracle; here it is compiled against the library and the oracle (a CPU
check that the header builds and links) and run on the GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "test_advance.cpp"


def _build(tmp_path):
    import build as b
    import knc_oracle
    from knc import abi
    if not abi.LIB_PATH.exists():
        b.build()
    knc_oracle.build()
    gxx = shutil.which("g++") or shutil.which("c++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "test_advance"
    lib_dir = abi.LIB_PATH.parent
    oracle_dir = ROOT / "oracle" / "_build"
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", str(SRC), "-o", str(exe),
           f"-L{lib_dir}", "-lknc_gpu", f"-L{oracle_dir}", "-lknc_oracle",
           f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{oracle_dir}", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_host_builds_and_links(tmp_path):
    assert _build(tmp_path).exists()


@pytest.mark.gpu
def test_cpp_host_matches_oracle(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok  ") == 5, r.stdout
