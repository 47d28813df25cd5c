"""The C++ host layer over the C ABI (include/hp_cuda.hpp, the mirror of the
reference's backend traits) and the C++ port of the reference's device-backend
integration tests (tests/cpp/backend_parity.cpp, after
backend/src/ascend910b3/integration_tests.rs), built with g++ against
libhp_cuda.so and the oracle library.  CPU: the header compiles on its own
with warnings as errors and the parity program links; GPU: the program runs
and every case passes."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "backend_parity.cpp"
OUT_DIR = ROOT / "tests" / "cpp" / "_build"

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


def _build_parity() -> pathlib.Path:
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    out = OUT_DIR / "backend_parity"
    lib_dir = ROOT / "hyperplonk_gb300" / "_build"
    oracle_dir = ROOT / "oracle" / "_build"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
                    f"-I{ROOT / 'oracle'}", str(SRC), "-o", str(out), f"-L{lib_dir}", "-lhp_cuda", f"-L{oracle_dir}",
                    "-lhp_oracle", "-lpthread", f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{oracle_dir}"],
                   check=True, capture_output=True, text=True)
    return out


def test_header_compiles_standalone(tmp_path):
    tu = tmp_path / "tu.cpp"
    tu.write_text('#include "hp_cuda.hpp"\n'
                  "int main() {\n"
                  "  using namespace hp_cuda;\n"
                  "  const Fr a = fr::from_u64(7), b = fr::from_u64(6);\n"
                  "  return fr::mul(a, b) == fr::from_u64(42) && fr::mul(fr::inv(a), a) == fr::one() &&\n"
                  "         fr::sub(b, a) == fr::neg(fr::one()) ? 0 : 1;\n"
                  "}\n")
    exe = tmp_path / "tu"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Wpedantic", "-Werror", f"-I{ROOT / 'include'}",
                    str(tu), "-o", str(exe), f"-L{ROOT / 'hyperplonk_gb300' / '_build'}", "-lhp_cuda",
                    f"-Wl,-rpath,{ROOT / 'hyperplonk_gb300' / '_build'}"], check=True, capture_output=True, text=True)
    # the host field helpers need no GPU
    assert subprocess.run([str(exe)]).returncode == 0


def test_parity_program_builds(native_lib, oracle):
    assert _build_parity().exists()


@pytest.mark.gpu
def test_cpp_backend_parity(native_lib, oracle):
    exe = _build_parity()
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stdout[-4000:] + res.stderr[-4000:]
    assert " 0 failed;" in res.stdout and res.stdout.rstrip().endswith("0 failed")
