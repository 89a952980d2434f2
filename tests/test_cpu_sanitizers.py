"""The library's host code under AddressSanitizer (with leak checking) and
UndefinedBehaviorSanitizer: the pattern, fill-in, level, sweep-schedule,
record and gather-map builders (delfem_gb300/csrc/sched.cpp), the GiD reader
(meshio.cpp), the sweep emulator and the oracle, driven by
tests/cpu/sanitize_main.cpp on structured, permuted, high-valence and empty
meshes, with every result checked against the oracle as well."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

BUILD = os.path.join(ROOT, "tests", "cpu", "_build")
FLAGS = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
         "-ffp-contract=off"]


def _sanitizers_available():
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(BUILD, "probe.cpp")
    with open(src, "w") as f:
        f.write("int main() { return 0; }\n")
    r = subprocess.run(["g++", *FLAGS, src, "-o", os.path.join(BUILD, "probe")], capture_output=True)
    return r.returncode == 0


def test_host_code_under_sanitizers():
    if shutil.which("g++") is None or shutil.which("gcc") is None or not _sanitizers_available():
        pytest.skip("no g++/gcc with ASan and UBSan")
    inc = [d for d in ("/usr/local/cuda/include",) if os.path.isdir(d)]
    if not inc:
        pytest.skip("CUDA headers absent (sched.cpp names cudaStream_t)")
    oracle_obj = os.path.join(BUILD, "dfg_oracle_san.o")
    subprocess.run(["gcc", *FLAGS, "-c", os.path.join(ROOT, "oracle", "dfg_oracle.c"), "-o", oracle_obj], check=True)
    exe = os.path.join(BUILD, "sanitize")
    csrc = os.path.join(ROOT, "delfem_gb300", "csrc")
    subprocess.run(["g++", *FLAGS, "-std=c++17", f"-I{inc[0]}",
                    os.path.join(ROOT, "tests", "cpu", "sanitize_main.cpp"),
                    os.path.join(ROOT, "tests", "cpu", "sweep_emul.cpp"),
                    os.path.join(csrc, "sched.cpp"), os.path.join(csrc, "meshio.cpp"), oracle_obj,
                    "-o", exe, "-lm"], check=True)
    scratch = os.path.join(BUILD, "sanitize_scratch")
    os.makedirs(scratch, exist_ok=True)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([exe, scratch], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]
    assert "checks passed" in r.stdout
