"""The C++ host classes (include/fhist.hpp) driven like the reference drives
its solvers, checked against the oracle by a compiled C++ program."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def host_parity_bin(tmp_path_factory):
    from oracle import oracle as O
    O.build()
    lib = os.path.join(ROOT, "theses_code_gb300")
    orc = os.path.join(ROOT, "oracle", "_build")
    out = str(tmp_path_factory.mktemp("cpp") / "host_parity")
    cmd = ["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "host_parity.cpp"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
           "-I", "/usr/local/cuda/include",
           "-L", lib, "-lfhist", "-L", orc, "-lfh_oracle", f"-Wl,-rpath,{lib}:{orc}", "-o", out]
    subprocess.run(cmd, check=True)
    return out


def test_host_classes_match_oracle(host_parity_bin):
    r = subprocess.run([host_parity_bin], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    names = [line.split()[0] for line in r.stdout.strip().splitlines()]
    assert names == ["tg_solver_fp64", "tg_solver_df64", "tg_solver_blocked", "tg_solver_massN_variable_d",
                     "tg_solver_two_series", "h_solver_l1", "h_solver_psi", "h_batch_restart", "ab_solver"]
