"""The 2D drop-in binding (oracle/ref/binding_tg_fhist.cpp: a subclass of the
reference's TG_solver_<0,1,0> whose calc_step is one libfhist step) compiles
against the reference's own fr_d_t_g_2d.cpp and links with libfhist.so.  CPU
only: needs the reference sources, so it is skipped where they are absent.
Without a GPU the binary takes the library's error path and exits cleanly."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(REPO, "oracle", "ref")
EXE = os.path.join(REPO, "oracle", "_ref", "tg_fhist")


def test_tg_binding_compiles_and_links_against_the_reference_class():
    from theses_code_gb300 import build
    build.build()
    out = subprocess.run(["make", "-s", "-C", REF_DIR, "binding"], capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr
    if "not found" in out.stdout:
        pytest.skip("reference sources not present")
    assert os.access(EXE, os.X_OK)
    import torch
    if torch.cuda.is_available():
        return
    n = 14 * 14
    stdin = " ".join(["0.5"] * n + ["0.1"] * n) + "\n"
    r = subprocess.run([EXE, "12", "12", "5e-4", "0.7", "0.1", "0.1", "0", "3"], input=stdin, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 4 and "libfhist:" in r.stderr, (r.returncode, r.stderr)
