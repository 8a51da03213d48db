"""The SUNDIALS vector shim (ceda_demonstrations_gb300/integration/sts_sundials_nvector.c),
the binding a maintainer adds to drive this library's vector from a real SUNDIALS build of the
reference: it compiles against a stand-in of SUNDIALS' public N_Vector header (SUNDIALS is an
empty submodule in the reference), links against libstsgpu.so with every symbol resolved, and
wraps a vector with all the operations it forwards. No GPU work."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sundials_shim_compiles_links_and_wires_the_ops(stslib, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = stslib.lib()._name
    exe = str(tmp_path / "shim_check")
    cmd = [cc, "-std=c11", "-Wall", "-Wextra", "-Werror",
           "-I" + os.path.join(ROOT, "tests", "sundials_standin"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "ceda_demonstrations_gb300", "integration", "sts_sundials_nvector.c"),
           os.path.join(ROOT, "tests", "sundials_standin", "standin.c"), "-o", exe,
           "-L" + os.path.dirname(lib), "-lstsgpu", "-Wl,-rpath," + os.path.dirname(lib), "-Wl,--no-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
