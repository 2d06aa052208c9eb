"""The drop-in claim: the reference's own drivers and system plugin
(src/qms.cu, src/qsa.cu, src/evo.cu, src/test_suqa.cu, src/system.cu) compile,
unchanged, against the suqa_gb300 headers alone and link against libsq.
Runs where the reference sources are present; compiles into a temporary
directory (nothing is copied into the repository)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"
BUILD = os.path.join(ROOT, "suqa_gb300", "_build")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference sources not present")


def _compile(src, out, tmp, extra=()):
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-DNDEBUG", *extra, "-x", "c++",
           "-I" + os.path.join(ROOT, "suqa_gb300", "include"), "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.parametrize("driver,gatecount", [("qms", False), ("qsa", False), ("evo", False), ("test_suqa", False),
                                             ("qms", True), ("qsa", True), ("test_suqa", True)])
def test_reference_driver_compiles_and_links_unchanged(driver, gatecount, tmp_path):
    """Also with -DGATECOUNT, the reference's gate-cost counter build."""
    lib = os.path.join(BUILD, "libsq.so")
    shim = os.path.join(BUILD, "suqa_shim.o")
    if not (os.path.exists(lib) and os.path.exists(shim)):
        pytest.skip("libsq not built")
    objs = []
    for name in (driver, "system"):
        o = str(tmp_path / f"{name}.o")
        _compile(os.path.join(REF, "src", f"{name}.cu"), o, tmp_path, ("-DGATECOUNT",) if gatecount else ())
        objs.append(o)
    exe = str(tmp_path / driver)
    r = subprocess.run(["g++"] + objs + [shim, "-L" + BUILD, "-lsq", "-Wl,-rpath," + BUILD, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(exe)
