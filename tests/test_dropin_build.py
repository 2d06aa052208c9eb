"""The drop-in claim: the reference's own drivers and system plugin
(src/qms.cu, src/qsa.cu, src/evo.cu, src/test_suqa.cu, src/system.cu) compile,
unchanged, against the suqa_gb300 headers alone and link against libsq; the
linked reference qms binary runs, and on a machine without a GPU it stops
cleanly with libsq's no-device status.  Runs where the reference sources are
present (SUQA_REFERENCE, default the reference checkout of this machine);
compiles into a temporary directory (nothing is copied into the repository)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SUQA_REFERENCE", "/root/reference")
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


def test_linked_reference_qms_runs_and_reports_a_missing_gpu(tmp_path):
    """The reference's own qms driver, linked against libsq, parses its command
    line and reaches suqa::setup; without a GPU the shim ends it with exit status
    SQ_ERR_NODEVICE (5) and a one-line message, before any output file exists."""
    lib = os.path.join(BUILD, "libsq.so")
    shim = os.path.join(BUILD, "suqa_shim.o")
    if not (os.path.exists(lib) and os.path.exists(shim)):
        pytest.skip("libsq not built")
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present: the driver would run for real")
    except ImportError:
        pass
    objs = []
    for name in ("qms", "system"):
        o = str(tmp_path / f"{name}.o")
        _compile(os.path.join(REF, "src", f"{name}.cu"), o, tmp_path)
        objs.append(o)
    exe = str(tmp_path / "qms")
    r = subprocess.run(["g++"] + objs + [shim, "-L" + BUILD, "-lsq", "-Wl,-rpath," + BUILD, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = tmp_path / "out"
    r = subprocess.run([exe, "1.0", "200", "1", "4", str(out), "--seed", "42", "--ene-min", "-1", "--ene-max", "3",
                        "--thermalization", "20"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 5, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
    assert "no CUDA device" in r.stderr
    assert not out.exists()
