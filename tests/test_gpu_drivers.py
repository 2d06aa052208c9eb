"""Full QMS / QSA / evo runs through the C++ drop-in layer (suqa_gb300/include,
shim, triangle plugin, drivers) on the GPU, diffed against the output files the
reference CPU build wrote for the same command lines (tests/golden/runs)."""
import os
import re
import subprocess

import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "suqa_gb300", "_build")


def run_driver(name, tmp_path):
    man = golden_io.run_manifest()[name]
    out = str(tmp_path / f"{name}.txt")
    exe = os.path.join(BUILD, man["driver"] if not name.startswith("tfim")
                       else "qms_tfim_s" + re.match(r"tfim_s(\d+)", name).group(1))
    argv = [exe] + [a.replace("{out}", out) for a in man["args"]]
    env = dict(os.environ)
    env.update(man["env"])
    cp = subprocess.run(argv, capture_output=True, text=True, env=env, timeout=900)
    assert cp.returncode == 0, cp.stdout[-2000:] + cp.stderr[-2000:]
    return man, out, cp.stdout


@pytest.mark.parametrize("name", ["qms_c1", "qms_e6", "qms_rev", "qms_win"])
def test_qms_runs_match_reference_output(name, tmp_path):
    man, out, stdout = run_driver(name, tmp_path)
    assert open(out).read() == golden_io.run_output(name)
    acc = re.findall(r"acceptance: *([^\n]*)", stdout)
    assert acc and acc[0].strip() == man["acceptance"]
    if man["revcounts"]:
        assert open(out + "_revcounts").read() == golden_io.run_output(f"{name}_revcounts")


@pytest.mark.parametrize("name", ["qsa_c1", "qsa_s3"])
def test_qsa_runs_match_reference_output(name, tmp_path):
    man, out, _ = run_driver(name, tmp_path)
    assert open(out).read() == golden_io.run_output(name)


def test_evo_probabilities_match_reference(tmp_path):
    man, out, _ = run_driver("evo", tmp_path)
    got = np.loadtxt(out)
    want = np.loadtxt(os.path.join(golden_io.GOLDEN, "runs", "evo.txt"))
    assert got.shape == want.shape
    assert np.max(np.abs(got - want)) < 1e-11


@pytest.mark.parametrize("name", ["tfim_s4", "tfim_s5", "tfim_s6", "tfim_s7_e6"])
def test_qms_tfim_drivers_match_reference_output(name, tmp_path):
    """The host-driven drop-in path with the TFIM ring plugin."""
    man, out, stdout = run_driver(name, tmp_path)
    assert open(out).read() == golden_io.run_output(name)


def _gate_count_table(stdout):
    lines = stdout.splitlines()
    i = lines.index("Gate counts")
    out = []
    for ln in lines[i:]:
        if out and ln == "" and len(out) > 3:
            break
        out.append(ln)
    return "\n".join(out).strip() + "\n"


@pytest.mark.parametrize("name", ["qms_c1", "qms_rev", "qsa_c1"])
def test_gate_count_tables_match_reference(name, tmp_path):
    """Drivers built with -DGATECOUNT print the reference's gate-cost table
    (one- and two-qubit gate counts per metro step, sample, measurement,
    restoration / annealing step) identically."""
    man = golden_io.run_manifest()[name]
    out = str(tmp_path / f"{name}.txt")
    argv = [os.path.join(BUILD, man["driver"] + "_gc")] + [a.replace("{out}", out) for a in man["args"]]
    cp = subprocess.run(argv, capture_output=True, text=True, timeout=900)
    assert cp.returncode == 0, cp.stdout[-2000:] + cp.stderr[-2000:]
    assert _gate_count_table(cp.stdout) == golden_io.run_output(f"{name}_gatecounts")
    assert open(out).read() == golden_io.run_output(name)  # counting changes no result
