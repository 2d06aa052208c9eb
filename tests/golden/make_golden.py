"""Regenerates the golden fixtures in this directory from the reference CPU build.

Run where the reference sources are present (it builds oracle/_ref from them):

    python tests/golden/make_golden.py

Fixtures written:
  gates_scripts.txt.gz  seeded gate scripts (dumper grammar), one block per case
  gates_results.npz     the reference's outputs for each script (states, measured
                        bits, probabilities, norms)
  runs/*.txt            output files of the reference qms / qsa / evo drivers
  runs/manifest.json    command line, seed, environment and acceptance line of each run
  pcg32_draws.txt       first 16 doubles of the reference pcg wrapper for a few seeds
"""
from __future__ import annotations

import gzip
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import circuits  # noqa: E402
import oracle  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")

# (name, seed, n, ngates, dump_every) — n up to 12 so the GPU tile path is exercised
GATE_CASES = [(f"rand{s}", s, 3 + s % 10, 60, 5) for s in range(36)]
# scripts whose gates may act on qubits of the global control mask (the patterns
# the reference's QSA produces through its aliased registers)
OVERLAP_CASES = [(f"ovl{s}", 900 + s, 4 + s % 6, 60) for s in range(10)]

RUNS = [
    # config 1: the triangle, 3 + 4 + 1 = 8 qubits
    ("qms_c1", "qms", ["1.0", "200", "1", "4", "{out}", "--seed", "42", "--ene-min", "-1", "--ene-max", "3",
                       "--thermalization", "20"], {}),
    ("qms_e6", "qms", ["0.5", "150", "1", "6", "{out}", "--seed", "7", "--ene-min", "-1", "--ene-max", "3",
                       "--thermalization", "10"], {}),
    ("qms_rev", "qms", ["2.0", "150", "3", "4", "{out}", "--seed", "1", "--ene-min", "-1", "--ene-max", "3",
                        "--thermalization", "5", "--max-reverse", "3", "--record-reverse"], {}),
    ("qms_win", "qms", ["1.0", "100", "2", "3", "{out}", "--seed", "5", "--thermalization", "4"], {}),
    ("qsa_c1", "qsa", ["1.0", "5", "2", "2", "{out}", "--seed", "42", "--annealing-sequences", "20"], {}),
    ("qsa_s3", "qsa", ["0.5", "3", "2", "3", "{out}", "--seed", "3", "--annealing-sequences", "6"], {}),
    ("evo", "evo", ["12", "0.1", "{out}"], {}),
    # transverse-field Ising rings (project plugin oracle/systems/tfim_ring.cpp)
    ("tfim_s4", "qms_tfim_s4", ["1.3", "40", "1", "4", "{out}", "--seed", "11", "--ene-min", "-8", "--ene-max", "8",
                                "--thermalization", "2"], {"TFIM_J": "1.0", "TFIM_H": "0.8"}),
    ("tfim_s5", "qms_tfim_s5", ["0.7", "20", "1", "4", "{out}", "--seed", "12", "--ene-min", "-10", "--ene-max", "10",
                                "--thermalization", "2"], {"TFIM_J": "1.0", "TFIM_H": "1.2"}),
    ("tfim_s6", "qms_tfim_s6", ["2.0", "12", "1", "5", "{out}", "--seed", "13", "--ene-min", "-9", "--ene-max", "9",
                                "--thermalization", "1"], {"TFIM_J": "1.0", "TFIM_H": "0.5"}),
    # 7-10 spins with the 6-qubit energy register (14-17 qubits); the reference CPU
    # build needs 20 s to 2 min per run, so the runs are short
    ("tfim_s7_e6", "qms_tfim_s7", ["1.1", "12", "1", "6", "{out}", "--seed", "21", "--ene-min", "-14", "--ene-max",
                                   "14", "--thermalization", "0"], {"TFIM_J": "1.0", "TFIM_H": "0.9"}),
    ("tfim_s8_e6", "qms_tfim_s8", ["0.6", "6", "1", "6", "{out}", "--seed", "22", "--ene-min", "-16", "--ene-max",
                                   "16", "--thermalization", "0"], {"TFIM_J": "1.0", "TFIM_H": "1.3"}),
    ("tfim_s9_e6", "qms_tfim_s9", ["1.7", "6", "1", "6", "{out}", "--seed", "23", "--ene-min", "-18", "--ene-max",
                                   "18", "--thermalization", "0"], {"TFIM_J": "1.0", "TFIM_H": "0.6"}),
    ("tfim_s10_e6", "qms_tfim_s10", ["1.0", "3", "1", "6", "{out}", "--seed", "24", "--ene-min", "-20", "--ene-max",
                                     "20", "--thermalization", "0"], {"TFIM_J": "1.0", "TFIM_H": "1.0"}),
]


def build_reference():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "tfim", "port", "gatecount", "-j8"], check=True)


def gate_fixtures():
    blocks = []
    arrays = {}
    meta = []
    with tempfile.TemporaryDirectory() as d:
        for name, seed, n, ng, _ in GATE_CASES:
            lines = circuits.random_script(seed, n, ng, random_init=n <= 8,
                                           dump_every=5 if n <= 8 else 30)
            res = oracle.run_reference(lines, d)
            blocks.append(f"## {name}\n" + "\n".join(lines))
            kinds = []
            for k, (kind, val) in enumerate(res):
                kinds.append(kind)
                if kind == "S":
                    arrays[f"{name}__{k}"] = val
                elif kind in ("M", "P", "N"):
                    arrays[f"{name}__{k}"] = np.array([val], dtype=np.float64)
            meta.append({"name": name, "kinds": "".join(kinds)})
        for name, seed, n, ng in OVERLAP_CASES:
            lines = circuits.random_script(seed, n, ng, overlap="engine", dump_every=6)
            res = oracle.run_reference(lines, d)
            blocks.append(f"## {name}\n" + "\n".join(lines))
            kinds = []
            for k, (kind, val) in enumerate(res):
                kinds.append(kind)
                if kind == "S":
                    arrays[f"{name}__{k}"] = val
                elif kind in ("M", "P", "N"):
                    arrays[f"{name}__{k}"] = np.array([val], dtype=np.float64)
            meta.append({"name": name, "kinds": "".join(kinds)})
        lines = circuits.test_suqa_sequence()
        res = oracle.run_reference(lines, d)
        blocks.append("## test_suqa\n" + "\n".join(lines))
        for k, (kind, val) in enumerate(res):
            arrays[f"test_suqa__{k}"] = val
        meta.append({"name": "test_suqa", "kinds": "".join(k for k, _ in res)})
    with gzip.open(os.path.join(HERE, "gates_scripts.txt.gz"), "wt") as f:
        f.write("\n".join(blocks) + "\n")
    arrays["__meta__"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "gates_results.npz"), **arrays)


def run_fixtures(only=None):
    """Runs the reference drivers of RUNS (or the named subset, merged into the
    existing manifest) and records their output files."""
    rdir = os.path.join(HERE, "runs")
    os.makedirs(rdir, exist_ok=True)
    manifest = {}
    mpath = os.path.join(rdir, "manifest.json")
    if only and os.path.exists(mpath):
        manifest = json.load(open(mpath))
    for name, exe, args, env in RUNS:
        if only and name not in only:
            continue
        out = os.path.join(rdir, f"{name}.txt")
        for p in (out, out + "_revcounts"):
            if os.path.exists(p):
                os.remove(p)
        argv = [os.path.join(REF, exe)] + [a.replace("{out}", out) for a in args]
        e = dict(os.environ)
        e.update(env)
        cp = subprocess.run(argv, env=e, capture_output=True, text=True, check=True)
        acc = re.findall(r"acceptance: *([^\n]*)", cp.stdout)
        manifest[name] = {"driver": exe.split("_tfim")[0], "args": args, "env": env,
                          "acceptance": acc[0].strip() if acc else None,
                          "revcounts": os.path.exists(out + "_revcounts")}
        if os.path.exists(out + "_revcounts"):
            os.replace(out + "_revcounts", os.path.join(rdir, f"{name}_revcounts.txt"))
    with open(os.path.join(rdir, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


# runs repeated with the reference built with -DGATECOUNT: the printed gate-cost tables
GATECOUNT_RUNS = ["qms_c1", "qms_rev", "qsa_c1"]


def gate_count_table(stdout: str) -> str:
    """The 'Gate counts' block the drivers print at suqa::clear()."""
    lines = stdout.splitlines()
    i = lines.index("Gate counts")
    out = []
    for ln in lines[i:]:
        if out and ln == "" and len(out) > 3:
            break
        out.append(ln)
    return "\n".join(out).strip() + "\n"


def gatecount_fixtures():
    rdir = os.path.join(HERE, "runs")
    spec = {name: (exe, args) for name, exe, args, env in RUNS}
    for name in GATECOUNT_RUNS:
        exe, args = spec[name]
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "out.txt")
            argv = [os.path.join(REF, exe + "_gc")] + [a.replace("{out}", out) for a in args]
            cp = subprocess.run(argv, capture_output=True, text=True, check=True)
        with open(os.path.join(rdir, f"{name}_gatecounts.txt"), "w") as f:
            f.write(gate_count_table(cp.stdout))


def pcg_fixture():
    cp = subprocess.run([os.path.join(REF, "pcg_dump")], capture_output=True, text=True, check=True)
    with open(os.path.join(HERE, "pcg32_draws.txt"), "w") as f:
        f.write(cp.stdout)


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--runs":  # regenerate only the named run fixtures
        build_reference()
        run_fixtures(sys.argv[2:])
        sys.exit(0)
    build_reference()
    gate_fixtures()
    run_fixtures()
    gatecount_fixtures()
    pcg_fixture()
    print("fixtures written to", HERE)
