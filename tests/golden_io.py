"""Loader for the committed golden fixtures (tests/golden/)."""
from __future__ import annotations

import gzip
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gate_cases():
    """Yields (name, script lines, expected results) with results in dumper order."""
    text = gzip.open(os.path.join(GOLDEN, "gates_scripts.txt.gz"), "rt").read()
    blocks = {}
    for blk in text.split("## ")[1:]:
        name, _, body = blk.partition("\n")
        blocks[name] = [l for l in body.split("\n") if l]
    npz = np.load(os.path.join(GOLDEN, "gates_results.npz"))
    meta = json.loads(bytes(npz["__meta__"]).decode())
    for m in meta:
        res = []
        for k, kind in enumerate(m["kinds"]):
            key = f"{m['name']}__{k}"
            if kind == "S":
                res.append(("S", npz[key]))
            elif kind == "M":
                res.append(("M", int(npz[key][0])))
            elif kind in ("P", "N"):
                res.append((kind, float(npz[key][0])))
            else:
                res.append((kind, None))
        yield m["name"], blocks[m["name"]], res


def run_manifest():
    with open(os.path.join(GOLDEN, "runs", "manifest.json")) as f:
        return json.load(f)


def run_output(name):
    with open(os.path.join(GOLDEN, "runs", f"{name}.txt")) as f:
        return f.read()


def compare_results(got, want, *, rtol=1e-12, exact=False):
    """Compare two result lists.  States: max |a-b| <= rtol * max|b| (amplitude
    error relative to the state's largest amplitude), or bit-exact when exact.
    Measured bits must be identical; probabilities and norms within rtol."""
    assert len(got) == len(want), (len(got), len(want))
    flips = 0
    worst = 0.0
    for (kg, vg), (kw, vw) in zip(got, want):
        assert kg == kw, (kg, kw)
        if kg == "S":
            if exact:
                assert np.array_equal(vg, vw, equal_nan=True)
            elif np.isnan(vw).any():
                # a script that zeroed the state (H under an overlapping control)
                # renormalises 0/0; both sides must agree on where that happened
                assert np.array_equal(np.isnan(vg), np.isnan(vw))
            else:
                scale = max(np.max(np.abs(vw)), 1e-300)
                err = float(np.max(np.abs(vg - vw)) / scale)
                worst = max(worst, err)
                assert err <= rtol, err
        elif kg == "M":
            if vg != vw:
                flips += 1
        elif kg in ("P", "N"):
            if vw != vw:
                assert vg != vg
            elif exact:
                assert vg == vw
            else:
                assert abs(vg - vw) <= rtol * max(1.0, abs(vw)), (vg, vw)
    assert flips == 0, f"{flips} measured bits differ"
    return worst
