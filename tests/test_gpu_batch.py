"""Batched QMS chains on the device against the reference CPU qms driver built
with the same transverse-field Ising plugin (fixtures tests/golden/runs/tfim_*):
the written (E, A) rows must be identical, in FP64."""
import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu


def chain_from_manifest(name):
    man = golden_io.run_manifest()[name]
    a = man["args"]
    spins = int(name.split("_s")[1])
    kv = {a[i]: a[i + 1] for i in range(5, len(a) - 1) if a[i].startswith("--")}
    from suqa_gb300.batch import TfimChain
    return TfimChain(spins=spins, ene_qbits=int(a[3]), steps=int(a[1]), beta=float(a[0]),
                     h=float(man["env"]["TFIM_H"]), J=float(man["env"]["TFIM_J"]),
                     ene_min=float(kv["--ene-min"]), ene_max=float(kv["--ene-max"]),
                     thermalization=int(kv.get("--thermalization", 100)), reset_each=int(a[2]),
                     seed=int(kv["--seed"]))


def parse_rows(text):
    rows = [l.split() for l in text.splitlines() if l and not l.startswith("#")]
    return [r[0] for r in rows], [r[1] for r in rows]


def fmt(xs):
    # the reference driver writes "%.16lg"
    return ["%.16g" % x for x in xs]


@pytest.mark.parametrize("name", ["tfim_s4", "tfim_s5", "tfim_s6"])
def test_batched_chain_matches_reference_run(name):
    from suqa_gb300.batch import run_tfim_batch
    c = chain_from_manifest(name)
    runs, ms = run_tfim_batch([c], "f64")
    E, A = runs[0].reference_rows(c.steps)
    wE, wA = parse_rows(golden_io.run_output(name))
    assert fmt(E) == wE
    assert fmt(A) == wA


def test_batch_of_mixed_chains_each_matches_its_single_run():
    """Chains run together (different widths, interleaved on the grid) give the
    same results as run alone: no cross-talk between CTAs."""
    from suqa_gb300.batch import TfimChain, run_tfim_batch
    rng = np.random.default_rng(3)
    chains = [TfimChain(spins=int(rng.integers(3, 7)), ene_qbits=int(rng.integers(3, 5)), steps=12,
                        beta=float(rng.uniform(0.2, 2.0)), h=float(rng.uniform(0.5, 1.5)), thermalization=1,
                        seed=100 + i) for i in range(24)]
    together, _ = run_tfim_batch(chains, "f64")
    for i in (0, 7, 23):
        alone, _ = run_tfim_batch([chains[i]], "f64")
        assert alone[0].accepted == together[i].accepted
        assert np.array_equal(alone[0].E, together[i].E) and np.array_equal(alone[0].A, together[i].A)


@pytest.mark.parametrize("spins,ene,steps", [(8, 5, 6), (10, 5, 3)])
def test_cluster_chains_match_host_driven_driver(spins, ene, steps, tmp_path):
    """Chains wider than one CTA's shared memory (14 and 16 qubits in FP64) run on
    a 2- and 8-CTA cluster; their rows equal those of the host-driven drop-in
    driver (libsq state API) for the same chain."""
    import os
    import subprocess
    from suqa_gb300.batch import TfimChain, run_tfim_batch
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    c = TfimChain(spins=spins, ene_qbits=ene, steps=steps, beta=1.1, h=0.9, thermalization=0, seed=77,
                  ene_min=-2.0 * spins, ene_max=2.0 * spins)
    runs, _ = run_tfim_batch([c], "f64")
    out = str(tmp_path / "drv.txt")
    env = dict(os.environ, TFIM_J="1.0", TFIM_H="0.9")
    cp = subprocess.run([os.path.join(root, "suqa_gb300", "_build", f"qms_tfim_s{spins}"), "1.1", str(steps), "1",
                         str(ene), out, "--seed", "77", "--ene-min", str(-2.0 * spins), "--ene-max", str(2.0 * spins),
                         "--thermalization", "0"], env=env, capture_output=True, text=True, timeout=1200)
    assert cp.returncode == 0, cp.stderr[-2000:]
    wE, wA = parse_rows(open(out).read())
    E, A = runs[0].reference_rows(steps)
    assert fmt(E) == wE and fmt(A) == wA
