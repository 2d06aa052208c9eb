"""Batched QMS chains on the device against the reference CPU qms driver built
with the same transverse-field Ising plugin (fixtures tests/golden/runs/tfim_*):
the written (E, A) rows must be identical, in FP64."""
import re

import numpy as np
import pytest

import golden_io

pytestmark = pytest.mark.gpu


def chain_from_manifest(name):
    man = golden_io.run_manifest()[name]
    a = man["args"]
    spins = int(re.match(r"tfim_s(\d+)", name).group(1))
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


@pytest.mark.parametrize("name", ["tfim_s4", "tfim_s5", "tfim_s6", "tfim_s7_e6", "tfim_s8_e6", "tfim_s9_e6",
                                  "tfim_s10_e6"])
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


def _golden_rows(name):
    wE, wA = parse_rows(golden_io.run_output(name))
    return wE, wA


@pytest.mark.parametrize("name", ["tfim_s4", "tfim_s6"])
@pytest.mark.parametrize("layout", ["cluster", "global", "threads128"])
def test_golden_chains_in_every_storage_mode(name, layout):
    """The reference rows come out identical whether a chain's state sits in one
    CTA's shared memory, is spread over a cluster's shared memory, or is worked
    on in global memory by a cluster, and at any CTA size."""
    from suqa_gb300.batch import Batch
    c = chain_from_manifest(name)
    kw = {"cluster": dict(cta_qubits=c.nqubits - 2), "global": dict(global_qubits=1),
          "threads128": dict(threads=128)}[layout]
    b = Batch([c], "f64", **kw)
    plan = b.plan()
    want_mode = {"cluster": "cluster-shared", "global": "cluster-global", "threads128": "shared"}[layout]
    assert plan[0]["mode"] == want_mode, plan
    b.run(c.steps)
    E, A = b.results()[0].reference_rows(c.steps)
    b.close()
    wE, wA = _golden_rows(name)
    assert fmt(E) == wE and fmt(A) == wA


def _mixed(n, steps, seed=5, spins=(3, 7), ene=(3, 5)):
    from suqa_gb300.batch import TfimChain
    rng = np.random.default_rng(seed)
    return [TfimChain(spins=int(rng.integers(*spins)), ene_qbits=int(rng.integers(*ene)), steps=steps,
                      beta=float(rng.uniform(0.2, 2.0)), h=float(rng.uniform(0.5, 1.5)), thermalization=1,
                      seed=500 + i) for i in range(n)]


def _same(r1, r2):
    for a, b in zip(r1, r2):
        assert (a.accepted, a.failures, a.phase_estimations) == (b.accepted, b.failures, b.phase_estimations)
        assert np.array_equal(a.E, b.E) and np.array_equal(a.A, b.A) and np.array_equal(a.step, b.step)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_segments_graph_checkpoint_resume(precision):
    """A batch advanced in graph-replayed segments, checkpointed half-way and
    resumed in a fresh batch gives exactly the one-shot results and states."""
    from suqa_gb300.batch import Batch, run_tfim_batch
    chains = _mixed(40, 9)
    ref, _ = run_tfim_batch(chains, precision)
    b = Batch(chains, precision, segment_steps=2, use_graph=True)
    b.run(4)
    assert (b.progress() == 4).all()
    blob = b.checkpoint()
    b.run(5)
    seg = b.results()
    _same(ref, seg)
    b2 = Batch(chains, precision, segment_steps=3, use_graph=True)
    b2.restore(blob)
    assert (b2.progress() == 4).all()
    b2.run(100)  # runs to the end of every chain
    assert (b2.progress() == 9).all()
    _same(ref, b2.results())
    for i in (0, 17, 39):
        assert np.array_equal(b.state(i), b2.state(i))
    with pytest.raises(Exception):
        Batch(chains[:-1], precision).restore(blob)
    b.close()
    b2.close()


def test_autotuned_batch_same_results():
    from suqa_gb300.batch import Batch, run_tfim_batch
    chains = _mixed(64, 4, seed=9, spins=(4, 9), ene=(4, 6))
    ref, _ = run_tfim_batch(chains, "f32")
    b = Batch(chains, "f32", autotune=True)
    plan = b.plan()
    assert all(p["threads"] in (128, 256, 512) and p["probe_ms"] > 0 for p in plan), plan
    b.run(4)
    _same(ref, b.results())
    b.close()


@pytest.mark.parametrize("layout", ["cluster", "global"])
def test_long_ring_matches_host_driven_driver(layout, tmp_path):
    """12-spin rings (longer than a warp-group chunk of 10 spins: the extra spin
    bits rotate between warps through shared memory) match the host-driven
    drop-in driver; FP64, 17 qubits."""
    import os
    import subprocess
    from suqa_gb300.batch import Batch, TfimChain
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spins, ene, steps = 12, 4, 2
    c = TfimChain(spins=spins, ene_qbits=ene, steps=steps, beta=0.9, h=1.1, thermalization=0, seed=31,
                  ene_min=-2.0 * spins, ene_max=2.0 * spins)
    kw = dict(global_qubits=17) if layout == "global" else {}
    b = Batch([c], "f64", **kw)
    assert b.plan()[0]["mode"] == ("cluster-global" if layout == "global" else "cluster-shared")
    b.run(steps)
    run = b.results()[0]
    b.close()
    out = str(tmp_path / "drv.txt")
    env = dict(os.environ, TFIM_J="1.0", TFIM_H="1.1")
    cp = subprocess.run([os.path.join(root, "suqa_gb300", "_build", f"qms_tfim_s{spins}"), "0.9", str(steps), "1",
                         str(ene), out, "--seed", "31", "--ene-min", str(-2.0 * spins), "--ene-max", str(2.0 * spins),
                         "--thermalization", "0"], env=env, capture_output=True, text=True, timeout=1200)
    assert cp.returncode == 0, cp.stderr[-2000:]
    wE, wA = parse_rows(open(out).read())
    E, A = run.reference_rows(steps)
    assert fmt(E) == wE and fmt(A) == wA


def test_wide_fp32_chains_in_global_memory_match_fp64():
    """19-qubit chains (12 spins, 6 energy qubits: the warm-start evaluation
    width) run from L2-resident global memory; FP32 takes the same path as FP64."""
    from suqa_gb300.batch import Batch, TfimChain
    chains = [TfimChain(spins=12, ene_qbits=6, steps=2, beta=b_, h=h_, thermalization=0, seed=70 + i)
              for i, (b_, h_) in enumerate([(0.5, 0.7), (1.5, 1.2), (1.0, 1.0)])]
    res = {}
    for p in ("f32", "f64"):
        b = Batch(chains, p)
        assert b.plan()[0]["mode"] == "cluster-global"
        b.run(2)
        res[p] = b.results()
        st = b.state(0)
        assert abs(np.vdot(st, st).real - 1.0) < 1e-4
        b.close()
    _same(res["f32"], res["f64"])


def test_sharded_batches_sum_to_the_whole():
    """Each rank's share run as its own batch (here one after the other on one
    GPU) gives per-group sums that add up to the unsharded batch's, to the bit."""
    from suqa_gb300 import shard
    from suqa_gb300.batch import Batch
    chains = _mixed(30, 5, seed=12)
    key = lambda c: c.spins
    b = Batch(chains, "f32")
    b.run(5)
    keys, whole = shard.group_sums(chains, b.results(), key)
    b.close()
    acc = np.zeros_like(whole)
    pos = {k: i for i, k in enumerate(keys)}
    for part in shard.partition(chains, 3):
        sub = [chains[i] for i in part]
        bs = Batch(sub, "f32")
        bs.run(5)
        k2, a2 = shard.group_sums(sub, bs.results(), key)
        bs.close()
        for k, row in zip(k2, a2):
            acc[pos[k]] += row
    assert np.allclose(acc, whole, rtol=1e-15, atol=0)
    assert shard.run_sharded(chains, "f32", key=key, rank=0, world=1) == shard.averages(keys, whole)


def test_uneven_lengths_and_fp64_autotune():
    """Chains of different lengths (including zero steps) in one resumable FP64
    batch with autotuned CTA sizes: every chain stops at its own length and the
    results equal the one-shot run."""
    from suqa_gb300.batch import Batch, TfimChain, run_tfim_batch
    chains = _mixed(20, 6, seed=21)
    for i, c in enumerate(chains):
        c.steps = (0, 3, 7)[i % 3]
    ref, _ = run_tfim_batch(chains, "f64")
    b = Batch(chains, "f64", autotune=True, segment_steps=2, use_graph=True)
    assert all(p["threads"] in (128, 256) for p in b.plan())
    b.run(3)
    assert list(b.progress()) == [min(c.steps, 3) for c in chains]
    b.run(10)
    assert list(b.progress()) == [c.steps for c in chains]
    _same(ref, b.results())
    for i, c in enumerate(chains):
        if c.steps == 0:
            with pytest.raises(Exception):
                b.state(i)  # a chain that never ran has no state yet
    b.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_reference_chains_of_every_ring_length_in_one_batch(precision):
    """The seven reference runs (rings of 4-10 spins, energy registers of 4-6
    qubits: 9 to 17 qubits, every storage mode) as one batch: each chain writes
    the reference's rows.  FP32 must reproduce the same rows too: every
    measurement of these runs has a probability margin far above FP32 rounding."""
    from suqa_gb300.batch import run_tfim_batch
    names = ["tfim_s4", "tfim_s5", "tfim_s6", "tfim_s7_e6", "tfim_s8_e6", "tfim_s9_e6", "tfim_s10_e6"]
    chains = [chain_from_manifest(n) for n in names]
    runs, _ = run_tfim_batch(chains, precision)
    for name, c, r in zip(names, chains, runs):
        E, A = r.reference_rows(c.steps)
        wE, wA = _golden_rows(name)
        if precision == "f64":
            assert fmt(E) == wE and fmt(A) == wA, name
        else:
            # FP32 energies come from the same integer register read-outs; the
            # observable is an average of measured spins: identical when every
            # outcome is
            assert [float(x) for x in wE] == [float(x) for x in fmt(E)], name
            assert [float(x) for x in wA] == [float(x) for x in fmt(A)], name
