"""Batched Szegedy-walk annealing on the GPU against the oracle walk driver:
the same PCG32 streams give the same restarts, step counts and spin readouts,
and the per-step probability of the zero walk phase agrees to rounding."""
import numpy as np
import pytest

import oracle
import qsa_walk as qw

pytestmark = pytest.mark.gpu


def _walks(n, seed, spins=(2, 7), q=(1, 7), stages=3, per=4, J=(-2, 3), beta=(0.3, 3.0), max_steps=0):
    from suqa_gb300.walk import QsaWalk
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        s = int(rng.integers(*spins))
        out.append(QsaWalk(s, [int(v) for v in rng.integers(J[0], J[1], s)], float(rng.uniform(*beta)), stages, per,
                           int(rng.integers(*q)), 900 + k, max_steps))
    return out


def _oracle(w):
    return qw.run_walk(w.spins, w.J, w.beta, w.stages, w.steps_per_stage, w.phase_qbits, w.seed, w.max_steps,
                       rng=oracle.Pcg32(w.seed))


def _check(runs, walks, tol):
    for r, w in zip(runs, walks):
        o = _oracle(w)
        assert (r.done, r.restarts, r.steps, r.readout) == (bool(o.done), o.restarts, o.steps, o.readout), w
        assert (r.E, r.absM) == (o.E, o.absM)
        assert np.max(np.abs(r.p0 - np.array(o.p0))) < tol, w


def test_fp64_walks_match_the_oracle():
    from suqa_gb300.walk import run_qsa_walks
    walks = _walks(24, 1)
    runs, ms = run_qsa_walks(walks, "f64", trace=True)
    assert ms > 0
    _check(runs, walks, 1e-10)


def test_fp32_walks_match_the_oracle():
    from suqa_gb300.walk import run_qsa_walks
    walks = _walks(24, 2, q=(2, 5))
    runs, _ = run_qsa_walks(walks, "f32", trace=True)
    _check(runs, walks, 2e-5)


def test_capped_and_restarting_walks():
    """Cold rings with a wide walk-phase register restart often; a small cap
    stops them with done = 0 after exactly max_steps steps."""
    from suqa_gb300.walk import run_qsa_walks
    walks = _walks(12, 3, spins=(3, 6), q=(5, 7), stages=4, per=5, beta=(4.0, 8.0), max_steps=9)
    runs, _ = run_qsa_walks(walks, "f64", trace=True)
    _check(runs, walks, 1e-10)
    assert any(not r.done for r in runs) and all(r.steps <= 9 for r in runs)


def test_eight_spin_rings_match_the_oracle():
    from suqa_gb300.walk import run_qsa_walks
    walks = _walks(3, 4, spins=(8, 9), q=(6, 7), stages=1, per=3, J=(-1, 2))
    for w in walks:
        w.J = [v if v != 0 else 1 for v in w.J]
    runs, _ = run_qsa_walks(walks, "f64", trace=True)
    _check(runs, walks, 1e-10)


def test_ten_spin_rings_fp32_follow_fp64():
    """The configured ring length (10 spins, 2^21 amplitudes per walk): FP32
    and FP64 give the same walks, p0 to FP32 rounding."""
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    walks = ising_ring_walks(16, 10, 1.0, 5, 2, 6, seed=7)
    r64, _ = run_qsa_walks(walks, "f64", trace=True)
    r32, _ = run_qsa_walks(walks, "f32", trace=True)
    same = 0
    for a, b in zip(r32, r64):
        assert 0.0 <= b.last_p0 <= 1.0 + 1e-12
        if (a.done, a.restarts, a.steps, a.readout) == (b.done, b.restarts, b.steps, b.readout):
            same += 1
            assert np.max(np.abs(a.p0 - b.p0)) < 1e-4
    assert same >= 14


def test_walk_results_do_not_depend_on_the_batch_split():
    """Walks are independent: each rank's share (shard.partition) reproduces the
    walks of the whole batch, so the sharded sums equal the one-batch sums."""
    from suqa_gb300 import shard
    from suqa_gb300.walk import run_qsa_walks
    walks = _walks(20, 5, spins=(3, 8), q=(3, 7))
    whole, _ = run_qsa_walks(walks, "f32", trace=True)
    keys, acc = shard.walk_sums(walks, whole, lambda w: w.spins)
    tot = np.zeros_like(acc)
    for part in shard.partition(walks, 3, shard.walk_cost):
        sub = [walks[i] for i in part]
        runs, _ = run_qsa_walks(sub, "f32", trace=True)
        for i, r in zip(part, runs):
            a = whole[i]
            assert (r.restarts, r.steps, r.readout) == (a.restarts, a.steps, a.readout)
            assert np.array_equal(r.p0, a.p0)
        k2, a2 = shard.walk_sums(sub, runs, lambda w: w.spins)
        for k, row in zip(k2, a2):
            tot[keys.index(k)] += row
    assert np.allclose(tot, acc, rtol=0, atol=1e-9)


def test_twelve_spin_rings_at_the_size_limit():
    """The largest rings the entry point takes (12 spins, 2^25 amplitudes per
    walk): FP32 and FP64 take the same steps and readouts."""
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    walks = ising_ring_walks(3, 12, 1.0, 2, 2, 4, seed=12)
    r64, _ = run_qsa_walks(walks, "f64", trace=True)
    r32, _ = run_qsa_walks(walks, "f32", trace=True)
    for a, b in zip(r32, r64):
        assert (a.done, a.restarts, a.steps, a.readout) == (b.done, b.restarts, b.steps, b.readout)
        assert np.max(np.abs(a.p0 - b.p0)) < 1e-4
        assert b.done and abs(b.E) <= 12 and 0 <= b.absM <= 12


@pytest.mark.parametrize("precision,tol", [("f64", 1e-9), ("f32", 5e-5)])
def test_orbit_class_algorithm_matches_the_oracle(precision, tol):
    """Algorithm 1 (per orbit class: eigen-decomposition of (W + W^T)/2 and the
    sum of powers of W) gives the oracle's walks."""
    walks = _walks(20, 7, spins=(2, 8), q=(1, 7), J=(-1, 2))
    for w in walks:
        w.J = [v if v != 0 else 1 for v in w.J]
        w.algo = 1
    from suqa_gb300.walk import run_qsa_walks
    runs, _ = run_qsa_walks(walks, precision, trace=True)
    _check(runs, walks, tol)


def test_orbit_class_algorithm_on_ten_spin_rings_matches_iteration():
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    w0 = ising_ring_walks(12, 10, 1.0, 3, 2, 6, seed=9)
    w1 = ising_ring_walks(12, 10, 1.0, 3, 2, 6, seed=9, algo=1)
    for prec, tol in (("f64", 1e-9), ("f32", 1e-4)):
        r0, _ = run_qsa_walks(w0, prec, trace=True)
        r1, _ = run_qsa_walks(w1, prec, trace=True)
        same = 0
        for a, b in zip(r0, r1):
            if (a.done, a.restarts, a.steps, a.readout) == (b.done, b.restarts, b.steps, b.readout):
                same += 1
                assert np.max(np.abs(a.p0 - b.p0)) < tol
        assert same >= (12 if prec == "f64" else 11)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_class_table_matches_per_step_preparation(precision):
    """Algorithm 1 reads the class data from one table per batch (key x stage
    temperature), algorithm 2 prepares them per walk and step: the same
    arithmetic on the same inputs, so the walks agree bit for bit, with mixed
    schedules (beta, stages, walk-phase width) and rings sharing schedules."""
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    mixed = _walks(10, 17, spins=(3, 9), q=(1, 7), J=(-1, 2))
    for w in mixed:
        w.J = [v if v != 0 else 1 for v in w.J]
    rings = ising_ring_walks(6, 10, 1.0, 3, 2, 6, seed=4)
    runs = {}
    for algo in (1, 2):
        for w in mixed + rings:
            w.algo = algo
        runs[algo], _ = run_qsa_walks(mixed + rings, precision, trace=True)
    for a, b in zip(runs[1], runs[2]):
        assert (a.done, a.restarts, a.steps, a.readout, a.last_p0) == (b.done, b.restarts, b.steps, b.readout, b.last_p0)
        assert np.array_equal(a.p0, b.p0)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-9), ("f32", 5e-5)])
def test_orbit_class_algorithm_with_many_classes(precision, tol):
    """5-spin rings with couplings +-1, +-2 have 76-78 classes per move: the
    16-warp class-sorted FP32 pass holds them (up to 85 classes in shared
    memory); with the 8-warp setting (at most 71 classes) FP32 takes the orbit
    pass that reads every class through its own lane.  Both against the oracle."""
    from suqa_gb300 import _lib
    from suqa_gb300.walk import QsaWalk, run_qsa_walks
    rings = [[-2, 1, 1, -2, -2], [-1, -2, -1, -2, 2], [1, 1, -2, -1, -2], [2, -1, -2, -1, 1], [2, 2, -1, 2, -1]]
    walks = [QsaWalk(5, J, 0.5 + 0.3 * k, 3, 3, 1 + k, 700 + k, algo=1) for k, J in enumerate(rings)]
    L = _lib.load()
    try:
        for warps in (16, 8):
            assert L.sq_set_walk_orbit_warps(warps) == 0
            runs, _ = run_qsa_walks(walks, precision, trace=True)
            _check(runs, walks, tol)
    finally:
        L.sq_set_walk_orbit_warps(16)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-9), ("f32", 5e-5)])
def test_orbit_class_keys_with_wide_couplings(precision, tol):
    """Couplings of magnitude 8 use all five bit planes of the register-formed
    class keys (J_b + offset up to 16); few classes, so FP32 takes the
    class-sorted pass.  The walks must still be the oracle's."""
    from suqa_gb300.walk import QsaWalk, run_qsa_walks
    rings = [[8, -8, 8, -8, 8, 8], [-8, -8, 8, 8, -8, 8], [8, 8, 8, 8, 8, 8], [-8, 8, -8, 8, -8, 8]]
    walks = [QsaWalk(6, J, 0.04 + 0.03 * k, 3, 3, 2 + k, 810 + k, algo=1) for k, J in enumerate(rings)]
    runs, _ = run_qsa_walks(walks, precision, trace=True)
    _check(runs, walks, tol)


def test_orbit_class_algorithm_refuses_rings_with_too_many_classes():
    """An 8-spin ring with couplings in -3..3 has 130-338 classes per move, more than
    algorithm 1 holds (96): the call fails with SQ_ERR_UNSUPPORTED and the same
    walk runs with algorithm 0."""
    from suqa_gb300._lib import SqUnsupported
    from suqa_gb300.walk import QsaWalk, run_qsa_walks
    w = QsaWalk(8, [1, 1, 2, 3, -3, -2, 2, 3], 1.0, 2, 2, 3, 5, algo=1)
    with pytest.raises(SqUnsupported, match="orbit classes"):
        run_qsa_walks([w], "f32")
    w.algo = 0
    runs, _ = run_qsa_walks([w], "f64", trace=True)
    _check(runs, [w], 1e-10)


def test_presorted_orbit_pass_is_bit_identical_to_the_sorting_pass():
    """The 16-warp orbit pass with the batch's orbit order table (orbits placed
    by class from a table made once per batch) and without it (a counting sort
    of every chunk at every step): the same places, hence the same sums in the
    same order -- identical walks and identical p0 traces; each against the
    oracle."""
    from suqa_gb300 import _lib
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    L = _lib.load()
    walks = ising_ring_walks(24, 10, 1.0, 3, 2, 6, seed=23, algo=1)
    walks += ising_ring_walks(8, 7, 0.7, 2, 3, 4, seed=5, algo=1)
    out = {}
    try:
        for on in (0, 1):
            assert L.sq_set_walk_presort(on) == 0
            out[on], _ = run_qsa_walks(walks, "f32", trace=True)
    finally:
        L.sq_set_walk_presort(1)
    assert L.sq_set_walk_presort(2) != 0
    for a, b in zip(out[0], out[1]):
        assert (a.done, a.restarts, a.steps, a.readout, a.E, a.absM) == (b.done, b.restarts, b.steps, b.readout,
                                                                         b.E, b.absM)
        assert np.array_equal(a.p0, b.p0)
    _check(out[1][:4], walks[:4], 5e-5)
    _check(out[1][24:26], walks[24:26], 5e-5)


def test_tensor_and_cuda_core_orbit_products_agree():
    """The 16-warp orbit pass with its class products on the tensor cores
    (mma.sync TF32, three-product split) and on the CUDA cores (FP32): the same
    walks (restarts, steps, read-outs) and probabilities to FP32 rounding; the
    tensor-core walks against the oracle."""
    from suqa_gb300 import _lib
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    L = _lib.load()
    walks = ising_ring_walks(24, 10, 1.0, 3, 2, 6, seed=29, algo=1)
    walks += ising_ring_walks(8, 6, 0.8, 2, 3, 5, seed=31, algo=1)
    out = {}
    try:
        for on in (0, 1):
            assert L.sq_set_walk_mma(on) == 0
            out[on], _ = run_qsa_walks(walks, "f32", trace=True)
    finally:
        L.sq_set_walk_mma(1)
    assert L.sq_set_walk_mma(3) != 0
    same = 0
    for a, b in zip(out[0], out[1]):
        if (a.done, a.restarts, a.steps, a.readout) == (b.done, b.restarts, b.steps, b.readout):
            same += 1
            assert np.max(np.abs(a.p0 - b.p0)) < 2e-5
    assert same >= len(walks) - 1
    _check(out[1][:6], walks[:6], 5e-5)
    _check(out[1][24:28], walks[24:28], 5e-5)


def test_sixteen_and_eight_warp_orbit_passes_agree():
    """The class-sorted FP32 orbit pass with 16 warps per CTA (CTA-level class
    sums, end-of-range sums added in warp order) and with 8 warps (per-warp class
    sums): the same walks (restarts, steps, read-outs) and probabilities to FP32
    rounding; each against the oracle."""
    from suqa_gb300 import _lib
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    L = _lib.load()
    walks = ising_ring_walks(24, 10, 1.0, 3, 2, 6, seed=21, algo=1)
    out = {}
    try:
        for warps in (8, 16):
            assert L.sq_set_walk_orbit_warps(warps) == 0
            out[warps], _ = run_qsa_walks(walks, "f32", trace=True)
    finally:
        L.sq_set_walk_orbit_warps(16)
    same = 0
    for a, b in zip(out[8], out[16]):
        if (a.done, a.restarts, a.steps, a.readout) == (b.done, b.restarts, b.steps, b.readout):
            same += 1
            assert np.max(np.abs(a.p0 - b.p0)) < 2e-5
    assert same >= 23
    _check(out[16][:6], walks[:6], 5e-5)
