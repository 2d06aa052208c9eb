"""The synthetic workloads (suqa_gb300.workloads), host side: determinism, the
benchmark circuit's gate mix and the single-kind circuits of the instruction
counts."""
from suqa_gb300.workloads import KINDS, algorithmic_bytes, random_circuit, single_kind_circuit


def test_random_circuit_is_deterministic_and_well_formed():
    a = random_circuit(28, 1000, seed=7)
    assert a == random_circuit(28, 1000, seed=7)
    gates = [g for g in a if g[0] != "measure"]
    assert len(gates) == 1000 and sum(1 for g in a if g[0] == "measure") == 10
    for g in gates:
        qs = []
        if g[0] in ("x", "h", "u1"):
            qs = [g[1]]
        elif g[0] == "cx":
            qs = [g[1], g[2]]
        elif g[0] == "mcx":
            qs = list(g[1]) + [g[2]]
            assert 2 <= len(g[1]) <= 4
        elif g[0] == "ptp":
            qs = list(g[1])
            assert 2 <= len(qs) <= 6 and all(p in (1, 2, 3) for p in g[2])
        assert len(set(qs)) == len(qs) and all(0 <= q < 28 for q in qs)
    assert {g[0] for g in gates} == set(KINDS)


def test_single_kind_circuits():
    for kind in KINDS:
        c = single_kind_circuit(22, kind, 60)
        assert c == single_kind_circuit(22, kind, 60)
        assert c[:22] == [("h", q) for q in range(22)]
        assert len(c) == 82 and all(g[0] == kind for g in c[22:])
    assert single_kind_circuit(22, "h", 0) == [("h", q) for q in range(22)]


def test_algorithmic_bytes_per_gate():
    n, B = 10, 16
    N = 1 << n
    assert algorithmic_bytes([("h", 0)], n, B) == 2 * B * N
    assert algorithmic_bytes([("u1", 0, 0.1)], n, B) == B * N
    assert algorithmic_bytes([("mcx", [0, 1, 2], 3)], n, B) == 2 * B * N // 8
