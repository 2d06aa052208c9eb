"""The premises of the orbit-class walk algorithm, checked on the CPU against the
oracle's walk operator W (qsa_walk.CompressedWalk):

* the orbits of a move C, enumerated as the walk kernels enumerate them, split
  the compressed state psi[acc][d][x] into disjoint sets of 16 amplitudes (8 for
  d' = 0), and W maps each set to itself;
* two orbits with the same key (the energy differences at their four a = 0
  positions) carry the same 16 x 16 block of W;
* with V the eigenvectors of A = (B + B^T)/2 of an orbit's block B,
  <psi, W^k psi> = sum_i (v_i^T psi)^2 v_i^T B^k v_i summed over orbits (weight
  1/2 for the 8-amplitude orbits, held duplicated), and
  sum_{k<L} W^k = prod_{j<q} (I + W^(2^j));
* the energy differences of the key follow from the ring's couplings alone:
  E(x ^ d) - E(x) = 2 J(m) - 4 J(m & (x ^ rot x)), m = d ^ rot d.
"""
import numpy as np
import pytest

import qsa_walk as qw


def ins0(p, b):
    return ((p >> b) << (b + 1)) | (p & ((1 << b) - 1))


def orbits(s, C):
    """(dp, x0, single) for every orbit, in the kernels' order (orbit_decode)."""
    out = [(0, ins0(o, C), True) for o in range(1 << (s - 1))]
    for o2 in range(((1 << (s - 1)) - 1) << (s - 2)):
        di, ri = 1 + (o2 >> (s - 2)), o2 & ((1 << (s - 2)) - 1)
        dp = ins0(di, C)
        p = (dp & -dp).bit_length() - 1
        out.append((dp, ins0(ins0(ri, min(p, C)), max(p, C)), False))
    return out


def slot_index(s, C, dp, x0):
    """Flat index of psi[acc][d][x] for the 16 slots (a, b, c, acc), slot = 8a + 4b + 2c + acc."""
    N, eC = 1 << s, 1 << C
    idx = []
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                for acc in (0, 1):
                    x = x0 ^ (dp if a else 0) ^ (eC if b else 0)
                    d = dp ^ (eC if c else 0)
                    idx.append(acc * N * N + d * N + x)
    return np.array(idx)


def orbit_key(E, s, C, dp, x0):
    eC = 1 << C
    key = []
    for j in range(4):
        x = x0 ^ (eC if j & 1 else 0)
        d = dp ^ (eC if j & 2 else 0)
        key.append(int(E[x ^ d] - E[x]))
    return tuple(key)


def walk_matrix(cw, C, beta):
    e, r = cw.coeffs(beta)
    n = 2 * cw.N * cw.N
    W = np.empty((n, n))
    for j in range(n):
        u = np.zeros(n)
        u[j] = 1.0
        W[:, j] = cw.apply(u.reshape(2, cw.N, cw.N), C, e, r).ravel()
    return W


CASES = [(4, [1, -1, 1, 1], 0.7, 2), (4, [2, -1, 1, -2], 1.3, 0), (5, [1, 1, -1, 1, -1], 0.9, 3),
         (5, [-2, 1, 2, -1, 1], 2.1, 4)]


@pytest.fixture(scope="module", params=CASES, ids=lambda c: f"s{c[0]}C{c[3]}")
def case(request):
    s, J, beta, C = request.param
    cw = qw.CompressedWalk(s, J)
    return s, J, beta, C, cw, walk_matrix(cw, C, beta)


def test_orbits_partition_the_state_and_w_keeps_each_orbit(case):
    s, J, beta, C, cw, W = case
    n = W.shape[0]
    seen = np.zeros(n, dtype=int)
    for dp, x0, single in orbits(s, C):
        idx = slot_index(s, C, dp, x0)
        own = np.unique(idx)
        assert len(own) == (8 if single else 16)
        seen[own] += 1
        outside = np.setdiff1d(np.arange(n), own)
        assert np.max(np.abs(W[np.ix_(outside, own)])) == 0.0
    assert np.all(seen == 1)
    assert np.allclose(W.T @ W, np.eye(n), atol=1e-13)


def test_orbits_with_one_key_share_one_block(case):
    s, J, beta, C, cw, W = case
    blocks = {}
    for dp, x0, single in orbits(s, C):
        if single:
            continue
        idx = slot_index(s, C, dp, x0)
        B = W[np.ix_(idx, idx)]
        key = orbit_key(cw.E, s, C, dp, x0)
        if key in blocks:
            assert np.array_equal(blocks[key], B), key
        else:
            blocks[key] = B
    assert len(blocks) < len(orbits(s, C))


def test_eigen_decomposition_and_sum_of_powers_reproduce_the_walk_step(case):
    s, J, beta, C, cw, W = case
    rng = np.random.default_rng(s * 10 + C)
    n = W.shape[0]
    psi = rng.standard_normal(n)
    q = 3
    L = 1 << q
    Wk = [np.eye(n)]
    for _ in range(L):
        Wk.append(W @ Wk[-1])
    g_ref = np.array([psi @ Wk[k] @ psi for k in range(L)])
    S_ref = sum(Wk[k] for k in range(L)) @ psi
    g = np.zeros(L)
    S = np.zeros(n)
    for dp, x0, single in orbits(s, C):
        idx = slot_index(s, C, dp, x0)
        if single:
            # 8 distinct amplitudes held twice in the 16 slots: any orthogonal block
            # that maps [v, v] to [W v, W v] serves, its class sums weighted by 1/2
            W8 = W[np.ix_(idx[:8], idx[:8])]
            B = np.block([[W8, np.zeros((8, 8))], [np.zeros((8, 8)), W8]])
        else:
            B = W[np.ix_(idx, idx)]
        v = psi[idx]
        wgt = 0.5 if single else 1.0
        A = 0.5 * (B + B.T)
        _, V = np.linalg.eigh(A)
        y = V.T @ v
        Bk = np.eye(16)
        for k in range(L):
            g[k] += wgt * np.sum(y * y * np.einsum("ji,jk,ki->i", V, Bk, V))
            Bk = B @ Bk
        Q = np.eye(16) + B
        P = B.copy()
        for _ in range(1, q):
            P = P @ P
            Q = Q + Q @ P
        assert np.allclose(Q, sum(np.linalg.matrix_power(B, k) for k in range(L)), atol=1e-12)
        Sv = Q @ v
        S[idx[:8] if single else idx] = Sv[:8] if single else Sv
    assert np.allclose(g, g_ref, rtol=1e-12, atol=1e-12)
    assert np.allclose(S, S_ref, atol=1e-12)


def test_key_energy_differences_from_the_couplings():
    rng = np.random.default_rng(11)
    for _ in range(200):
        s = int(rng.integers(2, 13))
        J = [int(v) for v in rng.integers(-8, 9, s)]
        E = qw.ring_energies(s, J)
        off = max(0, -min(J))
        vals = [j + off for j in J]
        planes = [sum(((vals[b] >> k) & 1) << b for b in range(s)) for k in range(max(vals).bit_length())]
        smask = (1 << s) - 1

        def bond_sum(m):
            return sum(bin(m & pl).count("1") << k for k, pl in enumerate(planes)) - off * bin(m).count("1")

        def rot(v):
            return ((v >> 1) | (v << (s - 1))) & smask

        for _ in range(40):
            x, d = int(rng.integers(0, 1 << s)), int(rng.integers(0, 1 << s))
            m = d ^ rot(d)
            assert 2 * bond_sum(m) - 4 * bond_sum(m & (x ^ rot(x))) == E[x ^ d] - E[x]
