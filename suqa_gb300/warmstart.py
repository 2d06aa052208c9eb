"""Learned warm start for QMS chains of transverse-field Ising rings.

A small network (inputs: spin count, J, h, beta; 3 hidden layers of 128 GELU
units; outputs: one RY angle per spin, up to 12) is trained on the GPU by the
libsq kernels (sq_mlp_*) on data produced by plain cold-start chains, and its
angles prepare the chains' initial product state RY(theta_i)|0> in place of
|0...0>.  The Metropolis steps themselves are unchanged; the cold start stays
the fallback and the judge of the thermal averages.

Training target: the chains' equilibrium energy E of a parameter set is turned
into the angle of the product state with that energy,
    E(theta) = -J s cos(theta)^2 - h s sin(theta)   (all spins at theta),
solved on the branch theta in [-pi/2, theta_min] that runs from E = +h s down to
the product-state minimum (bisection; energies outside the range are clamped).
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import _lib
from ._lib import check

MAX_SPINS = 12


def features(spins, J, h, beta):
    return np.array([spins / 12.0, J, h, beta], dtype=np.float32)


def product_energy(theta, spins, J, h):
    return -J * spins * math.cos(theta) ** 2 - h * spins * math.sin(theta)


def angle_for_energy(E, spins, J, h):
    """Product-state angle whose energy is E (see the module docstring)."""
    # minimum of E(theta) on [-pi/2, pi/2]: sin(theta*) = h / (2J) if h < 2J else pi/2
    tmin = math.asin(min(1.0, h / (2.0 * J))) if J > 0 else math.pi / 2
    lo, hi = -math.pi / 2, tmin  # E decreases from +h s at lo to its minimum at hi
    if E >= product_energy(lo, spins, J, h):
        return lo
    if E <= product_energy(hi, spins, J, h):
        return hi
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        if product_energy(mid, spins, J, h) > E:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


class WarmStartNet:
    def __init__(self, hidden=128, layers=3, seed=1):
        self.L = _lib.load()
        h = C.c_void_p()
        check(self.L.sq_mlp_create(C.byref(h), 4, hidden, layers, MAX_SPINS, seed))
        self.h = h
        n = C.c_uint32()
        check(self.L.sq_mlp_num_params(self.h, C.byref(n)))
        self.nparams = n.value
        self.dims = [4] + [hidden] * layers + [MAX_SPINS]

    def close(self):
        if getattr(self, "h", None):
            self.L.sq_mlp_destroy(self.h)
            self.h = None

    __del__ = close

    def params(self):
        p = np.empty(self.nparams, dtype=np.float32)
        check(self.L.sq_mlp_get_params(self.h, p.ctypes.data_as(C.c_void_p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self.L.sq_mlp_set_params(self.h, p.ctypes.data_as(C.c_void_p)))

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((x.shape[0], MAX_SPINS), dtype=np.float32)
        check(self.L.sq_mlp_forward(self.h, x.ctypes.data_as(C.c_void_p), x.shape[0], y.ctypes.data_as(C.c_void_p)))
        return y

    def gradients(self, x, t, mask=None):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_float()
        check(self.L.sq_mlp_gradients(self.h, x.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p),
                                      None if m is None else m.ctypes.data_as(C.c_void_p), x.shape[0],
                                      g.ctypes.data_as(C.c_void_p), C.byref(loss)))
        return g, loss.value

    def train_step(self, x, t, mask=None, lr=1e-3):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        loss = C.c_float()
        check(self.L.sq_mlp_train_step(self.h, x.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p),
                                       None if m is None else m.ctypes.data_as(C.c_void_p), x.shape[0], lr,
                                       C.byref(loss)))
        return loss.value

    def fit(self, x, t, mask, iters=2000, batch=256, lr=2e-3, seed=0):
        rng = np.random.default_rng(seed)
        losses = []
        for it in range(iters):
            idx = rng.integers(0, x.shape[0], size=min(batch, x.shape[0]))
            losses.append(self.train_step(x[idx], t[idx], mask[idx], lr))
        return losses

    def angles(self, spins, J, h, beta):
        y = self.forward(features(spins, J, h, beta)[None, :])[0]
        return [float(a) for a in y[:spins]]


def training_set(chains, runs, burn_in):
    """(x, target angles, mask) from plain chains: the mean energy of each chain's
    samples after burn_in steps gives its parameter set's target angle."""
    xs, ts, ms = [], [], []
    for c, r in zip(chains, runs):
        keep = r.step >= burn_in
        if not np.any(keep):
            continue
        E = float(np.mean(r.E[keep]))
        th = angle_for_energy(E, c.spins, c.J, c.h)
        xs.append(features(c.spins, c.J, c.h, c.beta))
        t = np.zeros(MAX_SPINS, np.float32)
        m = np.zeros(MAX_SPINS, np.float32)
        t[:c.spins] = th
        m[:c.spins] = 1.0
        ts.append(t)
        ms.append(m)
    return np.array(xs), np.array(ts), np.array(ms)


def spin_bloch(psi, spins):
    """Per-spin <X_i> and bond <Z_i Z_{i+1}> of a chain state (spins on the low
    qubits, the energy and acceptance registers above them, traced out)."""
    S = 1 << spins
    amp = np.asarray(psi).reshape(-1, S)  # [higher registers][spin configuration]
    pz = np.sum(np.abs(amp) ** 2, axis=0)
    x = np.arange(S)
    bits = (x[:, None] >> np.arange(spins)[None, :]) & 1
    z = 1.0 - 2.0 * bits  # [config][spin]
    zz = np.array([float(np.dot(pz, z[:, i] * z[:, (i + 1) % spins])) for i in range(spins)])
    X = np.zeros(spins)
    for i in range(spins):
        low = x[(x >> i) & 1 == 0]
        X[i] = 2.0 * float(np.real(np.sum(np.conj(amp[:, low]) * amp[:, low | (1 << i)])))
    return X, zz


def bloch_targets(points, ene_qbits, chains_per_point, burn, samples, every, precision="f32", seed=7):
    """Warm-start targets from the plain chains' equilibrium states: for every
    parameter point (spins, J, h, beta), cold chains run `burn` steps, then their
    states are read `samples` times, `every` steps apart.  Each state's per-spin
    Bloch data give the target angle of a product state RY(theta)|0>, whose Bloch
    vector is (sin theta, 0, cos theta): theta_i = atan2(<X_i>, sqrt(<Z_i Z_{i+1}>)).
    <Z_i> itself vanishes in the chains' states (they are parity eigenstates of the
    ring), so the symmetry-broken magnitude sqrt(<Z_i Z_{i+1}>) stands for it; the
    angle then reproduces the field term sin theta = <X> and the bond term
    cos^2 theta = <ZZ> of the equilibrium state in their ratio.  Returns the
    training rows (one per point, angles averaged over its chains and samples) and
    a summary per point."""
    from .batch import Batch, TfimChain
    chains, owner = [], []
    for pi, (sp, J, h, beta) in enumerate(points):
        for k in range(chains_per_point):
            chains.append(TfimChain(spins=sp, ene_qbits=ene_qbits, steps=burn + samples * every, beta=beta, h=h, J=J,
                                    thermalization=0, seed=seed * 100_000 + 1000 * pi + k))
            owner.append(pi)
    b = Batch(chains, precision, segment_steps=0, use_graph=False)
    acc = [[] for _ in points]
    b.run(burn)
    for _ in range(samples):
        for ci, c in enumerate(chains):
            X, zz = spin_bloch(b.state(ci), c.spins)
            acc[owner[ci]].append(np.arctan2(X, np.sqrt(np.clip(zz, 0.0, None))))
        b.run(every)
    b.close()
    xs, ts, ms, info = [], [], [], []
    for pi, (sp, J, h, beta) in enumerate(points):
        th = np.mean(np.array(acc[pi]), axis=0)
        t = np.zeros(MAX_SPINS, np.float32)
        m = np.zeros(MAX_SPINS, np.float32)
        t[:sp] = th
        m[:sp] = 1.0
        xs.append(features(sp, J, h, beta))
        ts.append(t)
        ms.append(m)
        info.append({"spins": sp, "J": J, "h": h, "beta": beta, "theta_mean": float(np.mean(th)),
                     "samples": len(acc[pi])})
    return np.array(xs), np.array(ts), np.array(ms), info


def scan_targets(points, ene_qbits, thetas, warm_chains, warm_steps, cold_chains, cold_steps, precision="f32",
                 seed=7):
    """Warm-start targets from plain chains by an angle scan.  For every
    parameter point (spins, J, h, beta): cold-started chains give the long-run
    mean energy (the mean over the second half of cold_steps), and chains started
    from RY(theta) on every spin, for each theta of the grid, give their mean
    energy over their first warm_steps steps; the target angle is where that
    early mean meets the cold long-run mean (linear interpolation between grid
    angles where the difference changes sign, else the closest grid angle).
    Every chain is a plain QMS chain (the Metropolis steps are untouched), so the
    targets come from chains the plain method generates.  Returns (x, t, mask,
    details)."""
    from .batch import TfimChain, run_tfim_batch
    chains = []
    for pi, (sp, J, h, beta) in enumerate(points):
        base = dict(spins=sp, ene_qbits=ene_qbits, beta=beta, h=h, J=J, thermalization=0)
        chains += [TfimChain(steps=cold_steps, seed=seed * 1_000_000 + 10_000 * pi + k, **base)
                   for k in range(cold_chains)]
        for ti, th in enumerate(thetas):
            chains += [TfimChain(steps=warm_steps, seed=seed * 1_000_000 + 10_000 * pi + 1000 * (ti + 1) + k,
                                 warm_angles=[float(th)] * sp, **base) for k in range(warm_chains)]
    runs, ms = run_tfim_batch(chains, precision)
    xs, ts, mk, det = [], [], [], []
    o = 0
    for sp, J, h, beta in points:
        cold = runs[o:o + cold_chains]
        o += cold_chains
        late = np.concatenate([r.E[r.step >= cold_steps // 2] for r in cold])
        target_E = float(np.mean(late))
        early = []
        for _ in thetas:
            rr = runs[o:o + warm_chains]
            o += warm_chains
            early.append(float(np.mean(np.concatenate([r.E[r.step >= 1] for r in rr]))))
        d = np.array(early) - target_E
        th = float(thetas[int(np.argmin(np.abs(d)))])
        for i in range(len(thetas) - 1):  # first sign change along the grid
            if d[i] == 0.0 or d[i] * d[i + 1] < 0.0:
                f = d[i] / (d[i] - d[i + 1]) if d[i] != d[i + 1] else 0.0
                th = float(thetas[i] + f * (thetas[i + 1] - thetas[i]))
                break
        xs.append(features(sp, J, h, beta))
        t = np.zeros(MAX_SPINS, np.float32)
        m = np.zeros(MAX_SPINS, np.float32)
        t[:sp] = th
        m[:sp] = 1.0
        ts.append(t)
        mk.append(m)
        det.append({"spins": sp, "J": J, "h": h, "beta": beta, "cold_long_run_E": target_E,
                    "warm_early_E": [round(v, 3) for v in early], "target_angle": th,
                    "cold_samples": int(late.size)})
    info = {"chains": len(chains), "chain_steps": cold_chains * cold_steps * len(points) +
            warm_chains * warm_steps * len(points) * len(thetas), "device_ms": ms, "points": det}
    return np.array(xs), np.array(ts), np.array(mk), info


def burn_in_experiment(spins=(4, 5, 6), ene_qbits=4, train_chains=512, train_steps=12, train_burn=6,
                       eval_groups=((6, 1.0, 0.3), (6, 1.0, 1.0), (6, 0.7, 1.8)), eval_chains=96, eval_steps=8,
                       precision="f32", iters=1500, seed=7, eval_ene_qbits=None, target="energy", scan=None,
                       eval_seed=50_000):
    """Trains the network on plain chains and compares warm- and cold-started
    chains of held-out parameter sets.  Returns a dict with, per group, the
    equilibrium energy (cold chains after burn-in), the mean energy error of the
    first samples for cold and warm starts, and the number of steps each start
    needs before its step-averaged energy stays within two standard errors of
    equilibrium.

    target = "energy": the training angle of a parameter set is the product
    state with the cold chains' mean energy (training_set); the chains use
    ene_qbits energy qubits, the evaluation chains eval_ene_qbits (default: the
    same).  target = "scan": the angles come from scan_targets(**scan) (chains of
    the evaluation width started at a grid of angles), the angle whose plain
    chains reach the cold chains' long-run energy first.  target = "bloch": the
    angles come from bloch_targets(**scan), the per-spin Bloch data of the plain
    chains' states."""
    from .batch import TfimChain, run_tfim_batch
    ee = ene_qbits if eval_ene_qbits is None else eval_ene_qbits
    rng = np.random.default_rng(seed)
    if target == "scan":
        t0 = time.perf_counter()
        x, t, m, sinfo = scan_targets(precision=precision, seed=seed, **scan)
        data = {"target": "angle scan", "scan": sinfo, "scan_s": time.perf_counter() - t0,
                "train_rows": int(x.shape[0]), "train_qubits": [scan["points"][0][0] + scan["ene_qbits"] + 1]}
    elif target == "bloch":
        t0 = time.perf_counter()
        x, t, m, binfo = bloch_targets(precision=precision, seed=seed, **scan)
        data = {"target": "equilibrium Bloch angles", "bloch": binfo, "bloch_s": time.perf_counter() - t0,
                "train_rows": int(x.shape[0]), "train_qubits": [scan["points"][0][0] + scan["ene_qbits"] + 1]}
    else:
        chains = [TfimChain(spins=int(rng.choice(spins)), ene_qbits=ene_qbits, steps=train_steps,
                            beta=float(rng.uniform(0.2, 2.0)), h=float(rng.uniform(0.5, 1.5)), thermalization=0,
                            seed=10_000 + i) for i in range(train_chains)]
        runs, ms_data = run_tfim_batch(chains, precision)
        x, t, m = training_set(chains, runs, train_burn)
        data = {"target": "product-state energy", "train_chains": train_chains,
                "train_qubits": sorted({c.nqubits for c in chains}),
                "train_samples": int(sum(int(np.sum(r.step >= train_burn)) for r in runs)),
                "train_rows": int(x.shape[0]), "data_device_ms": ms_data,
                "data_chain_steps_per_s": train_chains * train_steps / (ms_data / 1e3)}
    net = WarmStartNet(seed=seed)
    t0 = time.perf_counter()
    losses = net.fit(x, t, m, iters=iters, batch=256, lr=2e-3, seed=seed)
    fit_s = time.perf_counter() - t0
    out = dict(data)
    out.update({"fit_iters": iters, "fit_s": fit_s,
                "loss_first": float(np.mean(losses[:20])), "loss_last": float(np.mean(losses[-20:])),
                "eval_chains_per_group": eval_chains, "eval_qubits": None, "groups": []})
    # every group's cold and warm chains run as one batch (better load balance)
    allc, angs = [], []
    for gi, (s, h, beta) in enumerate(eval_groups):
        base = dict(spins=s, ene_qbits=ee, steps=eval_steps, beta=beta, h=h, thermalization=0)
        ang = net.angles(s, 1.0, h, beta)
        angs.append(ang)
        allc += [TfimChain(seed=eval_seed + 1000 * gi + k, **base) for k in range(eval_chains)]
        allc += [TfimChain(seed=eval_seed + 1000 * gi + k, warm_angles=ang, **base) for k in range(eval_chains)]
    out["eval_qubits"] = allc[0].nqubits
    rall, ms_eval = run_tfim_batch(allc, precision)
    out["eval_device_ms"] = ms_eval
    out["eval_chain_steps_per_s"] = len(allc) * eval_steps / (ms_eval / 1e3)
    for gi, (s, h, beta) in enumerate(eval_groups):
        o = 2 * eval_chains * gi
        rc, rw = rall[o:o + eval_chains], rall[o + eval_chains:o + 2 * eval_chains]
        ang = angs[gi]

        def per_step(rr):
            mat = np.full((len(rr), eval_steps), np.nan)
            for i, r in enumerate(rr):
                mat[i, r.step.astype(int)] = r.E
            cnt = np.sum(~np.isnan(mat), axis=0)
            mean = np.full(eval_steps, np.nan)
            sem = np.full(eval_steps, np.nan)
            for k in np.nonzero(cnt)[0]:  # steps without a single sample stay NaN
                col = mat[~np.isnan(mat[:, k]), k]
                mean[k] = col.mean()
                sem[k] = col.std() / np.sqrt(len(col))
            return mean, sem

        mc, sc = per_step(rc)
        mw, _ = per_step(rw)
        eq = float(np.nanmean(mc[eval_steps // 2:]))
        err = float(np.nanmean(sc[eval_steps // 2:]))  # standard error of one step's mean
        err_eq = err / np.sqrt(max(1, eval_steps - eval_steps // 2))  # ... of the equilibrium estimate
        first = slice(1, 4)  # step 0 is never sampled (the driver samples from step 1 on)

        def burn(mean):
            # first step from which every 3-step average of the step means stays
            # within two standard errors of the equilibrium estimate
            tol = 2.0 * (err / np.sqrt(3.0) + err_eq) + 1e-12
            for k in range(1, eval_steps - 2):
                if all(abs(np.nanmean(mean[j:j + 3]) - eq) <= tol for j in range(k, eval_steps - 2)):
                    return k
            return eval_steps

        late = slice(eval_steps // 2, eval_steps)
        q4 = slice(3 * eval_steps // 4, eval_steps)
        head = slice(1, min(11, eval_steps))
        out["groups"].append({"spins": s, "h": h, "beta": beta, "E_eq": eq, "E_eq_err": float(err_eq),
                              "step_mean_err": err,
                              "cold_excess_first10": float(np.nansum(np.abs(mc[head] - eq))),
                              "warm_excess_first10": float(np.nansum(np.abs(mw[head] - eq))),
                              "cold_curve": [round(float(v), 3) for v in mc[:min(12, eval_steps)]],
                              "warm_curve": [round(float(v), 3) for v in mw[:min(12, eval_steps)]],
                              "warm_angle": ang[0], "cold_first_err": float(np.nanmean(np.abs(mc[first] - eq))),
                              "warm_first_err": float(np.nanmean(np.abs(mw[first] - eq))),
                              "cold_burn_in_steps": burn(mc), "warm_burn_in_steps": burn(mw),
                              "warm_late_E": float(np.nanmean(mw[late])),
                              "cold_last_quarter_E": float(np.nanmean(mc[q4])),
                              "warm_last_quarter_E": float(np.nanmean(mw[q4])),
                              "cold_curve_by_10": [round(float(np.nanmean(mc[k:k + 10])), 3)
                                                   for k in range(0, eval_steps, 10)],
                              "warm_curve_by_10": [round(float(np.nanmean(mw[k:k + 10])), 3)
                                                   for k in range(0, eval_steps, 10)],
                              "warm_late_minus_cold_late": float(np.nanmean(mw[late]) - eq)})
    net.close()
    return out


# The learned warm-start study at its full size: 12-spin TFIM rings, training
# data from 1024 plain cold-start chains (4 energy qubits, 17 qubits) with 50
# samples each after 10 burn-in steps (~48k samples), evaluation on 2 groups of
# 48 chains of 12 spins + 6 energy qubits (19 qubits), 100 steps, FP32; the
# equilibrium energy of a group is the cold chains' mean over steps 50-99.
FULL_STUDY = dict(spins=(12,), ene_qbits=4, train_chains=1024, train_steps=60, train_burn=10,
                  eval_groups=((12, 1.0, 1.0), (12, 0.8, 1.9)),
                  eval_chains=48, eval_steps=100, eval_ene_qbits=6, iters=2000)

# A small angle-scan study (6-spin rings, 4 energy qubits: 11 qubits), seconds
# on one GPU: the configuration of the test suite.
SMALL_SCAN_STUDY = dict(ene_qbits=4, eval_groups=((6, 0.8, 0.9), (6, 1.2, 1.6)), eval_chains=64, eval_steps=30,
                        iters=1500, target="scan",
                        scan=dict(points=[(6, 1.0, h, b) for h in (0.6, 1.0, 1.4) for b in (0.5, 1.2, 1.9)],
                                  ene_qbits=4, thetas=tuple(float(v) for v in np.linspace(-1.2, 0.0, 7)),
                                  warm_chains=16, warm_steps=8, cold_chains=32, cold_steps=30))

# The same evaluation with angle-scan targets: 12 parameter points of 12-spin
# rings (h in {0.6, 1.0, 1.4} x beta in {0.4, 0.9, 1.4, 1.9}) with the evaluation
# width (6 energy qubits, 19 qubits): 32 cold chains x 60 steps per point and 8
# chains x 12 steps per grid angle; the evaluation groups are off the grid.
SCAN_ANGLES = tuple(float(v) for v in np.linspace(-1.2, 0.0, 9))

# Equilibrium Bloch-angle targets (bloch_targets): small (6-spin rings, 11 qubits)
# and full size (12-spin rings at the evaluation width, 19 qubits).
SMALL_BLOCH_STUDY = dict(ene_qbits=4, eval_groups=((6, 0.8, 0.9), (6, 1.2, 1.6)), eval_chains=64, eval_steps=30,
                         iters=1500, target="bloch",
                         scan=dict(points=[(6, 1.0, h, b) for h in (0.6, 1.0, 1.4) for b in (0.5, 1.2, 1.9)],
                                   ene_qbits=4, chains_per_point=16, burn=10, samples=4, every=5))
FULL_BLOCH_STUDY = dict(ene_qbits=6, eval_groups=((12, 0.8, 1.15), (12, 1.2, 1.65)), eval_chains=48,
                        eval_steps=100, eval_ene_qbits=6, iters=2000, target="bloch",
                        scan=dict(points=[(12, 1.0, h, b) for h in (0.6, 1.0, 1.4) for b in (0.4, 0.9, 1.4, 1.9)],
                                  ene_qbits=6, chains_per_point=8, burn=30, samples=3, every=10))
FULL_SCAN_STUDY = dict(ene_qbits=6, eval_groups=((12, 0.8, 1.15), (12, 1.2, 1.65)), eval_chains=48,
                       eval_steps=100, eval_ene_qbits=6, iters=2000, target="scan",
                       scan=dict(points=[(12, 1.0, h, b) for h in (0.6, 1.0, 1.4) for b in (0.4, 0.9, 1.4, 1.9)],
                                 ene_qbits=6, thetas=SCAN_ANGLES, warm_chains=8, warm_steps=12, cold_chains=32,
                                 cold_steps=60))


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="learned warm-start burn-in study")
    ap.add_argument("--full", action="store_true", help="the full-size study (several GPU minutes)")
    ap.add_argument("--scan", action="store_true", help="angle-scan targets (with --full: FULL_SCAN_STUDY)")
    ap.add_argument("--bloch", action="store_true", help="equilibrium Bloch-angle targets (with --full: "
                                                         "FULL_BLOCH_STUDY)")
    ap.add_argument("--eval-seed", type=int, default=50_000, help="first seed of the evaluation chains")
    a = ap.parse_args()
    if a.bloch:
        st = FULL_BLOCH_STUDY if a.full else SMALL_BLOCH_STUDY
        res = burn_in_experiment(eval_seed=a.eval_seed, **st)
    elif a.scan:
        res = burn_in_experiment(**FULL_SCAN_STUDY) if a.full else burn_in_experiment(**SMALL_SCAN_STUDY)
    else:
        res = burn_in_experiment(**FULL_STUDY) if a.full else burn_in_experiment()
    print(json.dumps(res))
