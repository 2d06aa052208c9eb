"""Benchmark: the gate-engine microbenchmark (28-qubit FP64 state, 1000 random
gates, a measurement every 100 gates) on one GB300, through libsq.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl own|reference]

A step applies the whole 1000-gate circuit to the resident state.  `value` is
the algorithmic gate bandwidth: the sum over gates of 2*B*N*f (B = 16 bytes per
FP64 amplitude, f = fraction of amplitudes the gate must touch) divided by the
device time of the step, so fused passes can exceed the HBM peak; `roofline`
reports the bytes the executed passes really moved.  `e2e` repeats the step
through the public API with the state copied in from, and out to, page-locked
host memory inside the timed region.  The state (4 GiB) is larger than L2, so
no flush is needed between steps.  N > 1 runs independent replicas (one state
per GPU; the path has no exchange step).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "gate HBM GB/s (gate-engine microbenchmark)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="own", choices=["own", "reference"])
    ap.add_argument("--n", type=int, default=28)
    ap.add_argument("--gates", type=int, default=1000)
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"])
    ap.add_argument("--no-fusion", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-qms", action="store_true")
    ap.add_argument("--qms-chains", type=int, default=1024)
    ap.add_argument("--qms-steps", type=int, default=6)
    ap.add_argument("--skip-30", action="store_true", help="skip the 30-qubit FP64 repeat")
    ap.add_argument("--skip-qsa", action="store_true")
    ap.add_argument("--qsa-walks", type=int, default=1024)
    # walk steps per walk in the walk line: enough for the 16-warp orbit pass's order
    # table to serve most steps, as it does over a full anneal
    ap.add_argument("--qsa-steps", type=int, default=32)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(n, gates, seconds, bytes_per_amp):
    """The CPU oracle (a restatement of the reference's dense CPU loops, pinned
    bit-exact to it) on this host's cores, over a time-bounded prefix of the same
    circuit.  Returns (GB/s, gates timed, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle
    from suqa_gb300.workloads import algorithmic_bytes, random_state
    threads = os.cpu_count() or 1
    L = oracle.load()
    L.or_set_threads(threads)
    ost = oracle.OracleState(n)
    re, im = random_state(n, 7)
    N = 1 << n
    buf = np.ctypeslib.as_array(ost.p.contents.data, shape=(2 * N,))
    buf[:N] = re
    buf[N:] = im
    done = 0
    t0 = time.perf_counter()
    while done < len(gates) and time.perf_counter() - t0 < seconds:
        oracle.apply_circuit(ost, gates[done:done + 1])
        done += 1
    dt = time.perf_counter() - t0
    L.or_set_threads(1)
    ost.close()
    alg = algorithmic_bytes(gates[:done], n, bytes_per_amp)
    return alg / dt / 1e9, done, threads, dt


def qms_section(n_chains, steps, seed=2024):
    """Batched quantum Metropolis sampling of TFIM rings: a sample of the
    4096-chain workload (spins 4-10, energy register 4-6 qubits, J = 1,
    h ~ U[0.5, 1.5], beta ~ U[0.2, 2.0], dt = 0.1, one PCG32 stream per chain),
    run as resumable batches (segments of 2 steps replayed from a CUDA graph;
    FP32 with autotuned CTA sizes) in FP32 and FP64; then the host-driven plain
    GPU chain (the drop-in qms driver on the libsq state API) on a 7-spin,
    5-energy-qubit ring against a batch of chains of that same configuration."""
    import numpy as np
    from suqa_gb300.batch import Batch, TfimChain, run_tfim_batch
    rng = np.random.default_rng(seed)
    chains = [TfimChain(spins=int(rng.integers(4, 11)), ene_qbits=int(rng.integers(4, 7)), steps=steps,
                        beta=float(rng.uniform(0.2, 2.0)), h=float(rng.uniform(0.5, 1.5)), thermalization=0,
                        seed=1 + i) for i in range(n_chains)]
    out = {"workload": f"{n_chains} TFIM-ring chains x {steps} Metropolis steps (8-17 qubits)",
           "mode": "resumable batch, segments of 2 steps from a CUDA graph, all width classes concurrent"}
    runs, batches = {}, {}
    for prec in ("f32", "f64"):
        t0 = time.perf_counter()
        b = Batch(chains, prec, segment_steps=2, use_graph=True, autotune=(prec == "f32"))
        t1 = time.perf_counter()
        ms = b.run(steps)
        r = b.results()
        runs[prec], batches[prec] = r, b
        cyc = sum(x.cycles for x in r)
        out[prec] = {"chain_steps_per_s": n_chains * steps / (ms / 1e3), "device_ms": ms,
                     "setup_s": t1 - t0, "wall_s": time.perf_counter() - t0,
                     "phase_estimations_per_step": float(np.mean([x.phase_estimations for x in r])) / steps,
                     "evolution_share_of_sm_time": sum(x.evolution_cycles for x in r) / max(cyc, 1),
                     "plan": b.plan()}
    # FP32 vs FP64 on identical chains and draws: measured sequences, energies, and
    # the final amplitudes of chains whose sequences agree (the FP64 batch chain is
    # the plain reference procedure, outcome for outcome)
    same = [i for i, (a, b) in enumerate(zip(runs["f32"], runs["f64"]))
            if a.accepted == b.accepted and np.array_equal(a.E, b.E) and np.array_equal(a.A, b.A)]
    amp_err = []
    for i in same[:32]:
        s32, s64 = batches["f32"].state(i), batches["f64"].state(i)
        amp_err.append(float(np.max(np.abs(s32 - s64)) / np.max(np.abs(s64))))
    groups = {}
    for c, a, b in zip(chains, runs["f32"], runs["f64"]):
        g = groups.setdefault(c.spins, {"f32": [], "f64": []})
        g["f32"].append(a.E)
        g["f64"].append(b.E)
    per_group = {}
    for sp, g in sorted(groups.items()):
        e32, e64 = np.concatenate(g["f32"]), np.concatenate(g["f64"])
        if len(e64) < 2:
            continue
        per_group[str(sp)] = {"mean_E_f32": float(e32.mean()), "mean_E_f64": float(e64.mean()),
                              "stderr_E_f64": float(e64.std() / len(e64) ** 0.5), "samples": int(len(e64))}
    out["fp32_vs_fp64"] = {"chains_identical": len(same), "chains": n_chains,
                           "max_rel_amplitude_error_f32": max(amp_err) if amp_err else None,
                           "amplitude_error_chains": len(amp_err), "energy_by_ring_length": per_group}
    for b in batches.values():
        b.close()
    # Like-for-like comparator.  The plain GPU chain is the drop-in qms driver
    # (host-driven, one libsq state, host sync per measurement) on one 7-spin ring
    # with a 5-qubit energy register (13 qubits); its rate is the driver's own
    # timer around the Metropolis loop (no process start, device set-up or initial
    # state).  The batched rate is the same chain configuration (spins, register,
    # beta, h, window), 1024 chains with their own seeds, FP32, in one batch.
    plain_steps = 50
    exe = os.path.join(ROOT, "suqa_gb300", "_build", "qms_tfim_s7")
    env = dict(os.environ, TFIM_J="1.0", TFIM_H="1.0")
    t0 = time.perf_counter()
    cp = subprocess.run([exe, "1.0", str(plain_steps), "1", "5", "/tmp/suqa_plain_chain.txt", "--seed", "5",
                         "--ene-min", "-14", "--ene-max", "14", "--thermalization", "0"], env=env,
                        capture_output=True, text=True)
    wall = time.perf_counter() - t0
    if os.path.exists("/tmp/suqa_plain_chain.txt"):
        os.remove("/tmp/suqa_plain_chain.txt")
    loop_s = _chain_loop_seconds(cp.stdout) if cp.returncode == 0 else None
    plain = plain_steps / loop_s if loop_s else None
    same_cfg = [TfimChain(spins=7, ene_qbits=5, steps=steps, beta=1.0, h=1.0, ene_min=-14.0, ene_max=14.0,
                          thermalization=0, seed=5 + k) for k in range(n_chains)]
    tb = time.perf_counter()
    bs = Batch(same_cfg, "f32", segment_steps=2, use_graph=True, autotune=True)
    tb1 = time.perf_counter()
    ms_same = bs.run(steps)
    wall_same = time.perf_counter() - tb1
    rs = bs.results()
    bs.close()
    batched_same = n_chains * steps / (ms_same / 1e3)
    batched_same_wall = n_chains * steps / wall_same
    # phase estimations per step differ between chains (restoration loops): the
    # per-estimation rates remove that from the comparison (the batch engine's FP64
    # chain with the plain chain's seed has the plain chain's outcomes, hence its
    # number of phase estimations)
    plain_pe_rate = None
    if loop_s:
        same50, _ = run_tfim_batch([TfimChain(spins=7, ene_qbits=5, steps=plain_steps, beta=1.0, h=1.0,
                                              ene_min=-14.0, ene_max=14.0, thermalization=0, seed=5)], "f64")
        plain_pe_rate = same50[0].phase_estimations / loop_s
    batched_pe_rate = sum(x.phase_estimations for x in rs) / (ms_same / 1e3)
    out["plain_gpu_chain"] = {"steps_per_s": plain, "steps": plain_steps, "loop_s": loop_s,
                              "process_wall_s": wall, "phase_estimations_per_s": plain_pe_rate,
                              "timer": "the driver's own timer around its Metropolis loop",
                              "config": "7 spins, 5 energy qubits (13 qubits), beta 1, h 1, FP64, host-driven "
                                        "(libsq state API, drop-in qms driver)"}
    out["batched_same_config_f32"] = {"chain_steps_per_s_device": batched_same,
                                      "chain_steps_per_s_wall": batched_same_wall,
                                      "chains": n_chains, "steps": steps, "device_ms": ms_same,
                                      "setup_s": tb1 - tb, "phase_estimations_per_s": batched_pe_rate}
    out["batched_f32_over_plain_steps"] = (batched_same / plain) if plain else None
    out["batched_f32_over_plain_steps_wall"] = (batched_same_wall / plain) if plain else None
    out["batched_f32_over_plain_phase_estimations"] = (batched_pe_rate / plain_pe_rate) if plain_pe_rate else None
    return out


def _chain_loop_seconds(stdout):
    """Seconds of the Metropolis loop from the qms driver's 'chain loop: N steps
    in T s' line."""
    for ln in stdout.splitlines():
        if ln.startswith("chain loop:"):
            return float(ln.split(" in ")[1].split()[0])
    return None


def config1_section():
    """Config 1: the triangle (3 spins, 4 energy qubits + acceptance = 8 qubits),
    beta 1, 200 steps, seed 42, window [-1, 3], 20 thermalisation steps, through the
    drop-in qms driver on the GPU; the rate is the driver's own loop timer."""
    exe = os.path.join(ROOT, "suqa_gb300", "_build", "qms")
    outp = "/tmp/suqa_config1.txt"
    if os.path.exists(outp):
        os.remove(outp)
    cp = subprocess.run([exe, "1.0", "200", "1", "4", outp, "--seed", "42", "--ene-min", "-1", "--ene-max", "3",
                         "--thermalization", "20"], capture_output=True, text=True)
    loop_s = _chain_loop_seconds(cp.stdout) if cp.returncode == 0 else None
    rows = 0
    if os.path.exists(outp):
        rows = sum(1 for ln in open(outp) if ln and not ln.startswith("#"))
        os.remove(outp)
    acc = None
    for ln in cp.stdout.splitlines():
        if "acceptance:" in ln:
            acc = ln.split("acceptance:")[1].strip()
    return {"workload": "triangle QMS, 8 qubits FP64, beta 1, 200 steps, seed 42 (drop-in qms driver)",
            "steps_per_s": 200 / loop_s if loop_s else None, "loop_s": loop_s, "rows_written": rows,
            "acceptance": acc, "rc": cp.returncode}


def qsa_section(n_walks, walk_steps, f64_walks=16, cpu=True, seed=2025):
    """Batched Szegedy-walk annealing on 10-spin Ising rings (J = +-1 drawn per
    walk, h = 0, beta 0 -> 1 over 50 stages x 20 walk steps, 6-qubit walk-phase
    register, one PCG32 stream per walk): every walk capped at its first
    `walk_steps` walk steps (restarts included), FP32 for all walks, FP64 for the
    first `f64_walks`, with algorithm 1 (orbit classes); algorithm 0 (the per-orbit
    iteration) runs the same FP32 walks for comparison.  Rates are also given as
    the per-orbit iteration's flops per second: 2^9 + 511 * 2^8 orbits per walk
    step, each 63 applications of W (272 flops: 4 Hadamards x 16, 4 rotations x 48,
    2 reflections x 8) plus 64 overlap/sum updates (48 flops)."""
    import numpy as np
    from suqa_gb300.walk import ising_ring_walks, run_qsa_walks
    walks = ising_ring_walks(n_walks, 10, 1.0, 50, 20, 6, seed=seed, max_steps=walk_steps, algo=1)
    run_qsa_walks(walks[:4], "f32")  # first launch, module load
    r32, ms32 = run_qsa_walks(walks, "f32", trace=True)
    r64, ms64 = run_qsa_walks(walks[:f64_walks], "f64", trace=True)
    walks0 = ising_ring_walks(n_walks, 10, 1.0, 50, 20, 6, seed=seed, max_steps=walk_steps, algo=0)
    r0, ms0 = run_qsa_walks(walks0, "f32")
    st32 = sum(r.steps for r in r32)
    st64 = sum(r.steps for r in r64)
    same = [i for i, (a, b) in enumerate(zip(r32, r64)) if (a.restarts, a.steps) == (b.restarts, b.steps)]
    p0_err = max((float(np.max(np.abs(r32[i].p0 - r64[i].p0))) for i in same), default=None)
    # flops of the per-orbit iteration (algorithm 0) per walk step: the rate either
    # algorithm delivers, expressed as that work per second
    norb, L = (1 << 9) + ((1 << 9) - 1) * (1 << 8), 64
    flops = norb * ((L - 1) * 272 + L * 48)
    # algorithm 1's own work per walk step: per orbit V^T psi and Q psi (2 x 16 x 16
    # multiply-adds); the state (2^21 amplitudes) is read and written once
    cls_flops = norb * 2 * 16 * 16 * 2
    out = {"workload": f"{n_walks} walks on 10-spin Ising rings (2^21 amplitudes each), first {walk_steps} walk "
                       f"steps of the beta 0->1 anneal (50 stages x 20 steps), 6-qubit walk-phase register",
           "algorithm": "1 (orbit classes); f32_per_orbit_iteration: algorithm 0 on the same walks",
           "f32_per_orbit_iteration": {"walk_steps_per_s": sum(r.steps for r in r0) / (ms0 / 1e3),
                                       "fp32_tflops": flops * sum(r.steps for r in r0) / (ms0 / 1e3) / 1e12},
           "f32": {"walk_steps_per_s": st32 / (ms32 / 1e3), "walk_steps": st32, "device_ms": ms32,
                   "restarts": int(sum(r.restarts for r in r32)),
                   "equivalent_fp32_tflops": flops * st32 / (ms32 / 1e3) / 1e12,
                   "own_fp32_tflops": cls_flops * st32 / (ms32 / 1e3) / 1e12,
                   "state_hbm_gbs": 2 * 4 * (1 << 21) * st32 / (ms32 / 1e3) / 1e9},
           "f64": {"walk_steps_per_s": st64 / (ms64 / 1e3), "walk_steps": st64, "device_ms": ms64,
                   "equivalent_fp64_tflops": flops * st64 / (ms64 / 1e3) / 1e12, "walks": f64_walks},
           "fp32_vs_fp64": {"walks_identical": len(same), "walks": f64_walks, "max_abs_p0_diff": p0_err},
           "flops_per_walk_step": flops, "own_flops_per_walk_step": cls_flops}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import qsa_walk as qw
        cw = qw.CompressedWalk(10, walks[0].J)
        t0 = time.perf_counter()
        qw.walk_step(cw, cw.initial(), 3, 0.02, 6)
        dt = time.perf_counter() - t0
        out["cpu_port"] = {"s_per_walk_step": dt, "kind": "port", "cores": 1,
                           "sample": "one walk step of one walk, numpy FP64 oracle"}
    return out


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    from suqa_gb300.workloads import random_circuit
    bpa = 16 if args.precision == "f64" else 8
    gates = random_circuit(args.n, args.gates, seed=7)
    vals = []
    sample = None
    for i in range(args.warmup + args.steps):
        v, done, threads, dt = cpu_baseline(args.n, gates, args.cpu_seconds, bpa)
        sample = f"first {done} of {len(gates)} ops of the {args.n}-qubit circuit, {dt:.1f} s"
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    from suqa_gb300.workloads import algorithmic_bytes
    ms_per_step = algorithmic_bytes(gates, args.n, bpa) / (value * 1e9) * 1e3  # whole circuit at this rate
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "impl": "reference",
            "dtype": args.precision, "data": "synthetic",
            "config": {"workload": f"random circuit, {args.n} qubits {args.precision.upper()}, "
                                   f"{args.gates} gates, measure every 100", "n_qubits": args.n},
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from suqa_gb300 import State
    from suqa_gb300.workloads import algorithmic_bytes, apply_circuit, fp64_instructions, random_circuit, random_state

    n = args.n
    bpa = 16 if args.precision == "f64" else 8
    dt_np = np.float64 if args.precision == "f64" else np.float32
    gates = random_circuit(n, args.gates, seed=7)
    alg = algorithmic_bytes(gates, n, bpa)
    # a dedicated stream: the states run on it and the CUDA events are recorded on
    # it (the legacy default stream's handle is 0, which libsq reads as "the
    # state's own stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    st = State(n, args.precision)
    st.set_stream(stream.cuda_stream)
    st.set_fusion(not args.no_fusion)
    re, im = random_state(n, 7, dt_np)
    h_re = torch.from_numpy(re).pin_memory()
    h_im = torch.from_numpy(im).pin_memory()
    o_re = torch.empty_like(h_re).pin_memory()
    o_im = torch.empty_like(h_im).pin_memory()
    del re, im
    st.upload(h_re.data_ptr(), h_im.data_ptr())

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident: K steps of the circuit on the resident state
    for _ in range(args.warmup):
        apply_circuit(st, gates)
    st.flush()
    barrier()
    st.reset_stats()
    st.set_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            apply_circuit(st, gates)
        st.flush()
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    kms, klaunch, kbytes = st.kernel_time()
    st.set_timing(False)
    stats = st.stats()
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = alg * world / (ms_step / 1e3) / 1e9

    # ---- end to end: host state in, circuit, host state out, per step
    for _ in range(1):
        st.upload(h_re.data_ptr(), h_im.data_ptr())
        apply_circuit(st, gates)
        st.download(o_re.data_ptr(), o_im.data_ptr())
    barrier()
    t0 = time.perf_counter()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    bits_all = []
    for _ in range(args.steps):
        st.upload(h_re.data_ptr(), h_im.data_ptr())
        bits_all.append(apply_circuit(st, gates))
        st.download(o_re.data_ptr(), o_im.data_ptr())
    e3.record(stream)
    barrier()
    ms_e2e_serial = e2.elapsed_time(e3) / args.steps
    state_bytes = (1 << n) * bpa  # re + im

    # ---- end to end, pipelined: two states, each on its own stream and host
    # thread; every step still uploads its input, runs the circuit and downloads
    # its result.  The circuits take turns (one at a time on the GPU, strictly
    # alternating between the states), so each state's download and next upload
    # run on the copy engines while the other state's circuit has every SM; two
    # circuits sharing the SMs would put their copies in the same window and
    # leave the SMs idle while both copy
    import threading
    st2 = State(n, args.precision)
    s2 = torch.cuda.Stream()
    st2.set_stream(s2.cuda_stream)
    st2.set_fusion(not args.no_fusion)
    o2_re = torch.empty_like(h_re).pin_memory()
    o2_im = torch.empty_like(h_im).pin_memory()
    st2.upload(h_re.data_ptr(), h_im.data_ptr())
    apply_circuit(st2, gates)
    st2.download(o2_re.data_ptr(), o2_im.data_ptr())
    # an even number of steps, so both pipelines finish together
    pipe_steps = args.steps + (args.steps & 1)
    pipe_bits = [None] * pipe_steps
    # per step and state: events around the upload, the circuit and the download
    # on the state's stream, so the end-to-end time can be attributed
    pipe_ev = [None] * pipe_steps

    # uploads also go in step order: the second state's first upload waits for the
    # first state's, instead of sharing the host link with it and delaying the
    # first circuit (later uploads fall inside the other state's circuit anyway)
    turn = {"next": 0, "uploaded": 0}
    turn_cv = threading.Condition()

    def pipeline(stx, strm, ore, oim, steps):
        for i in steps:
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            with turn_cv:
                turn_cv.wait_for(lambda: turn["uploaded"] >= i)
            ev[0].record(strm)
            stx.upload(h_re.data_ptr(), h_im.data_ptr())
            ev[1].record(strm)
            ev[1].synchronize()
            with turn_cv:
                turn["uploaded"] = max(turn["uploaded"], i + 1)
                turn_cv.notify_all()
            with turn_cv:  # step i's circuit runs after step i-1's has completed
                turn_cv.wait_for(lambda: turn["next"] == i)
            pipe_bits[i] = apply_circuit(stx, gates)
            stx.flush()
            ev[2].record(strm)
            ev[2].synchronize()
            with turn_cv:
                turn["next"] = i + 1
                turn_cv.notify_all()
            stx.download(ore.data_ptr(), oim.data_ptr())
            ev[3].record(strm)
            pipe_ev[i] = ev

    barrier()
    e4 = torch.cuda.Event(enable_timing=True)
    e5 = torch.cuda.Event(enable_timing=True)
    e4.record(stream)
    workers = [threading.Thread(target=pipeline, args=(st, stream, o_re, o_im, range(0, pipe_steps, 2))),
               threading.Thread(target=pipeline, args=(st2, s2, o2_re, o2_im, range(1, pipe_steps, 2)))]
    for w in workers:
        w.start()
    for w in workers:
        w.join()
    torch.cuda.synchronize()
    e5.record(stream)
    barrier()
    ms_e2e = e4.elapsed_time(e5) / pipe_steps
    e2e_value = alg * world / (ms_e2e / 1e3) / 1e9
    pipe_ok = all(b == bits_all[0] for b in pipe_bits + bits_all)
    up_ms = [e[0].elapsed_time(e[1]) for e in pipe_ev]
    cir_ms = [e[1].elapsed_time(e[2]) for e in pipe_ev]
    down_ms = [e[2].elapsed_time(e[3]) for e in pipe_ev]
    state_b = (1 << n) * bpa
    e2e_parts = {"upload_ms_median": statistics.median(up_ms), "upload_ms_max": max(up_ms),
                 "upload_gbs_median": state_b / (statistics.median(up_ms) / 1e3) / 1e9,
                 "circuit_ms_median": statistics.median(cir_ms), "circuit_ms_max": max(cir_ms),
                 "download_ms_median": statistics.median(down_ms), "download_ms_max": max(down_ms),
                 "download_gbs_median": state_b / (statistics.median(down_ms) / 1e3) / 1e9,
                 "note": "device-side intervals on each state's stream; a circuit interval includes the "
                         "wait for the other state's circuit (turns) and for its measurements' host decisions"}
    st2.close()
    del o2_re, o2_im

    # FP64 peak of this GPU, measured here with cuBLAS DGEMM (the pass kernel's
    # arithmetic bound in FP64)
    fp64_peak = None
    try:
        xa = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
        xb = torch.randn_like(xa)
        torch.matmul(xa, xb)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        torch.matmul(xa, xb)
        ev1.record()
        torch.cuda.synchronize()
        fp64_peak = 2 * 8192 ** 3 / (ev0.elapsed_time(ev1) / 1e3) / 1e12
        del xa, xb
        torch.cuda.empty_cache()
    except Exception:
        pass

    # FP64 fused multiply-add rate of the CUDA cores (the pass kernel's own pipe;
    # DGEMM above runs on the FP64 tensor path)
    fma_gops = fp64_fma_rate()
    fp64_ins = fp64_instructions(gates, n) * args.steps if args.precision == "f64" else None

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = kbytes / (kms / 1e3) / 1e9 if kms > 0 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None,
                "traffic": traffic_per_launch(),
                "kernel": "sqk::k_pass<%s>" % ("double" if args.precision == "f64" else "float"),
                "launches": klaunch, "avg_launch_ms": kms / klaunch if klaunch else None,
                "bytes_per_launch": kbytes / klaunch if klaunch else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback",
                "fp64_tflops_achieved": stats["flops"] / (kms / 1e3) / 1e12 if kms > 0 else None,
                "fp64_tflops_peak": fp64_peak,
                "fp64_frac": (stats["flops"] / (kms / 1e3) / 1e12 / fp64_peak) if (kms > 0 and fp64_peak) else None,
                "fp64_peak_source": "cuBLAS DGEMM 8192^3 measured in this run",
                "limiter": ("the FP64 CUDA-core pipe (fp64_pipe below; HBM traffic is a small fraction)"
                            if args.precision == "f64" else "shared-memory sweeps (issue-bound)"),
                "fp64_pipe": {"instructions_per_step": fp64_ins / args.steps if fp64_ins else None,
                              "achieved_gops": (fp64_ins / (kms / 1e3) / 1e9) if (fp64_ins and kms > 0) else None,
                              "peak_gops": fma_gops,
                              "frac": (fp64_ins / (kms / 1e3) / 1e9 / fma_gops) if (fp64_ins and kms > 0 and fma_gops)
                              else None,
                              "peak_source": "sqb_fp64_fma_rate (libsq_probe.so): independent DFMA chains on every SM, measured in "
                                             "this run (of measured)"}}

    # secondary: the same FP64 circuit with double-float arithmetic (hi + lo FP32
    # pairs on the FP32 pipe, doubles in memory), against the FP64-arithmetic result
    # of the same circuit and state (o_re, o_im; bits_all[0])
    df_line = None
    if args.precision == "f64" and rank == 0:
        st.set_double_float(True)
        st.upload(h_re.data_ptr(), h_im.data_ptr())
        bits_df = apply_circuit(st, gates)
        dfr = torch.empty_like(o_re).pin_memory()
        dfi = torch.empty_like(o_im).pin_memory()
        st.download(dfr.data_ptr(), dfi.data_ptr())
        flipped_df = sum(1 for x, y in zip(bits_df, bits_all[0]) if x != y)
        df_err = None
        if flipped_df == 0:
            r64, i64 = o_re.numpy(), o_im.numpy()
            dr = dfr.numpy() - r64
            di = dfi.numpy() - i64
            nrm = math.sqrt(float(np.dot(r64, r64)) + float(np.dot(i64, i64)))
            amax = float(np.sqrt(np.max(r64 * r64 + i64 * i64)))
            df_err = {"normwise_rel": math.sqrt(float(np.dot(dr, dr)) + float(np.dot(di, di))) / nrm,
                      "max_abs_over_max_amplitude": float(np.sqrt(np.max(dr * dr + di * di))) / amax}
            del dr, di
        del dfr, dfi
        for _ in range(args.warmup):
            apply_circuit(st, gates)
        st.flush()
        torch.cuda.synchronize()
        st.set_timing(True)
        st.kernel_time()
        d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        d0.record(stream)
        for _ in range(args.steps):
            apply_circuit(st, gates)
        st.flush()
        d1.record(stream)
        torch.cuda.synchronize()
        msdf = d0.elapsed_time(d1) / args.steps
        kdf, ldf, bdf = st.kernel_time()
        st.set_timing(False)
        st.set_double_float(False)
        df_line = {"value": alg / (msdf / 1e3) / 1e9, "unit": "GB/s", "ms_per_step": msdf,
                   "speedup_over_fp64_arithmetic": ms_step / msdf,
                   "pass_kernel_gbs": bdf / (kdf / 1e3) / 1e9 if kdf > 0 else None,
                   "pass_kernel_frac_of_hbm": (bdf / (kdf / 1e3) / 1e9 / peaks.get("hbm_gbs", 6800.0))
                   if kdf > 0 else None,
                   "vs_fp64_arithmetic": {"measured_bits": len(bits_df), "flipped_bits": flipped_df,
                                          "amplitude_error": df_err},
                   "arithmetic": "double-float (hi + lo FP32, 48 significand bits) on the FP32 pipe; amplitudes "
                                 "stored as IEEE doubles; not the headline (FP64 arithmetic is)"}

    # secondary: the same circuit with FP32 amplitudes (FP64 reductions)
    fp32_line = None
    if args.precision == "f64" and rank == 0:
        st.close()
        st32 = State(n, "f32")
        st32.set_stream(stream.cuda_stream)
        r32, i32 = random_state(n, 7, np.float32)
        h32r = torch.from_numpy(r32).pin_memory()
        h32i = torch.from_numpy(i32).pin_memory()
        st32.upload(h32r.data_ptr(), h32i.data_ptr())
        bits32 = apply_circuit(st32, gates)
        # FP32 against the FP64 result of the same circuit from the same state
        # (o_re, o_im hold the FP64 state after one application, bits_all[0] its
        # measured bits): flipped measurement bits, and the amplitude error when
        # every bit agrees
        d32r = torch.empty(1 << n, dtype=torch.float32).pin_memory()
        d32i = torch.empty(1 << n, dtype=torch.float32).pin_memory()
        st32.download(d32r.data_ptr(), d32i.data_ptr())
        flipped = sum(1 for a, b in zip(bits32, bits_all[0]) if a != b)
        fp32_err = None
        if flipped == 0:
            r64 = o_re.numpy()
            i64 = o_im.numpy()
            dr = d32r.numpy().astype(np.float64) - r64
            di = d32i.numpy().astype(np.float64) - i64
            nrm = math.sqrt(float(np.dot(r64, r64)) + float(np.dot(i64, i64)))
            amax = float(np.sqrt(np.max(r64 * r64 + i64 * i64)))
            emax = float(np.sqrt(np.max(dr * dr + di * di)))
            fp32_err = {"normwise_rel": math.sqrt(float(np.dot(dr, dr)) + float(np.dot(di, di))) / nrm,
                        "max_abs_over_max_amplitude": emax / amax}
            del dr, di
        del d32r, d32i
        st32.flush()
        torch.cuda.synchronize()
        st32.set_timing(True)
        st32.kernel_time()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            apply_circuit(st32, gates)
        st32.flush()
        f1.record(stream)
        torch.cuda.synchronize()
        ms32 = f0.elapsed_time(f1) / args.steps
        k32, l32, b32 = st32.kernel_time()
        alg32 = algorithmic_bytes(gates, n, 8)
        fp32_line = {"value": alg32 / (ms32 / 1e3) / 1e9, "unit": "GB/s", "ms_per_step": ms32,
                     "vs_fp64": {"measured_bits": len(bits32), "flipped_bits": flipped,
                                 "amplitude_error": fp32_err,
                                 "against": "the FP64 GPU result of the same circuit and initial state (FP64 is "
                                            "the oracle-pinned path)"},
                     "gates_per_s": len([g for g in gates if g[0] != "measure"]) / (ms32 / 1e3),
                     "pass_kernel_gbs": b32 / (k32 / 1e3) / 1e9 if k32 > 0 else None}
        # dense blocks on the tensor cores: a QFT-heavy FP32 circuit (40 QFT /
        # inverse-QFT pairs on random 5-qubit registers, 1200 gates) with automatic
        # dense fusion off and on, from the same state
        rng = np.random.default_rng(3)
        regs = [sorted(int(q) for q in rng.choice(n, size=5, replace=False)) for _ in range(40)]

        def qft_circuit(sx):
            for r in regs:
                sx.apply_qft(r)
                sx.apply_qft_inverse(r[::-1])

        dense = {}
        outs = {}
        for fusion in (0, 4):
            st32.set_dense_fusion(fusion)
            st32.upload(h32r.data_ptr(), h32i.data_ptr())
            qft_circuit(st32)
            st32.synchronize()
            st32.reset_stats()
            st32.set_timing(True)
            st32.kernel_time()
            q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            q0.record(stream)
            for _ in range(args.steps):
                qft_circuit(st32)
            st32.flush()
            q1.record(stream)
            torch.cuda.synchronize()
            kq, lq, bq = st32.kernel_time()
            st32.set_timing(False)
            sq = st32.stats()
            dense[f"fusion_{fusion}"] = {"ms_per_step": q0.elapsed_time(q1) / args.steps,
                                         "passes_per_step": sq["passes"] / args.steps,
                                         "pass_kernel_gbs": bq / (kq / 1e3) / 1e9 if kq > 0 else None}
            st32.upload(h32r.data_ptr(), h32i.data_ptr())
            qft_circuit(st32)
            outs[fusion] = st32.get_state()
        st32.set_dense_fusion(0)
        a0, a4 = outs[0], outs[4]
        dense["speedup"] = dense["fusion_0"]["ms_per_step"] / dense["fusion_4"]["ms_per_step"]
        dense["max_abs_diff_over_max_amplitude"] = float(np.max(np.abs(a4 - a0)) / np.max(np.abs(a0)))
        dense["workload"] = (f"{n}-qubit FP32 state, 40 QFT + inverse-QFT pairs on random 5-qubit registers "
                             f"(1200 gates); dense blocks by tcgen05 (TF32 high/remainder split, four products)")
        del outs, a0, a4
        fp32_line["dense_blocks"] = dense
        st32.close()
        del h32r, h32i
        st = None

    # secondary: the same gate mix on a 30-qubit FP64 state (16 GiB), device-resident
    # (the state is drawn on the device: re, im ~ N(0, 1) from torch's seeded
    # generator, normalised in FP64), one warm-up and one timed pass of 1000 gates
    n30_line = None
    if args.precision == "f64" and rank == 0 and not args.skip_30 and n < 30:
        n30 = 30
        g30 = random_circuit(n30, args.gates, seed=7)
        st30 = State(n30, "f64")
        st30.set_stream(stream.cuda_stream)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(7)
        pre, pim = st30.device_ptrs()
        N30 = 1 << n30
        nrm2 = 0.0
        for ptr in (pre, pim):
            t = torch.randn(N30, dtype=torch.float64, device="cuda", generator=gen)
            nrm2 += float((t * t).sum())
            torch.as_tensor(_DeviceArray(ptr, N30), device="cuda").copy_(t)
            del t
        nrm = nrm2 ** 0.5
        for ptr in (pre, pim):
            torch.as_tensor(_DeviceArray(ptr, N30), device="cuda").div_(nrm)
        torch.cuda.synchronize()
        apply_circuit(st30, g30)
        st30.flush()
        torch.cuda.synchronize()
        st30.set_timing(True)
        st30.kernel_time()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        apply_circuit(st30, g30)
        st30.flush()
        f1.record(stream)
        torch.cuda.synchronize()
        ms30 = f0.elapsed_time(f1)
        k30, l30, b30 = st30.kernel_time()
        alg30 = algorithmic_bytes(g30, n30, 16)
        n30_line = {"value": alg30 / (ms30 / 1e3) / 1e9, "unit": "GB/s", "ms_per_step": ms30,
                    "n_qubits": n30, "state_gib": 16, "steps": 1, "warmup": 1,
                    "gates_per_s": len([g for g in g30 if g[0] != "measure"]) / (ms30 / 1e3),
                    "pass_kernel_gbs": b30 / (k30 / 1e3) / 1e9 if k30 > 0 else None,
                    "pass_kernel_frac_of_hbm": (b30 / (k30 / 1e3) / 1e9 / peak) if (k30 > 0 and peak) else None,
                    "state": "device-drawn N(0,1), torch generator seed 7, normalised"}
        st30.close()

    qms = None
    if rank == 0 and not args.skip_qms:
        qms = qms_section(args.qms_chains, args.qms_steps)
        qms["config1_triangle"] = config1_section()
    qsa = None
    if rank == 0 and not args.skip_qsa:
        qsa = qsa_section(args.qsa_walks, args.qsa_steps, cpu=not args.skip_cpu)

    if rank == 0:
        cpu = None
        if not args.skip_cpu:
            v, done, threads, dt = cpu_baseline(n, gates, args.cpu_seconds, bpa)
            cpu = {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                   "sample": f"first {done} of {len(gates)} ops of the same {n}-qubit circuit, {dt:.1f} s"}
        line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
                "config": {"workload": f"random circuit, {n} qubits {args.precision.upper()}, {args.gates} gates "
                                       f"(X, H, CX, MCX 2-4 controls, U1, Pauli rotations on 2-6 qubits), "
                                       f"measure every 100; seed 7",
                           "n_qubits": n, "gates": args.gates, "fusion": not args.no_fusion,
                           "parallelism": f"replicas x{world}", "l2": "state (%d MiB) larger than L2" % (state_bytes >> 20)},
                "gates_per_s": (len([g for g in gates if g[0] != 'measure']) * world) / (ms_step / 1e3),
                "passes_per_step": stats["passes"] / args.steps,
                "gpu_launches": stats["launches"],
                "clocks": clk.summary(),
                "e2e": {"value": e2e_value, "unit": "GB/s", "ms_per_step": ms_e2e,
                        "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes,
                        "mode": "pipelined: two states on two streams and host threads, each step uploads "
                                "its input, runs the circuit, downloads its state; circuits take turns, one "
                                "state's copies overlap the other state's circuit",
                        "steps": pipe_steps,
                        "same_measured_bits": pipe_ok,
                        "parts": e2e_parts},
                "e2e_serial": {"value": alg * world / (ms_e2e_serial / 1e3) / 1e9, "unit": "GB/s",
                               "ms_per_step": ms_e2e_serial, "mode": "one state: upload, circuit, download in turn"},
                "roofline": roofline,
                "cpu_baseline": cpu,
                "fp32_same_circuit": fp32_line,
                "fp64_double_float": df_line,
                "fp64_30_qubits": n30_line,
                "qms_batched": qms,
                "qsa_walks": qsa}
        print(json.dumps(line), flush=True)
    if st is not None:
        st.close()
    if dist is not None:
        dist.destroy_process_group()


class _DeviceArray:
    """A device buffer of doubles owned by libsq, exposed to torch without a copy."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3}


def fp64_fma_rate():
    """FP64 FMA instructions per second (G/s) of this GPU's CUDA cores, from the
    benchmark's probe library (suqa_gb300/_build/libsq_probe.so), or None."""
    import ctypes
    try:
        lib = ctypes.CDLL(os.path.join(ROOT, "suqa_gb300", "_build", "libsq_probe.so"))
        lib.sqb_fp64_fma_rate.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)]
        g = ctypes.c_double()
        if lib.sqb_fp64_fma_rate(ctypes.byref(g), None) == 0:
            return g.value
    except OSError:
        pass
    return None


def traffic_per_launch():
    """DRAM bytes per launch of the pass kernel from the committed ncu summary
    (profiles/k_pass_f64_n28.txt, line 'traffic_per_launch_bytes: X'), if any."""
    p = os.path.join(ROOT, "profiles", "k_pass_f64_n28.txt")
    try:
        for ln in open(p):
            if ln.startswith("traffic_per_launch_bytes:"):
                return float(ln.split(":", 1)[1])
    except OSError:
        pass
    return None


if __name__ == "__main__":
    main()
