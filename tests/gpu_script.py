"""Runs a dumper-grammar gate script through the GPU engine (suqa_gb300.State),
producing results in the same order as oracle.run_script / the golden dumper."""
from __future__ import annotations

import math

import numpy as np

from suqa_gb300 import State


def _lst(a, i):
    k = int(a[i])
    return [int(x) for x in a[i + 1:i + 1 + k]], i + 1 + k


def _ph(x):
    return float.fromhex(x) if ("0x" in x or "0X" in x) else float(x)


def run_script(lines, precision="f64", fusion=True, dense_fusion=0, dfloat=False):
    st = None
    out = []
    it = iter(lines)
    for line in it:
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        tok = line.split()
        cmd, a = tok[0], tok[1:]
        if cmd == "setup":
            if st is not None:
                st.close()
            st = State(int(a[0]), precision)
            st.set_fusion(fusion)
            if dense_fusion:
                st.set_dense_fusion(dense_fusion)
            if dfloat:
                st.set_double_float(True)
            continue
        if cmd == "setstate":
            vals = np.array([float.fromhex(v) for v in next(it).split()])
            N = st.size()
            st.set_state(vals[:N] + 1j * vals[N:])
            continue
        r = apply(st, cmd, a)
        if r is not None:
            out.append(r)
    if st is not None:
        st.close()
    return out


def apply(st: State, cmd, a):
    if cmd == "init":
        st.init_state()
    elif cmd == "vnorm":
        return ("N", st.vnorm())
    elif cmd == "normalize":
        st.vnormalize()
    elif cmd == "dump":
        return ("S", st.get_state())
    elif cmd == "gc_on":
        st.activate_gc_mask(_lst(a, 0)[0])
    elif cmd == "gc_off":
        st.deactivate_gc_mask(_lst(a, 0)[0])
    elif cmd in ("x", "y", "z", "h", "s", "t", "tdg"):
        getattr(st, "apply_" + cmd)(int(a[0]))
    elif cmd == "u1":
        st.apply_u1(int(a[0]), _ph(a[1]))
    elif cmd == "u1m":
        st.apply_u1(int(a[0]), int(a[1]), _ph(a[2]))
    elif cmd == "cx":
        st.apply_cx(int(a[0]), int(a[1]), int(a[2]))
    elif cmd in ("mcx", "mcxm"):
        cs, i = _lst(a, 0)
        if cmd == "mcxm":
            ms = [int(x) for x in a[i:i + len(cs)]]
            st.apply_mcx(cs, ms, int(a[i + len(cs)]))
        else:
            st.apply_mcx(cs, int(a[i]))
    elif cmd == "cu1":
        st.apply_cu1(int(a[0]), int(a[1]), _ph(a[2]), int(a[3]))
    elif cmd in ("mcu1", "mcu1m"):
        cs, i = _lst(a, 0)
        if cmd == "mcu1m":
            ms = [int(x) for x in a[i:i + len(cs)]]
            i += len(cs)
            st.apply_mcu1(cs, ms, int(a[i]), _ph(a[i + 1]))
        else:
            st.apply_mcu1(cs, int(a[i]), _ph(a[i + 1]))
    elif cmd == "swap":
        st.apply_swap(int(a[0]), int(a[1]))
    elif cmd in ("ptp", "ptpg"):
        qs, i = _lst(a, 0)
        ps = [int(x) for x in a[i:i + len(qs)]]
        ph = _ph(a[i + len(qs)])
        if cmd == "ptp":
            try:
                st.apply_pauli_TP_rotation(qs, ps, ph)
            except RuntimeError:
                return ("E", "unsupported pauli rotation")
        else:
            st.apply_pauli_rotation(qs, ps, ph)
    elif cmd == "plist":
        q0, qsz = int(a[0]), int(a[1])
        st.apply_phase_list(q0, qsz, [_ph(x) for x in a[2:2 + (1 << qsz)]])
    elif cmd == "qft":
        st.apply_qft(_lst(a, 0)[0])
    elif cmd == "iqft":
        st.apply_qft_inverse(_lst(a, 0)[0])
    elif cmd == "measure":
        return ("M", st.measure_qbit(int(a[0]), _ph(a[1])))
    elif cmd == "reset":
        st.apply_reset(int(a[0]), _ph(a[1]))
    elif cmd == "prob":
        qs, i = _lst(a, 0)
        return ("P", st.prob_filter(qs, [int(x) for x in a[i:i + len(qs)]]))
    else:
        raise ValueError(f"unknown command {cmd}")
    return None
