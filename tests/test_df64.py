"""The double-float arithmetic of the FP64 tile pass (suqa_gb300/csrc/sq_df64.cuh),
compiled for the host and checked against IEEE double arithmetic on random
operands over the magnitudes a state vector holds: double -> df64 -> double
round trips, sums, differences, products and fused multiply-adds."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r'''
#include "sq_df64.cuh"
#include <cstdio>
#include <cstdlib>
#include <random>
using namespace sqk;
int main() {
    std::mt19937_64 g(7);
    // amplitudes from 2^-60 to 16 (stored amplitudes carry the state's global
    // scale), gate coefficients (cos, sin, tan, 1/sqrt 2 ...) from 2^-8 to 2
    std::uniform_real_distribution<double> u(-1.0, 1.0), ex(-60.0, 4.0), exc(-8.0, 1.0);
    auto draw = [&]() { return u(g) * std::exp2(ex(g)); };
    auto coef = [&]() { return u(g) * std::exp2(exc(g)); };
    double rt = 0, add = 0, mul = 0, fmad = 0, canc = 0;
    long zero_ok = 1;
    for (int i = 0; i < 2000000; ++i) {
        const double a = draw(), b = draw(), c = draw(), k = coef();
        const df64 A = df_from_double(a), B = df_from_double(b), C = df_from_double(c), Kc = df_from_double(k);
        rt = std::fmax(rt, std::fabs(df_to_double(A) - a) / std::fabs(a));
        const double s = df_to_double(df_add(A, B));
        add = std::fmax(add, std::fabs(s - (a + b)) / (std::fabs(a) + std::fabs(b)));
        const double p = df_to_double(df_mul(A, Kc));
        mul = std::fmax(mul, std::fabs(p - a * k) / std::fabs(a * k));
        const double f = df_to_double(df_fmadd(A, Kc, C));
        fmad = std::fmax(fmad, std::fabs(f - std::fma(a, k, c)) / (std::fabs(a * k) + std::fabs(c)));
        // cancellation: a - (a + tiny)
        const double t = a * 1e-9;
        const double d = df_to_double(df_sub(A, df_from_double(a + t)));
        canc = std::fmax(canc, std::fabs(d - (a - (a + t))) / std::fabs(a));
    }
    zero_ok = df_to_double(df_from_double(0.0)) == 0.0 && df_to_double(df_from_double(-0.0)) == 0.0;
    std::printf("%.3e %.3e %.3e %.3e %.3e %ld\n", rt, add, mul, fmad, canc, zero_ok);
    return 0;
}
'''


def test_df64_against_double(tmp_path):
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "suqa_gb300", "csrc"),
           str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr[-3000:])
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    rt, add, mul, fmad, canc = (float(x) for x in out[:5])
    assert int(out[5]) == 1
    # 48 significand bits: round trips within 2^-47; an operation (with the
    # conversions of its operands) within a few units of 2^-48
    assert rt <= 2.0 ** -47, rt
    assert add <= 2.0 ** -45, add
    assert mul <= 2.0 ** -43, mul
    assert fmad <= 2.0 ** -43, fmad
    assert canc <= 2.0 ** -45, canc
