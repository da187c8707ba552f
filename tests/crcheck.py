"""Inputs and float64 references for the correctly rounded library functions
(crmath.cuh): std::sin / std::cos of the sampling angles 2 pi u
(RandomSampler.h:87-103), std::asin / std::acos of the background lookup
(HdrBackground.cpp:61-63), std::pow(x, 5) and std::pow(x, -2) of the Fresnel
and GGX terms (BRDFModel.h:44-80).

The reference value of a float input is the float64 evaluation rounded once to
float32.  float64 sin, asin, ... are within a few units of 2^-53 relative, so
that rounding is the correctly rounded float32 except where the float64 value
lies within a few float64 ulps of a float32 rounding midpoint: those inputs are
reported as ambiguous and left out of the comparison.  x^5 and x^-2 are
rational, so their ambiguous inputs (and exact midpoints, which round to even)
are decided exactly with fractions instead."""
import math
import os
import subprocess

import numpy as np

SIN, COS, ASIN, ACOS, POW5, POW_M2 = range(6)
NAMES = ["sin", "cos", "asin", "acos", "pow5", "pow_m2"]


def _near_multiples(step: float, kmax: int, lo: float, hi: float, spread: int, rng, n: int) -> np.ndarray:
    """floats within `spread` ulps of k * step (k = 1..kmax) inside [lo, hi]:
    the arguments whose reduction cancels the most bits"""
    k = rng.integers(1, kmax + 1, n)
    c = np.float32(k * step)
    off = rng.integers(-spread, spread + 1, n).astype(np.int64)
    x = (c.view(np.int32).astype(np.int64) + off).astype(np.int32).view(np.float32)
    return x[(x >= lo) & (x <= hi)]


def inputs(fn: int, n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed + 101 * fn)
    if fn in (SIN, COS):
        # the angles 2 pi u of the samplers: [0, 2 pi) and a little beyond (8)
        parts = [rng.uniform(0.0, 8.0, n).astype(np.float32),
                 np.float32(2.0 * math.pi) * rng.uniform(0.0, 1.0, n // 4).astype(np.float32),
                 _near_multiples(math.pi / 2, 5, 0.0, 8.0, 2000, rng, n // 4),
                 _near_multiples(math.pi / 32, 80, 0.0, 8.0, 200, rng, n // 8),
                 np.exp2(rng.uniform(-30, 0, n // 8)).astype(np.float32)]
    elif fn in (ASIN, ACOS):
        parts = [rng.uniform(-1.0, 1.0, n).astype(np.float32),
                 (1.0 - np.exp2(rng.uniform(-24, -1, n // 4))).astype(np.float32) * rng.choice([-1, 1], n // 4),
                 (np.exp2(rng.uniform(-30, -1, n // 4)) * rng.choice([-1, 1], n // 4)).astype(np.float32),
                 np.array([-1.0, -0.5, 0.0, 0.5, 1.0], np.float32)]
    elif fn == POW5:
        # (1 - cos) of the Schlick term: [0, 1]; correctly rounded from 2^-20 up;
        # odd * 2^j with odd <= 31 make x^5 a rounding midpoint exactly (ties)
        ties = np.array([o * 2.0 ** j for o in range(1, 32, 2) for j in range(-25, 1)], np.float32)
        parts = [rng.uniform(2.0 ** -20, 1.0, n).astype(np.float32),
                 np.exp2(rng.uniform(-20, 0, n // 2)).astype(np.float32),
                 ties[(ties >= 2.0 ** -20) & (ties <= 1.0)]]
    else:
        parts = [np.exp2(rng.uniform(-40, 40, n)).astype(np.float32),
                 rng.uniform(0.0, 4.0, n // 2).astype(np.float32)]
        parts = [p[p > 0] for p in parts]
    return np.concatenate(parts).astype(np.float32)


def reference(fn: int, x: np.ndarray):
    """(expected float32 values, mask of inputs whose float64 value is too
    close to a float32 rounding midpoint to decide)"""
    d = x.astype(np.float64)
    if fn == SIN:
        y = np.sin(d)
    elif fn == COS:
        y = np.cos(d)
    elif fn == ASIN:
        y = np.arcsin(d)
    elif fn == ACOS:
        y = np.arccos(d)
    elif fn == POW5:
        y = d * d * d * d * d
    else:
        y = 1.0 / (d * d)
    y32 = y.astype(np.float32)
    # the float32 neighbour on y's far side of y32, and the midpoint between them
    up = np.where(y > y32.astype(np.float64), np.inf, -np.inf).astype(np.float32)
    nb = np.nextafter(y32, up)
    mid = 0.5 * (y32.astype(np.float64) + nb.astype(np.float64))
    amb = np.abs(y - mid) <= 16.0 * np.spacing(np.abs(y))
    if fn in (POW5, POW_M2):  # rational: decide those exactly (ties to even)
        for i in np.flatnonzero(amb):
            y32[i] = _round_exact(fn, float(x[i]))
        amb[:] = False
    return y32, amb


def _round_exact(fn: int, x: float) -> np.float32:
    from fractions import Fraction
    v = Fraction(x) ** 5 if fn == POW5 else 1 / Fraction(x) ** 2
    a = np.float32(float(v))  # within one float32 step of the answer
    best = None
    for c in (np.nextafter(a, np.float32(-np.inf)), a, np.nextafter(a, np.float32(np.inf))):
        d = abs(Fraction(float(c)) - v)
        if best is None or d < best[0] or (d == best[0] and int(c.view(np.uint32)) % 2 == 0):
            best = (d, c)
    return best[1]


HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "openmaterial-validation_gb300", "csrc")

_WRAPPER = r"""
#include "crmath.cuh"
extern "C" void cr_eval(int fn, long n, const float* x, float* y)
{
    for (long i = 0; i < n; ++i) {
        float s = 0.0f, c = 0.0f;
        switch (fn) {
        case 0: omv::cr::sincos_cr(x[i], s, c); y[i] = s; break;
        case 1: omv::cr::sincos_cr(x[i], s, c); y[i] = c; break;
        case 2: y[i] = omv::cr::asin_cr(x[i]); break;
        case 3: y[i] = omv::cr::acos_cr(x[i]); break;
        case 4: y[i] = omv::cr::pow5_cr(x[i]); break;
        default: y[i] = omv::cr::rcp_sq_cr(x[i]); break;
        }
    }
}
"""


def host_library(tmpdir: str):
    """crmath.cuh compiled for the host (g++, no floating-point contraction),
    loaded with ctypes; returns eval(fn, x) -> y"""
    import ctypes as C
    src = os.path.join(tmpdir, "cr_host.cpp")
    lib = os.path.join(tmpdir, "libcr_host.so")
    with open(src, "w") as f:
        f.write(_WRAPPER)
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, src,
                        "-o", lib], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(r.stderr)
    L = C.CDLL(lib)
    fp = C.POINTER(C.c_float)
    L.cr_eval.argtypes = [C.c_int, C.c_long, fp, fp]

    def ev(fn: int, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros_like(x)
        L.cr_eval(fn, len(x), x.ctypes.data_as(fp), y.ctypes.data_as(fp))
        return y
    return ev
