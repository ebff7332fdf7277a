"""visc_mixed (csrc/des_mixed.cu): the mixed step's Arrhenius viscosity,
restated in numpy and checked against the FP64 law of MatProps::visc
(matprops.cxx:276-312) for one material.

    ln visc = ln(0.25e6 coef) + pw ln(edot_II) + Q / (n R T)

with ln(edot_II) = logf(mantissa) + exponent ln 2, 1/T from an FP32 seed
and one FP64 Newton step, and exp(ln visc) = 2^k expf(r), |r| <= ln2/2.
The kernel's comment claims ~2e-7 relative error against the FP64 law.
Here numpy's FP32 log and exp stand in for CUDA's logf and expf (both
within a few ulp of the exact values), the fused multiply-adds are the C
library's fma, and the FP32 operations are numpy's IEEE float32 ones."""
import ctypes
import ctypes.util
import math

import numpy as np

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.fma.restype = ctypes.c_double
_libm.fma.argtypes = (ctypes.c_double,) * 3
fma = _libm.fma
F = np.float32
LN2 = 0.6931471805599453
R_GAS = 8.3144


def _material(n=3.0, Q=2e5, A=1e-7, vmin=1e18, vmax=1e24):
    coef = (0.75 * A) ** (-1 / n)
    return dict(n=n, Q=Q, coef=coef, pw=1 / n - 1, vmin=vmin, vmax=vmax, lnc=math.log(0.25e6 * coef),
                lnmin=math.log(vmin), lnmax=math.log(vmax), qnr=Q / (n * R_GAS))


def visc_fp64(mat, edot, T):
    a = (edot[0] + edot[1] + edot[2]) / 3
    j2 = 0.5 * ((edot[0] - a) ** 2 + (edot[1] - a) ** 2 + (edot[2] - a) ** 2) + edot[3] ** 2 + edot[4] ** 2 + edot[5] ** 2
    ed = max(math.sqrt(j2), 1e-30)
    visc0 = 0.25 * ed ** mat["pw"] * mat["coef"] * math.exp(mat["Q"] / (mat["n"] * R_GAS * T)) * 1e6
    return min(max(1 / (1 / visc0), mat["vmin"]), mat["vmax"])


def visc_mixed(mat, edot, T):
    t = [F(x) for x in edot]
    a = (t[0] + t[1] + t[2]) * (F(1) / F(3))
    j2 = F(0.5) * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a)) \
        + t[3] * t[3] + t[4] * t[4] + t[5] * t[5]
    ed = max(np.sqrt(j2), F(1e-30))
    mant, ex = np.frexp(ed)
    ln_ed = fma(float(ex), LN2, float(np.log(F(mant))))
    r = float(F(1) / F(T))
    r = r * fma(-T, r, 2.0)
    lnv = fma(mat["qnr"], r, fma(mat["pw"], ln_ed, mat["lnc"]))
    if lnv <= mat["lnmin"]:
        return mat["vmin"]
    if lnv >= mat["lnmax"]:
        return mat["vmax"]
    kf = float(min(max(np.rint(F(lnv) * F(1.44269504)), F(-1000)), F(1000)))
    rr = F(fma(-kf, LN2, lnv))
    m = float(np.exp(rr))
    return math.ldexp(m, int(kf))


def _cases(rng, n):
    for _ in range(n):
        T = rng.uniform(273.0, 1700.0)
        mag = 10 ** rng.uniform(-18, -11)
        e = rng.standard_normal(6) * mag
        yield list(e), T


def test_within_3e_minus_7_of_the_fp64_law():
    rng = np.random.default_rng(6)
    mat = _material()
    worst, inside = 0.0, 0
    for e, T in _cases(rng, 20_000):
        v64 = visc_fp64(mat, e, T)
        if not (mat["vmin"] < v64 < mat["vmax"]):
            continue
        inside += 1
        worst = max(worst, abs(visc_mixed(mat, e, T) - v64) / v64)
    assert inside > 5000
    assert worst < 3e-7, worst


def test_clamps_are_exact():
    rng = np.random.default_rng(7)
    mat = _material()
    for e, T in _cases(rng, 5_000):
        v64 = visc_fp64(mat, e, T)
        vm = visc_mixed(mat, e, T)
        if v64 == mat["vmax"] and vm >= mat["vmax"] * (1 - 1e-6):
            assert vm == mat["vmax"] or abs(vm - v64) / v64 < 3e-7
        if v64 == mat["vmin"] and vm <= mat["vmin"] * (1 + 1e-6):
            assert vm == mat["vmin"] or abs(vm - v64) / v64 < 3e-7


def test_other_laws():
    """Other exponents and activation energies (n = 3.05, Q = 376 kJ/mol:
    the default material; n = 1, a linear law)."""
    rng = np.random.default_rng(8)
    for mat in (_material(n=3.05, Q=3.76e5, A=1.25e-1), _material(n=1.0, Q=1.5e5, A=1e-6)):
        worst = 0.0
        for e, T in _cases(rng, 5_000):
            v64 = visc_fp64(mat, e, T)
            if mat["vmin"] < v64 < mat["vmax"]:
                worst = max(worst, abs(visc_mixed(mat, e, T) - v64) / v64)
        assert worst < 3e-7, (mat["n"], worst)


def test_maxwell_coefficients_in_fp32():
    """maxwell_coef (csrc/des_mixed.cu): tmp = dt G / (2 visc) and
    f2 - 1 = -tmp / (1 + tmp) formed in FP32, each within ~2^-22 of itself
    (2^-21 asserted), over the time steps, moduli and viscosities of the
    workloads and beyond."""
    rng = np.random.default_rng(9)
    worst_t = worst_u = 0.0
    for _ in range(20_000):
        dt = 10 ** rng.uniform(3, 9)
        G = 10 ** rng.uniform(9, 11.5)
        visc = 10 ** rng.uniform(17, 25)
        tf = (F(0.5) * F(dt) * F(G)) / F(visc)
        uf = -tf / (F(1) + tf)
        tmp = 0.5 * dt * G / visc
        u = -tmp / (1 + tmp)
        worst_t = max(worst_t, abs(float(tf) - tmp) / tmp)
        worst_u = max(worst_u, abs(float(uf) - u) / abs(u))
    assert worst_t < 2.0 ** -21 and worst_u < 2.0 ** -21, (worst_t, worst_u)
