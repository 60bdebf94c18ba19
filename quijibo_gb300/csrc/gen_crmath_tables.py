"""Writes qj_crmath_tables.h: the constants and tables of the correctly
rounded FP64 transcendentals in qj_crmath.h, computed here with mpmath at
300 bits and rounded to double-double pairs (hi = RN(v), lo = RN(v - hi)).

    python quijibo_gb300/csrc/gen_crmath_tables.py

Every value is a mathematical constant (powers of two, logarithms, sines,
cosines and arctangents at table points; pi and ln 2 split for Cody-Waite
reduction; Taylor coefficients 1/n!), so the table is the same on every
machine that runs this script.
"""
import os

import mpmath

mpmath.mp.prec = 300


def rn(v):
    return float(v)  # mpmath rounds to nearest even when converting


def dd(v):
    hi = rn(v)
    lo = rn(v - mpmath.mpf(hi))
    return hi, lo


def trunc_bits(v, bits):
    """v truncated to `bits` significant bits (toward zero)."""
    m, e = mpmath.frexp(v)  # v = m * 2^e, 0.5 <= |m| < 1
    scaled = mpmath.floor(abs(m) * 2 ** bits)
    r = mpmath.ldexp(scaled, e - bits)
    return float(r if v >= 0 else -r)


def hx(x):
    return float(x).hex()


def pair(p):
    return "{%s, %s}" % (hx(p[0]), hx(p[1]))


def main():
    out = []
    w = out.append
    w("// Generated by gen_crmath_tables.py (mpmath, 300 bits): do not edit.")
    w("// Double-double pairs {hi, lo}: hi = RN(v), lo = RN(v - hi).")
    w("#pragma once")
    w("")
    ln2 = mpmath.log(2)
    pi = mpmath.pi
    # exp: x = k ln2/64 + r; ln2/64 as L1 (36 bits, so k*L1 is exact for
    # |k| < 2^17) + L2 + L3
    c = ln2 / 64
    L1 = trunc_bits(c, 36)
    L2 = rn(c - L1)
    L3 = rn(c - L1 - L2)
    w("#define CRM_INV_LN2_64 %s" % hx(rn(64 / ln2)))
    w("#define CRM_LN2_64_1 %s" % hx(L1))
    w("#define CRM_LN2_64_2 %s" % hx(L2))
    w("#define CRM_LN2_64_3 %s" % hx(L3))
    lh, ll = dd(ln2)
    w("#define CRM_LN2_HI %s" % hx(lh))
    w("#define CRM_LN2_LO %s" % hx(ll))
    # pi/2 in 33 + 33 + 53 + 53 bits: k*P1 and k*P2 exact for |k| < 2^20
    h = pi / 2
    P1 = trunc_bits(h, 33)
    P2 = trunc_bits(h - P1, 33)
    P3 = rn(h - P1 - P2)
    P4 = rn(h - P1 - P2 - P3)
    w("#define CRM_2_PI %s" % hx(rn(2 / pi)))
    for i, v in enumerate((P1, P2, P3, P4), 1):
        w("#define CRM_PIO2_%d %s" % (i, hx(v)))
    ph, pl = dd(pi)
    w("#define CRM_PI_HI %s" % hx(ph))
    w("#define CRM_PI_LO %s" % hx(pl))
    w("")
    w("// 1/n! for n = 0..16")
    w("CRM_TAB crm_dd crm_inv_fact[17] = {")
    w(",\n".join("    " + pair(dd(1 / mpmath.factorial(n))) for n in range(17)) + "};")
    w("// 1/n for n = 0..16 (entry 0 unused)")
    w("CRM_TAB crm_dd crm_inv_n[17] = {")
    w(",\n".join("    " + pair(dd(1 / mpmath.mpf(n)) if n else (0.0, 0.0)) for n in range(17)) + "};")
    w("// 2^(j/64)")
    w("CRM_TAB crm_dd crm_exp2_64[64] = {")
    w(",\n".join("    " + pair(dd(mpmath.power(2, mpmath.mpf(j) / 64))) for j in range(64)) + "};")
    # log: entry i + 128 b covers y in [(1 + i/128) / 2^b, (1 + (i+1)/128) / 2^b);
    # inv = RN(1 / centre), exactly 1 on the two intervals next to y = 1
    inv = []
    nlog = []
    for b in (0, 1):
        for i in range(128):
            lo_ = (1 + mpmath.mpf(i) / 128) / 2 ** b
            ctr = (1 + (mpmath.mpf(i) + 0.5) / 128) / 2 ** b
            if (b == 0 and i == 0) or (b == 1 and i == 127):
                v = 1.0
            else:
                v = rn(1 / ctr)
            del lo_
            inv.append(v)
            nlog.append(dd(-mpmath.log(mpmath.mpf(v))) if v != 1.0 else (0.0, 0.0))
    w("// log: 1 / (centre of the interval), and -log of it")
    w("CRM_TAB double crm_log_inv[256] = {")
    w(",\n".join("    " + ", ".join(hx(v) for v in inv[k:k + 4]) for k in range(0, 256, 4)) + "};")
    w("CRM_TAB crm_dd crm_log_neg[256] = {")
    w(",\n".join("    " + pair(p) for p in nlog) + "};")
    w("// sin(j/64), cos(j/64)")
    w("CRM_TAB crm_dd crm_sin_64[52] = {")
    w(",\n".join("    " + pair(dd(mpmath.sin(mpmath.mpf(j) / 64))) for j in range(52)) + "};")
    w("CRM_TAB crm_dd crm_cos_64[52] = {")
    w(",\n".join("    " + pair(dd(mpmath.cos(mpmath.mpf(j) / 64))) for j in range(52)) + "};")
    w("// atan(j/64)")
    w("CRM_TAB crm_dd crm_atan_64[65] = {")
    w(",\n".join("    " + pair(dd(mpmath.atan(mpmath.mpf(j) / 64))) for j in range(65)) + "};")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "qj_crmath_tables.h")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
