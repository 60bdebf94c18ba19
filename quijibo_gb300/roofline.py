"""Algorithmic work counts of the field kernels, for the roofline figures of
bench.py and quijibo_gb300.benchmarks."""


def field_flops(rs, voxel_iters, de=True):
    """Algorithmic FP32 flops of `voxel_iters` map applications (FMA = 2).

    Per root term: 4 (q - r) + 11 per squaring (exponent 2) + 28 per
    accumulating Hamilton product (the first root of each product has none)
    + 16 for the distance-estimate gradient term (|d|^2 7, divide 1, 4 FMA 8).
    Per application: T * conj(B) 28, |B|^2 7, s/|B|^2 1, scaling 4, |q|^2 7,
    and with the estimate |g|^2 7 + two logs and their sum 3 (10)."""
    per = 0
    for pw, n in ((rs.top_powers, rs.n_top), (rs.bottom_powers, rs.n_bottom)):
        if n == 0:
            continue
        per += 4 * n + 28 * (n - 1) + sum(11 * (int(e) - 1) for e in pw)
        if de:
            per += 16 * n
    per += (28 + 7 + 1 if rs.n_bottom else 0) + 4 + 7 + (10 if de else 0)
    return per * voxel_iters


# Algorithmic counts of the squared-error energy (energy.cu), FP32 form.
# Divisions count as one flop; the transcendental calls (log2, exp2, atan2,
# sincospi, rsqrt in the polar power; the logs of |g| and |Q|; the square
# root of the escape test) are tallied apart as special operations.
#
# Forward, per root term: q - r 4, |d|^2 7, e / |d|^2 1, g += k d 8, polar
# power 18 (|v|^2 5, |d|^2 2, |v| 1, e log 2, e theta / pi 2, A s / |v| 2,
# A c 1, k v 3), Hamilton product 28 (none for the first root of each side).
# Per map application: conj(B) / |B|^2 12, T W 28, scaling 4 (with bottom
# roots; scaling alone without), log|g| 8, L update 10, |q|^2 of the escape
# test 7.
SQ_FWD_ROOT = 4 + 7 + 1 + 8 + 18 + 28
SQ_FWD_SPECIAL_ROOT = 5


def sq_forward_app_flops(nt, nb):
    sides = 2 if nb else 1
    per = SQ_FWD_ROOT * (nt + nb) - 28 * sides
    per += (12 + 28 + 4 if nb else 4) + 8 + 10 + 7
    return per


# Adjoint, per orbit step: the step's map application at the forward pass's
# kept q_n (its factors and prefix products), then per root term: the
# log|g| gradient loop 20, q - r 4, polar power 18, the prefix-product
# adjoint conj(F) U 28 and U conj(P) 28, the polar power's vector-Jacobian
# product 57, the log|g| term 40, the sums of the five components over the
# samples 5, the running q-bar 4; per step: Q-bar 16, d/d log s 7, the
# quotient's adjoint (conj(B) / |B|^2, two products, B-bar) 136 with bottom
# roots, g-bar 12.
SQ_BWD_ROOT = 20 + 4 + 18 + 28 + 28 + 57 + 40 + 5 + 4
SQ_BWD_SPECIAL_ROOT = 6


def sq_backward_step_flops(nt, nb):
    return sq_forward_app_flops(nt, nb) + SQ_BWD_ROOT * (nt + nb) + 16 + 7 + (136 if nb else 0) + 12


def energy_flops(nt, nb, applications, steps=0):
    """(flops, special operations) of an energy call with `applications`
    forward map applications and `steps` adjoint orbit steps."""
    nr = nt + nb
    flops = applications * sq_forward_app_flops(nt, nb) + steps * sq_backward_step_flops(nt, nb)
    special = applications * (SQ_FWD_SPECIAL_ROOT * nr + 4)
    special += steps * ((SQ_FWD_SPECIAL_ROOT * nr + 4) + SQ_BWD_SPECIAL_ROOT * nr)
    return flops, special
