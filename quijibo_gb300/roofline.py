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
