"""Writes tests/golden/crmath.npz: arguments of exp, log, sin, cos and acos
over the ranges QUATERNION::pow meets (and the hard ones around them), each
with its correctly rounded value (mpmath at 200 bits, rounded to nearest
even) and the value of this machine's C library (the reference build's).

    python tests/golden/gen_crmath.py
"""
import math
import os

import mpmath
import numpy as np

mpmath.mp.prec = 200
N = 1000


def args(rng):
    sgn = lambda n: rng.choice([-1.0, 1.0], n)  # noqa: E731
    return {
        "exp": np.concatenate([rng.uniform(-20, 20, N), rng.uniform(-745, 709.7, N // 2),
                               rng.uniform(-1e-3, 1e-3, N // 4),
                               np.exp(rng.uniform(-700, 0, N // 4)) * sgn(N // 4)]),
        "log": np.concatenate([np.exp(rng.uniform(-7, 7, N)), 1 + rng.uniform(-1e-3, 1e-3, N // 2),
                               np.exp(rng.uniform(-700, 700, N // 4)),
                               np.exp(rng.uniform(-744, -708, N // 4))]),
        "sin": np.concatenate([rng.uniform(0, 10, N), rng.uniform(-1e5, 1e5, N // 2),
                               rng.uniform(-1e-3, 1e-3, N // 4),
                               np.pi / 2 * rng.randint(1, 1000, N // 4) +
                               rng.uniform(-1e-6, 1e-6, N // 4)]),
        "cos": np.concatenate([rng.uniform(0, 10, N), rng.uniform(-1e5, 1e5, N // 2),
                               rng.uniform(-1e-3, 1e-3, N // 4),
                               np.pi / 2 * rng.randint(1, 1000, N // 4) +
                               rng.uniform(-1e-6, 1e-6, N // 4)]),
        "acos": np.concatenate([rng.uniform(-1, 1, N), 1 - np.exp(rng.uniform(-36, 0, N // 2)),
                                -1 + np.exp(rng.uniform(-36, 0, N // 4)),
                                rng.uniform(-1e-3, 1e-3, N // 4)]),
    }


def main():
    rng = np.random.RandomState(2024)
    out = {}
    for name, x in args(rng).items():
        f = getattr(mpmath, name)
        out[name + "_x"] = x
        out[name + "_cr"] = np.array([float(f(mpmath.mpf(float(v)))) for v in x])
        out[name + "_libc"] = np.array([getattr(math, name)(float(v)) for v in x])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "crmath.npz")
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    main()
