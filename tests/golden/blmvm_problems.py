"""Objectives for the BLMVM solver's parity fixtures (blmvm.npz), written
with Python float arithmetic only (+ - * / and abs), so every machine
computes bit-identical values and the solver's iterates can be compared bit
for bit with the ones the reference's own TAO port produced."""

FLT_MAX = 3.4028234663852886e38


def rosen(x):
    n = len(x)
    f = 0.0
    g = [0.0] * n
    for i in range(n - 1):
        a = x[i + 1] - x[i] * x[i]
        b = 1.0 - x[i]
        f += 100.0 * a * a + b * b
        g[i] += -400.0 * x[i] * a - 2.0 * b
        g[i + 1] += 200.0 * a
    return f, g


def quad(x):
    """0.5 x'Ax - b'x with A = diag(1..n) + 0.1, b evenly from -1 to 2."""
    n = len(x)
    s = 0.0
    for v in x:
        s += v
    f = 0.0
    g = [0.0] * n
    for i in range(n):
        b = -1.0 + 3.0 * i / (n - 1)
        ax = (i + 1.0) * x[i] + 0.1 * s
        f += 0.5 * x[i] * ax - b * x[i]
        g[i] = ax - b
    return f, g


def nanwall(x):
    """quad, not finite once x[1] > 0.9 (the line search backs off)."""
    f, g = quad(x)
    return (float("nan") if x[1] > 0.9 else f), g


def kinks(x):
    """sum |x - 1/2| + 0.01 |x|^2: non-smooth, runs to the iteration limit."""
    f = 0.0
    g = []
    for v in x:
        f += abs(v - 0.5) + 0.01 * v * v
        g.append((1.0 if v > 0.5 else -1.0 if v < 0.5 else 0.0) + 0.02 * v)
    return f, g


def wrong_gradient(x):
    """|x|^2 with the gradient's sign flipped: every line search fails."""
    f = 0.0
    for v in x:
        f += v * v
    return f, [-2.0 * v for v in x]


def pinned(x):
    """sum (x + 1)^2 from x = 0 with x >= 0: optimal on the bounds, so every
    search direction projects to zero and both line searches fail."""
    f = 0.0
    g = []
    for v in x:
        f += (v + 1.0) * (v + 1.0)
        g.append(2.0 * (v + 1.0))
    return f, g


def problems():
    """name -> (objective, x0, lower, upper)."""
    free = -FLT_MAX
    return {
        "rosen2_box": (rosen, [-1.2, 1.0], [-2.0, -2.0], [0.8, 2.0]),
        "rosen7": (rosen, [0.5] * 7, [free] + [0.0] * 6, [FLT_MAX] * 7),
        "rosen5_far": (rosen, [-3.0, -4.0, 5.0, 2.0, 0.1], [free] + [0.0] * 4, [FLT_MAX] * 5),
        "rosen8_box": (rosen, [-2.0 + 4.0 * i / 7 for i in range(8)], [-1.5] * 8, [0.7] * 8),
        "quad12": (quad, [1.0 + 2.0 * i / 11 for i in range(12)], [free] + [0.0] * 11,
                   [FLT_MAX] * 12),
        "quad5": (quad, [-1.0 + i for i in range(5)], [free] + [0.0] * 4, [FLT_MAX] * 5),
        "nanwall6": (nanwall, [0.2 + 0.04 * i for i in range(6)], [free] + [0.0] * 5,
                     [FLT_MAX] * 6),
        "kinks5": (kinks, [0.75 * i for i in range(5)], [free] + [0.0] * 4, [FLT_MAX] * 5),
        "pinned3": (pinned, [0.0, 0.0, 0.0], [0.0] * 3, [FLT_MAX] * 3),
        "wrong_gradient3": (wrong_gradient, [1.0, 2.0, 3.0], [free, 0.0, 0.0], [FLT_MAX] * 3),
    }
