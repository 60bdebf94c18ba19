"""Batches of squared-error energy + gradient calls (qjg_energy_backward_batch):
items with different root counts, sample counts (empty, one sample, chunk
boundaries), iteration caps and saturation distances in one pass give each
item's own energy and gradient (FP32, within rounding of the item's
qjg_energy_backward call), the same on every run."""
import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, conformal_scale, draw_rootset
from quijibo_gb300.samples import ShapeSDF, poisson_disk

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHAPES = [  # (n_top, n_bot, samples, max_it, d_sat)
    (8, 4, 3000, 10, 1.0),
    (4, 0, 1, 6, 1.0),
    (16, 8, 2049, 20, 0.0),
    (6, 2, 0, 5, 1.0),
    (12, 3, 5000, 30, 1.0),
    (64, 16, 4096, 12, 1.0),
]


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


@pytest.fixture(scope="module")
def items():
    out = []
    for j, (nt, nb, n, max_it, dsat) in enumerate(SHAPES):
        rs = draw_rootset(10 + j, nt, nb, -1.2, 1.2, exps=(1, 2))
        rs.scale = conformal_scale(rs, Grid((16, 16, 16), lengths=(2.0, 2.0, 2.0)))
        xyz, _ = poisson_disk(max(n, 64), seed=j)
        xyz = xyz[:n]
        t = ShapeSDF(j)(xyz) if n else np.zeros(0)
        p = dev(lib.params_of(rs))
        X, T = dev(xyz.reshape(-1, 3)), dev(t)
        out.append(dict(d_params=p.data_ptr(), n_top=nt, n_bot=nb, n=n, d_xyz=X.data_ptr(),
                        d_target=T.data_ptr(), max_it=max_it, escape=2.0, d_sat=dsat,
                        keep=(p, X, T)))
    return out


def single(ctx, it):
    g = torch.empty(5 * (it["n_top"] + it["n_bot"]) + 1, dtype=torch.float64, device="cuda")
    e = ctx.energy(it["d_params"], it["n_top"], it["n_bot"], it["n"], it["d_xyz"], it["d_target"],
                   it["max_it"], it["escape"], d_sat=it["d_sat"], precision=lib.QJG_FP32,
                   d_grad=g.data_ptr())
    return e, g.cpu().numpy()


def batch(ctx, items):
    grads = [torch.full((5 * (it["n_top"] + it["n_bot"]) + 1,), 7.0, dtype=torch.float64,
                        device="cuda") for it in items]
    for it, g in zip(items, grads):
        it["d_grad"] = g.data_ptr()
    es = ctx.energy_batch(items)
    return es, [g.cpu().numpy() for g in grads]


def test_batch_gives_each_item_its_own_energy_and_gradient(ctx, items):
    es, gs = batch(ctx, items)
    for it, e, g in zip(items, es, gs):
        e1, g1 = single(ctx, it)
        if it["n"] == 0:
            assert e == 0.0 and not g.any()
            continue
        assert abs(e - e1) <= 1e-6 * abs(e1), (e, e1)
        assert np.all(np.isfinite(g))
        assert np.linalg.norm(g - g1) <= 1e-5 * max(np.linalg.norm(g1), 1e-30), \
            np.linalg.norm(g - g1) / np.linalg.norm(g1)


def test_batch_is_deterministic_and_order_free(ctx, items):
    e1, g1 = batch(ctx, items)
    e2, g2 = batch(ctx, items)
    assert e1 == e2 and all(np.array_equal(a, b) for a, b in zip(g1, g2))
    # the same items in another order: each item's values do not depend on
    # the others
    rev = items[::-1]
    e3, g3 = batch(ctx, rev)
    for a, b, c, d in zip(e1, g1, e3[::-1], g3[::-1]):
        assert a == c and np.array_equal(b, d)


def test_empty_batch(ctx):
    assert ctx.energy_batch([]) == []
