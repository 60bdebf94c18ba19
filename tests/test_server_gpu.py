"""Continuous-batching server: results are the same alone and in the mix,
admission respects the HBM budget, and admitted work overlaps."""
import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, conformal_scale, draw_rootset
from quijibo_gb300.samples import ShapeSDF, poisson_disk

pytestmark = pytest.mark.gpu


def mixed_requests(seed=0, n=24):
    rng = np.random.RandomState(seed)
    reqs = []
    for i in range(n):
        kind = [lib.QJG_REQ_FIELD, lib.QJG_REQ_MESH, lib.QJG_REQ_ENERGY][i % 3]
        nt = int(rng.randint(4, 17))
        nb = int(rng.randint(0, 6))
        rs = draw_rootset(100 + i, nt, nb, -1.2, 1.2, exps=(1, 2))
        res = int(rng.choice([16, 24, 32, 48]))
        g = Grid((res, res, res))
        rs.scale = conformal_scale(rs, g, sample_res=16)
        max_it = int(rng.randint(5, 21))
        if kind == lib.QJG_REQ_ENERGY:
            xyz, _ = poisson_disk(500, seed=i)
            reqs.append(dict(kind=kind, rs=rs, params=lib.params_of(rs), xyz=xyz,
                             target=ShapeSDF(i)(xyz), max_it=max_it, precision=lib.QJG_FP32))
        else:
            reqs.append(dict(kind=kind, rs=rs, grid=g, max_it=max_it,
                             precision=[lib.QJG_FP64, lib.QJG_FP32_REFINE][i % 2]))
    return reqs


def run(server, reqs):
    tickets, outs = [], []
    for r in reqs:
        o = {}
        kw = dict(r)
        if r["kind"] == lib.QJG_REQ_FIELD:
            o["field"] = np.empty(r["grid"].n_voxels)
            kw["out_field"] = o["field"]
        elif r["kind"] == lib.QJG_REQ_MESH:
            cap = 3 * r["grid"].n_voxels
            o["verts"] = np.empty(3 * cap)
            o["tris"] = np.empty(3 * 2 * cap, dtype=np.int32)
            kw.update(vert_cap=cap, tri_cap=2 * cap, out_verts=o["verts"], out_tris=o["tris"])
        else:
            o["grad"] = np.empty(len(r["params"]))
            kw["out_grad"] = o["grad"]
        tickets.append(server.submit(**kw))
        outs.append(o)
    results = [server.wait(t) for t in tickets]
    for o, res in zip(outs, results):
        assert res["status"] == lib.QJG_STATUS_DONE, res
        if "verts" in o:
            o["verts"] = o["verts"][:3 * res["n_verts"]].copy()
            o["tris"] = o["tris"][:3 * res["n_tris"]].copy()
        o["energy"] = res["energy"]
    return outs, results


def test_results_same_alone_and_in_the_mix():
    reqs = mixed_requests()
    mix_srv = lib.Server(workers=6, hbm_budget=2 << 30)
    mixed, mres = run(mix_srv, reqs)
    st = mix_srv.stats()
    mix_srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["peak_running"] >= 2  # work overlapped on the device
    alone_srv = lib.Server(workers=1, hbm_budget=2 << 30)
    for r, m in zip(reqs, mixed):
        a, _ = run(alone_srv, [r])
        a = a[0]
        for k in m:
            if isinstance(m[k], np.ndarray):
                np.testing.assert_array_equal(m[k], a[k], err_msg=k)
            else:
                assert m[k] == a[k], k
    alone_srv.close()


def test_budget_limits_concurrency():
    reqs = [r for r in mixed_requests(seed=1) if r["kind"] == lib.QJG_REQ_FIELD]
    srv = lib.Server(workers=8, hbm_budget=1)  # every request exceeds it: one at a time
    _, res = run(srv, reqs)
    st = srv.stats()
    srv.close()
    assert st["peak_running"] == 1
    spans = sorted((r["t_admit_ms"], r["t_done_ms"]) for r in res)
    for (a0, d0), (a1, d1) in zip(spans, spans[1:]):
        assert a1 >= d0 - 1e-6


def test_server_matches_direct_calls(ctx):
    reqs = [r for r in mixed_requests(seed=2) if r["kind"] == lib.QJG_REQ_FIELD][:3]
    srv = lib.Server(workers=3)
    outs, _ = run(srv, reqs)
    srv.close()
    for r, o in zip(reqs, outs):
        h = ctx.upload(r["rs"])
        it = ctx.iter_params(r["max_it"], 2.0, precision=r["precision"],
                             refine_pow=lib.QJG_REFINE_INT)
        f, _, _ = ctx.field_host(h, r["grid"], it)
        ctx.free(h)
        np.testing.assert_array_equal(f.reshape(-1), o["field"])


def test_batched_field_requests_equal_direct_calls(ctx):
    """Small precision-form field requests submitted together are served in
    multi-request batch passes (a replayed CUDA graph); each field has the
    bits of its own qjg_field call.  FP64 and non-integer-exponent requests
    take the per-request workers."""
    rng = np.random.RandomState(5)
    reqs = []
    for i in range(40):
        nt, nb = int(rng.randint(3, 20)), int(rng.randint(0, 8))
        rs = draw_rootset(300 + i, nt, nb, -1.2, 1.2, exps=(1, 2))
        res = (int(rng.choice([8, 17, 24, 33])), int(rng.choice([9, 16, 31])),
               int(rng.choice([5, 12, 20])))
        g = Grid(res)
        rs.scale = conformal_scale(rs, g, sample_res=16)
        prec = lib.QJG_FP64 if i % 10 == 9 else lib.QJG_FP32_REFINE
        if i % 10 == 4:
            rs.top_powers = rs.top_powers * 1.5  # non-integer effective exponents
        reqs.append(dict(kind=lib.QJG_REQ_FIELD, rs=rs, grid=g, max_it=int(rng.randint(5, 31)),
                         precision=prec, rel_tol=[0.0, 1e-6][i % 2]))
    srv = lib.Server(workers=4)
    outs, res = run(srv, reqs)
    st = srv.stats()
    srv.close()
    n_batchable = sum(1 for i in range(40) if i % 10 not in (4, 9))
    assert st["batched"] == n_batchable and st["failed"] == 0
    assert st["max_batch"] > 1 and st["batches"] < n_batchable
    for r, o, rr in zip(reqs, outs, res):
        h = ctx.upload(r["rs"])
        it = ctx.iter_params(r["max_it"], 2.0, precision=r["precision"],
                             refine_pow=lib.QJG_REFINE_INT, rel_tol=r["rel_tol"])
        f, _, fs = ctx.field_host(h, r["grid"], it)
        ctx.free(h)
        np.testing.assert_array_equal(f.reshape(-1), o["field"])
        assert rr["voxel_iters"] == fs["voxel_iters"]


def test_batched_energy_requests_equal_direct_calls(ctx):
    """FP32 energy + gradient requests submitted together are served in
    multi-request energy batches (one forward and one adjoint pass over all
    of them); each result is its own qjg_energy_backward's within FP32
    rounding.  FP64 energy requests take the per-request workers."""
    torch = pytest.importorskip("torch")
    rng = np.random.RandomState(7)
    reqs = []
    for i in range(14):
        nt, nb = int(rng.randint(4, 17)), int(rng.randint(0, 6))
        rs = draw_rootset(500 + i, nt, nb, -1.2, 1.2, exps=(1, 2))
        rs.scale = conformal_scale(rs, Grid((16, 16, 16), lengths=(2.0, 2.0, 2.0)), 16)
        xyz, _ = poisson_disk(int(rng.randint(300, 3000)), seed=40 + i)
        reqs.append(dict(kind=lib.QJG_REQ_ENERGY, rs=rs, params=lib.params_of(rs), xyz=xyz,
                         target=ShapeSDF(i)(xyz), max_it=int(rng.randint(5, 21)),
                         precision=lib.QJG_FP64 if i % 7 == 6 else lib.QJG_FP32))
    srv = lib.Server(workers=2)
    outs, res = run(srv, reqs)
    st = srv.stats()
    srv.close()
    n32 = sum(1 for r in reqs if r["precision"] == lib.QJG_FP32)
    assert st["energy_batched"] == n32 and st["failed"] == 0
    assert st["max_energy_batch"] > 1 and st["energy_batches"] < n32
    for r, o in zip(reqs, outs):
        P = torch.from_numpy(r["params"]).cuda()
        X = torch.from_numpy(np.ascontiguousarray(r["xyz"])).cuda()
        T = torch.from_numpy(r["target"]).cuda()
        G = torch.empty_like(P)
        e = ctx.energy(P.data_ptr(), r["rs"].n_top, r["rs"].n_bottom, len(r["target"]),
                       X.data_ptr(), T.data_ptr(), r["max_it"], 2.0, precision=r["precision"],
                       d_grad=G.data_ptr())
        g = G.cpu().numpy()
        tol = 1e-5 if r["precision"] == lib.QJG_FP32 else 1e-12
        assert abs(o["energy"] - e) <= tol * abs(e)
        assert np.linalg.norm(o["grad"] - g) <= tol * np.linalg.norm(g)


def test_batched_mesh_requests_equal_direct_calls(ctx):
    """Precision-form mesh requests with integer exponents take their field
    from the field batch pass (with the field requests waiting beside them)
    and are meshed from it: each mesh has the vertices and triangles of its
    own qjg_mesh_stream call, bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.RandomState(7)
    reqs = []
    for i in range(12):
        nt, nb = int(rng.randint(3, 17)), int(rng.randint(0, 7))
        rs = draw_rootset(500 + i, nt, nb, -1.2, 1.2, exps=(1, 2))
        res = int(rng.choice([16, 24, 33, 40]))
        g = Grid((res, res, res))
        rs.scale = conformal_scale(rs, g, sample_res=16)
        kind = lib.QJG_REQ_FIELD if i % 4 == 3 else lib.QJG_REQ_MESH
        reqs.append(dict(kind=kind, rs=rs, grid=g, max_it=int(rng.randint(5, 25)),
                         precision=lib.QJG_FP32_REFINE, rel_tol=[0.0, 1e-6][i % 2]))
    srv = lib.Server(workers=4)
    outs, res = run(srv, reqs)
    st = srv.stats()
    srv.close()
    n_mesh = sum(1 for r in reqs if r["kind"] == lib.QJG_REQ_MESH)
    assert st["mesh_batched"] == n_mesh and st["batched"] == len(reqs) and st["failed"] == 0
    assert st["batches"] < len(reqs)
    tris = 0
    for r, o, rr in zip(reqs, outs, res):
        if r["kind"] != lib.QJG_REQ_MESH:
            continue
        cap = 3 * r["grid"].n_voxels
        v = torch.empty(3 * cap, dtype=torch.float64, device="cuda")
        t = torch.empty(3 * 2 * cap, dtype=torch.int32, device="cuda")
        h = ctx.upload(r["rs"])
        it = ctx.iter_params(r["max_it"], 2.0, precision=r["precision"],
                             refine_pow=lib.QJG_REFINE_INT, rel_tol=r["rel_tol"])
        _, ms = ctx.mesh_stream(h, r["grid"], it, d_verts64=v.data_ptr(), vert_cap=cap,
                                d_tris=t.data_ptr(), tri_cap=2 * cap)
        ctx.free(h)
        assert rr["n_verts"] == ms["n_verts"] and rr["n_tris"] == ms["n_tris"]
        tris += ms["n_tris"]
        np.testing.assert_array_equal(o["verts"], v[:3 * ms["n_verts"]].cpu().numpy())
        np.testing.assert_array_equal(o["tris"], t[:3 * ms["n_tris"]].cpu().numpy())
    assert tris > 0
