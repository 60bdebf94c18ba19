"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

`Oracle` wraps oracle/_build/libqj_oracle.so, the plain-C restatement of the
reference's hot path (qj_oracle.c).  `Reference` wraps the reference QUIJIBO
itself, compiled from its own sources into oracle/_ref/ (only where those
sources are present); it pins the restatement and generates golden fixtures.
Only tests, the smoke check and the benchmark's CPU-baseline leg use this.
"""
import contextlib
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libqj_oracle.so")
REF_SO = {"double": os.path.join(HERE, "_ref", "libqjref_double.so"),
          "ldouble": os.path.join(HERE, "_ref", "libqjref_ldouble.so")}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


def build(ref=False):
    """Compile the restatement (and, with ref=True, the reference flavours)."""
    subprocess.run(["make", "-s", "-C", HERE] + (["ref"] if ref else []), check=True)


class _Poly(C.Structure):
    _fields_ = [("n", C.c_int), ("roots", _dp), ("powers", _dp), ("power_scalar", C.c_double)]


class _Map(C.Structure):
    _fields_ = [("top", _Poly), ("bottom", _Poly), ("scale", C.c_double), ("lagrange", C.c_int)]


class _Grid(C.Structure):
    _fields_ = [("res", C.c_int * 3), ("center", C.c_double * 3), ("lengths", C.c_double * 3),
                ("rot", C.c_double * 4), ("slice", C.c_double)]


def make_map(rootset):
    """rootset: object with top_roots (n,4), top_powers, sigma_top, bottom_*, scale."""
    keep = []

    def poly(r, p, s):
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 4)
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1)
        keep.extend([r, p])
        return _Poly(len(p), _ptr(r), _ptr(p), float(s))

    m = _Map(poly(rootset.top_roots, rootset.top_powers, rootset.sigma_top),
             poly(rootset.bottom_roots, rootset.bottom_powers, rootset.sigma_bottom),
             float(rootset.scale), int(bool(getattr(rootset, "lagrange", False))))
    m._keep = keep
    return m


def make_grid(grid):
    g = _Grid()
    g.res[:] = list(grid.res)
    g.center[:] = list(grid.center)
    g.lengths[:] = list(grid.lengths)
    g.rot[:] = list(grid.rot)
    g.slice = float(grid.slice)
    return g


class Oracle:
    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.qjo_mt_rand.argtypes = [C.c_uint32, C.c_int, _dp]
        L.qjo_quat_pow.argtypes = [_dp, C.c_double, _dp]
        L.qjo_set_libm.argtypes = [C.c_int]
        L.qjo_set_libm.restype = None
        L.qjo_crm.argtypes = [C.c_int, C.c_double]
        L.qjo_crm.restype = C.c_double
        L.qjo_field.argtypes = [C.POINTER(_Map), C.POINTER(_Grid), C.c_int, C.c_double, C.c_int,
                                C.c_int, _dp, _dp, C.POINTER(C.c_int32), C.c_int]
        L.qjo_field.restype = C.c_int64
        L.qjo_field_window.argtypes = [C.POINTER(_Map), C.POINTER(_Grid), C.c_int, C.c_double,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp,
                                       C.c_int]
        L.qjo_field_window.restype = None
        L.qjo_nonlinear_value.argtypes = [C.POINTER(_Map), _dp, C.c_double, C.c_int, C.c_double,
                                          C.c_double]
        L.qjo_nonlinear_value.restype = C.c_double
        L.qjo_mesh.argtypes = [C.POINTER(_Map), C.POINTER(_Grid), _dp, C.c_int, C.c_int,
                               C.c_double, C.c_double, _dp, C.c_int64, C.POINTER(C.c_int32),
                               C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                               C.POINTER(C.c_int64), C.c_int]
        L.qjo_trilinear.argtypes = [C.POINTER(_Grid), _dp, _dp]
        L.qjo_trilinear.restype = C.c_double
        L.qjo_cell_center.argtypes = [C.POINTER(_Grid), C.c_int, C.c_int, C.c_int, _dp]
        L.qjo_tanh_score_grad.argtypes = [C.POINTER(_Map), C.POINTER(_Grid), C.POINTER(_Grid), _dp,
                                          C.c_int, C.c_double, C.c_double, _dp, _dp]
        L.qjo_tanh_score_grad.restype = C.c_double
        L.qjo_centered_gradient.argtypes = [C.POINTER(_Map), C.POINTER(_Grid), C.c_int, C.c_int,
                                            _dp, _dp, _dp, _dp]
        L.qjo_centered_gradient.restype = None
        L.qjo_sqerr_energy.argtypes = [C.POINTER(_Map), C.c_int64, _dp, _dp, C.c_double, C.c_int,
                                       C.c_double, C.c_double, C.POINTER(C.c_int32)]
        L.qjo_sqerr_energy.restype = C.c_double
        self.L = L

    def mt_rand(self, seed, n):
        out = np.empty(n)
        self.L.qjo_mt_rand(seed, n, _ptr(out))
        return out

    def set_libm(self, correctly_rounded):
        """Transcendentals of the map's QUATERNION::pow: False the C library's
        (the reference build's), True the correctly rounded ones."""
        self.L.qjo_set_libm(int(bool(correctly_rounded)))

    CRM = ("exp", "log", "sin", "cos", "acos")

    def crm(self, name, x):
        """The correctly rounded function `name` on each element of x."""
        fn = self.CRM.index(name)
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        return np.array([self.L.qjo_crm(fn, float(v)) for v in x])

    def quat_pow(self, q, e):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.empty(4)
        self.L.qjo_quat_pow(_ptr(q), e, _ptr(out))
        return out

    def cell_center(self, grid, x, y, z):
        out = np.empty(3)
        self.L.qjo_cell_center(C.byref(make_grid(grid)), x, y, z, _ptr(out))
        return out

    def field(self, rootset, grid, max_it, escape, z0=0, z1=None, de=False, iters=False,
              nthreads=0):
        X, Y, Z = grid.res
        z1 = Z if z1 is None else z1
        n = X * Y * (z1 - z0)
        f = np.empty(n)
        d = np.empty(n) if de else None
        it = np.empty(n, dtype=np.int32) if iters else None
        m, g = make_map(rootset), make_grid(grid)
        terms = self.L.qjo_field(C.byref(m), C.byref(g), max_it, escape, z0, z1, _ptr(f),
                                 _ptr(d), _ptr(it, C.POINTER(C.c_int32)), nthreads)
        shape = (z1 - z0, Y, X)
        out = {"field": f.reshape(shape), "root_terms": int(terms)}
        if de:
            out["de"] = d.reshape(shape)
        if iters:
            out["iters"] = it.reshape(shape)
        return out

    def field_window(self, rootset, grid, max_it, escape, x0, x1, y0, y1, z0, z1, nthreads=0):
        """log|q_N| on the cells [x0,x1) x [y0,y1) x [z0,z1) of `grid` (cell
        centres of the full grid), shaped (z, y, x)."""
        f = np.empty((z1 - z0) * (y1 - y0) * (x1 - x0))
        self.L.qjo_field_window(C.byref(make_map(rootset)), C.byref(make_grid(grid)), max_it,
                                escape, x0, x1, y0, y1, z0, z1, _ptr(f), nthreads)
        return f.reshape(z1 - z0, y1 - y0, x1 - x0)

    def nonlinear_value(self, rootset, p, slice_, max_it, escape, iso=0.0):
        p = np.ascontiguousarray(p, dtype=np.float64)
        return self.L.qjo_nonlinear_value(C.byref(make_map(rootset)), _ptr(p), slice_, max_it,
                                          escape, iso)

    def mesh(self, rootset, grid, classify, mode, max_it, escape, iso=0.0, nthreads=0):
        classify = np.ascontiguousarray(classify, dtype=np.float64).reshape(-1)
        N = classify.size
        cap_v, cap_t = 3 * N + 16, 5 * N + 16
        verts = np.empty(3 * cap_v)
        tris = np.empty(3 * cap_t, dtype=np.int32)
        nv, nt, nu = C.c_int64(), C.c_int64(), C.c_int64()
        m = make_map(rootset) if rootset is not None else _Map()
        rc = self.L.qjo_mesh(C.byref(m), C.byref(make_grid(grid)), _ptr(classify), mode, max_it,
                             escape, iso, _ptr(verts), cap_v, _ptr(tris, C.POINTER(C.c_int32)),
                             cap_t, C.byref(nv), C.byref(nt), C.byref(nu), nthreads)
        assert rc == 0, rc
        return {"verts": verts[:3 * nv.value].reshape(-1, 3).copy(),
                "tris": tris[:3 * nt.value].reshape(-1, 3).copy(), "unbracketed": nu.value}

    def tanh_score_grad(self, rootset, grid, wgrid, weights, max_it, alpha=10.0, threshold=0.0):
        """Score, gradient [log s, bottom exps, top exps, sigma_t, sigma_b], field."""
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
        grad = np.empty(3 + rootset.n_top + rootset.n_bottom)
        field = np.empty(grid.n_voxels)
        sc = self.L.qjo_tanh_score_grad(C.byref(make_map(rootset)), C.byref(make_grid(grid)),
                                        C.byref(make_grid(wgrid)), _ptr(w), max_it, alpha,
                                        threshold, _ptr(grad), _ptr(field))
        return sc, grad, field.reshape(grid.res[::-1])

    def centered_gradient(self, rootset, grid, max_it, kind, dist, curv=None):
        """(score, gradient) of the centered root gradients (kind 0 log-rational,
        1 its bottom-root form, 2 computeCenteredGradient)."""
        d = np.ascontiguousarray(dist, dtype=np.float64).reshape(-1)
        cv = None if curv is None else np.ascontiguousarray(curv, dtype=np.float64).reshape(-1)
        nt, nb = rootset.n_top, rootset.n_bottom
        grad = np.empty(4 * (nt + nb if kind == 0 else nb if kind == 1 else nt))
        sc = np.empty(1)
        self.L.qjo_centered_gradient(C.byref(make_map(rootset)), C.byref(make_grid(grid)), max_it,
                                     kind, _ptr(d), _ptr(cv), _ptr(grad), _ptr(sc))
        return float(sc[0]), grad

    def sqerr_energy(self, rootset, xyz, target, max_it, escape, slice_=0.0, iters=False,
                     d_sat=1.0):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(target, dtype=np.float64)
        it = np.empty(len(t), dtype=np.int32) if iters else None
        e = self.L.qjo_sqerr_energy(C.byref(make_map(rootset)), len(t), _ptr(xyz), _ptr(t), slice_,
                                    max_it, escape, d_sat, _ptr(it, C.POINTER(C.c_int32)))
        return (e, it) if iters else e

    def trilinear(self, grid, data, p):
        data = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
        p = np.ascontiguousarray(p, dtype=np.float64)
        return self.L.qjo_trilinear(C.byref(make_grid(grid)), _ptr(data), _ptr(p))


_REF_OBJECTIVE = C.CFUNCTYPE(None, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                             C.POINTER(C.c_double))


@contextlib.contextmanager
def _quiet():
    """Silence the reference's progress printing on stdout."""
    sys.stdout.flush()
    saved = os.dup(1)
    null = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(null, 1)
        yield
    finally:
        C.CDLL(None).fflush(None)
        os.dup2(saved, 1)
        os.close(null)
        os.close(saved)


class _MapArgs(C.Structure):
    _fields_ = [("nt", C.c_int), ("troots", _dp), ("tpows", _dp), ("tsig", C.c_double),
                ("nb", C.c_int), ("broots", _dp), ("bpows", _dp), ("bsig", C.c_double),
                ("s", C.c_double)]


def _map_args(rs):
    tr = np.ascontiguousarray(rs.top_roots, dtype=np.float64).reshape(-1, 4)
    tp = np.ascontiguousarray(rs.top_powers, dtype=np.float64)
    br = np.ascontiguousarray(rs.bottom_roots, dtype=np.float64).reshape(-1, 4)
    bp = np.ascontiguousarray(rs.bottom_powers, dtype=np.float64)
    a = _MapArgs(len(tp), _ptr(tr), _ptr(tp), rs.sigma_top, len(bp), _ptr(br), _ptr(bp),
                 rs.sigma_bottom, rs.scale)
    a._keep = (tr, tp, br, bp)
    return a


class Reference:
    """The reference implementation compiled from its own sources."""

    def __init__(self, flavour="double"):
        path = REF_SO[flavour]
        if not os.path.exists(path):
            build(ref=True)
        L = C.CDLL(path)
        L.ref_sizeof_real.restype = C.c_int
        L.ref_mt_rand.argtypes = [C.c_uint, C.c_int, _dp]
        L.ref_quat_pow.argtypes = [_dp, C.c_double, _dp]
        A = C.POINTER(_MapArgs)
        L.ref_field_escape.argtypes = [A, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_double, _dp]
        L.ref_field_map.argtypes = [A, _ip, _dp, _dp, C.c_double, C.c_int, _dp]
        L.ref_mesh_stream.argtypes = [A, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_double, _dp,
                                      C.c_int, _ip, C.c_int, _ip, _ip]
        L.ref_mesh_field_nonlinear.argtypes = [A, _ip, _dp, _dp, _dp, C.c_double, C.c_int,
                                               C.c_double, _dp, C.c_int, _ip, C.c_int, _ip, _ip]
        L.ref_mesh_linear.argtypes = [_ip, _dp, _dp, _dp, _dp, C.c_int, _ip, C.c_int, _ip, _ip]
        L.ref_tanh_score_grad.argtypes = [A, _ip, _dp, _dp, C.c_double, C.c_int, _ip, _dp, _dp,
                                          _dp, _dp, _dp]
        L.ref_tanh_score_grad.restype = C.c_double
        L.ref_field_lagrange.argtypes = [A, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_double,
                                         _dp]
        L.ref_mesh_lagrange.argtypes = [A, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_double,
                                        _dp, C.c_int, _ip, C.c_int, _ip, _ip]
        L.ref_o3d_write.argtypes = [C.c_char_p, A, _ip, _dp, _dp, _dp, _ip, _dp, _dp, _dp, _dp]
        L.ref_o3d_read.argtypes = [C.c_char_p, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_inverted_distance.argtypes = [_ip, _dp, _dp, _dp, C.c_int, _dp]
        L.ref_centered_gradient.argtypes = [A, _ip, _dp, _dp, C.c_double, C.c_int, C.c_int, _dp,
                                            _dp, _dp, _dp]
        L.ref_conformal_radius.argtypes = [A, _ip, _dp, _dp, C.c_double, _ip, _dp, _dp, _dp, _dp]
        L.ref_conformal_radius.restype = C.c_double
        L.ref_blmvm.argtypes = [C.c_int, _dp, _dp, _dp, _REF_OBJECTIVE]
        L.ref_tanh_fit.argtypes = [C.c_int, A, _ip, _dp, _dp, C.c_double, C.c_int, _ip, _dp, _dp,
                                   _dp, _dp, _dp, C.c_int]
        L.ref_tanh_fit.restype = C.c_int
        L.ref_tooth_run.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_int, _ip, _dp, _ip,
                                    _dp]
        L.ref_field_write.argtypes = [C.c_char_p, _ip, _dp, _dp, _dp]
        L.ref_mesh_write.argtypes = [_dp, C.c_int, _ip, C.c_int, C.c_char_p, C.c_char_p]
        L.ref_mesh_write.restype = C.c_int
        self.L = L
        self.sizeof_real = L.ref_sizeof_real()

    @staticmethod
    def _g(grid):
        res = np.array(grid.res, dtype=np.int32)
        return (res, np.array(grid.center, dtype=np.float64),
                np.array(grid.lengths, dtype=np.float64), np.array(grid.rot, dtype=np.float64))

    def field_lagrange(self, rs, grid, max_it, escape):
        """The Lagrange-order escape loop (computeLagrangeNonlinearSlice)."""
        res, c, ln, r = self._g(grid)
        out = np.empty(int(np.prod(grid.res)))
        self.L.ref_field_lagrange(C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c), _ptr(ln),
                                  _ptr(r), float(grid.slice), int(max_it), float(escape), _ptr(out))
        return out

    def mesh_lagrange(self, rs, grid, max_it, iso=0.0):
        res, c, ln, r = self._g(grid)
        return self._mesh_out(self.L.ref_mesh_lagrange, C.byref(_map_args(rs)), _ptr(res, _ip),
                              _ptr(c), _ptr(ln), _ptr(r), float(grid.slice), int(max_it),
                              float(iso), n=int(np.prod(grid.res)))

    def o3d_write(self, path, rs, grid, fractal, dgrid, dist, curv):
        """OPTIMIZE_3D::write of a state (the fractal on grid, the distance and
        curvature fields on dgrid)."""
        res, c, ln, _ = self._g(grid)
        dres, dc, dln, _ = self._g(dgrid)
        f = lambda a: _ptr(np.ascontiguousarray(a, dtype=np.float64).ravel())  # noqa: E731
        self.L.ref_o3d_write(str(path).encode(), C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c),
                             _ptr(ln), f(fractal), _ptr(dres, _ip), _ptr(dc), _ptr(dln), f(dist),
                             f(curv))

    def o3d_read(self, path, max_roots=256, max_cells=1 << 20):
        """OPTIMIZE_3D::read: what the reference takes from a state file."""
        counts = np.zeros(2, dtype=np.int32)
        tr, br = np.empty(4 * max_roots), np.empty(4 * max_roots)
        tp, bp = np.empty(max_roots), np.empty(max_roots)
        sc = np.empty(3)
        fr, di = np.empty(max_cells), np.empty(max_cells)
        self.L.ref_o3d_read(str(path).encode(), _ptr(counts, _ip), _ptr(tr), _ptr(tp), _ptr(br),
                            _ptr(bp), _ptr(sc), _ptr(fr), _ptr(di))
        nt, nb = int(counts[0]), int(counts[1])
        return {"top_roots": tr[:4 * nt].reshape(-1, 4), "top_powers": tp[:nt],
                "bottom_roots": br[:4 * nb].reshape(-1, 4), "bottom_powers": bp[:nb],
                "sigma_top": sc[0], "sigma_bottom": sc[1], "scale": sc[2], "fractal": fr,
                "dist": di}

    def inverted_distance(self, grid, dist, normalized=False):
        """FIELD_3D::invertedDistance[Normalized] of `dist` (x fastest)."""
        res, c, ln, _ = self._g(grid)
        out = np.empty(int(np.prod(grid.res)))
        self.L.ref_inverted_distance(_ptr(res, _ip), _ptr(c), _ptr(ln),
                                     _ptr(np.ascontiguousarray(dist, dtype=np.float64).ravel()),
                                     int(bool(normalized)), _ptr(out))
        return out

    def conformal_radius(self, rs, grid, dgrid, dist):
        """OPTIMIZE_3D::estimateConformalRadius: (lowest score, exp scaling)."""
        res, c, ln, _ = self._g(grid)
        dres, dc, dln, _ = self._g(dgrid)
        es = C.c_double()
        sc = self.L.ref_conformal_radius(C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c), _ptr(ln),
                                         float(grid.slice), _ptr(dres, _ip), _ptr(dc), _ptr(dln),
                                         _ptr(np.ascontiguousarray(dist, dtype=np.float64).ravel()),
                                         C.byref(es))
        return sc, es.value

    def blmvm(self, fun, x0, lower, upper):
        """TAO_SOLVER::optimizeBLMVM of fun(x) -> (f, grad); returns the
        solution and every evaluation as (f, x)."""
        hist = []

        def cb(n, xp, fp, gp):
            x = np.ctypeslib.as_array(xp, (n,)).copy()
            f, g = fun(x)
            hist.append((f, x))
            fp[0] = f
            np.ctypeslib.as_array(gp, (n,))[:] = g
        fn = _REF_OBJECTIVE(cb)
        x = np.array(x0, dtype=np.float64)
        lo = np.ascontiguousarray(lower, dtype=np.float64)
        hi = np.ascontiguousarray(upper, dtype=np.float64)
        with _quiet():
            self.L.ref_blmvm(len(x), _ptr(x), _ptr(lo), _ptr(hi), fn)
        return x, hist

    def tanh_fit(self, mode, rs, grid, wgrid, weights, max_it=1, hist_cap=1 << 22):
        """toothOptimizer's scaled-only (0) or scaled (1) BLMVM solve: final
        [bottom powers, top powers, sigma_t, sigma_b, expScaling] and the
        evaluations as rows {f, state...}."""
        res, c, l, _ = self._g(grid)
        wres, wc, wl, _ = self._g(wgrid)
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
        out = np.empty(rs.n_top + rs.n_bottom + 3)
        hist = np.empty(hist_cap)
        with _quiet():
            ne = self.L.ref_tanh_fit(int(mode), C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c),
                                     _ptr(l), grid.slice, int(max_it), _ptr(wres, _ip), _ptr(wc),
                                     _ptr(wl), _ptr(w), _ptr(out), _ptr(hist), hist_cap)
        n = 3 if mode == 0 else 3 + rs.n_top + rs.n_bottom
        return out, hist[:ne * (n + 1)].reshape(ne, n + 1)

    def tooth_run(self, path, n_top, n_bot, levels, radius=4.0, amp=-1.0):
        """toothOptimizer's main without the reweighted solve: per level
        [bottom powers, top powers, sigma_t, sigma_b, scale, final score],
        evaluations of its three solves, and the final roots (top then
        bottom)."""
        lv = np.asarray(levels, dtype=np.int32)
        out = np.empty((len(lv), n_top + n_bot + 4))
        ev = np.empty((len(lv), 3), dtype=np.int32)
        roots = np.empty((n_top + n_bot, 4))
        with _quiet():
            self.L.ref_tooth_run(str(path).encode(), float(radius), float(amp), len(lv),
                                 _ptr(lv, _ip), _ptr(out), _ptr(ev, _ip), _ptr(roots))
        return out, ev, roots

    def field_write(self, path, res, center, lengths, data):
        """FIELD_3D::write(string) of `data` (x fastest)."""
        self.L.ref_field_write(str(path).encode(), _ptr(np.asarray(res, dtype=np.int32), _ip),
                               _ptr(np.asarray(center, dtype=np.float64)),
                               _ptr(np.asarray(lengths, dtype=np.float64)),
                               _ptr(np.ascontiguousarray(data, dtype=np.float64).ravel()))

    def mesh_write(self, verts, tris, obj_path, raw_path):
        """TRIANGLE_MESH::read of the raw stream, then writeOBJ and write(FILE*)."""
        v = np.ascontiguousarray(verts, dtype=np.float64).ravel()
        t = np.ascontiguousarray(tris, dtype=np.int32).ravel()
        rc = self.L.ref_mesh_write(_ptr(v), len(v) // 3, _ptr(t, _ip), len(t) // 3,
                                   str(obj_path).encode(), str(raw_path).encode())
        assert rc == 0, rc

    def mt_rand(self, seed, n):
        out = np.empty(n)
        self.L.ref_mt_rand(seed, n, _ptr(out))
        return out

    def set_libm(self, correctly_rounded):
        """Transcendentals of the map's QUATERNION::pow: False the C library's
        (the reference build's), True the correctly rounded ones."""
        self.L.qjo_set_libm(int(bool(correctly_rounded)))

    CRM = ("exp", "log", "sin", "cos", "acos")

    def crm(self, name, x):
        """The correctly rounded function `name` on each element of x."""
        fn = self.CRM.index(name)
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        return np.array([self.L.qjo_crm(fn, float(v)) for v in x])

    def quat_pow(self, q, e):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.empty(4)
        self.L.ref_quat_pow(_ptr(q), e, _ptr(out))
        return out

    def field_escape(self, rs, grid, max_it, escape):
        res, c, l, r = self._g(grid)
        out = np.empty(int(np.prod(res)))
        self.L.ref_field_escape(C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c), _ptr(l), _ptr(r),
                                grid.slice, max_it, escape, _ptr(out))
        return out.reshape(res[2], res[1], res[0])

    def field_map(self, rs, grid, max_it):
        res, c, l, _ = self._g(grid)
        out = np.empty(int(np.prod(res)))
        self.L.ref_field_map(C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c), _ptr(l), grid.slice,
                             max_it, _ptr(out))
        return out.reshape(res[2], res[1], res[0])

    def _mesh_out(self, fn, *args, n):
        cap_v, cap_t = 3 * n + 16, 5 * n + 16
        verts = np.empty(3 * cap_v)
        tris = np.empty(3 * cap_t, dtype=np.int32)
        nv, nt = C.c_int(), C.c_int()
        rc = fn(*args, _ptr(verts), cap_v, _ptr(tris, _ip), cap_t, C.byref(nv), C.byref(nt))
        assert rc == 0, rc
        return {"verts": verts[:3 * nv.value].reshape(-1, 3).copy(),
                "tris": tris[:3 * nt.value].reshape(-1, 3).copy()}

    def mesh_stream(self, rs, grid, max_it, iso=0.0):
        res, c, l, r = self._g(grid)
        return self._mesh_out(self.L.ref_mesh_stream, C.byref(_map_args(rs)), _ptr(res, _ip),
                              _ptr(c), _ptr(l), _ptr(r), grid.slice, max_it, iso,
                              n=int(np.prod(res)))

    def mesh_field_nonlinear(self, rs, grid, field, max_it, iso=0.0):
        res, c, l, _ = self._g(grid)
        f = np.ascontiguousarray(field, dtype=np.float64).reshape(-1)
        return self._mesh_out(self.L.ref_mesh_field_nonlinear, C.byref(_map_args(rs)),
                              _ptr(res, _ip), _ptr(c), _ptr(l), _ptr(f), grid.slice, max_it, iso,
                              n=f.size)

    def mesh_linear(self, grid, field):
        res, c, l, _ = self._g(grid)
        f = np.ascontiguousarray(field, dtype=np.float64).reshape(-1)
        return self._mesh_out(self.L.ref_mesh_linear, _ptr(res, _ip), _ptr(c), _ptr(l), _ptr(f),
                              n=f.size)

    def centered_gradient(self, rs, grid, max_it, kind, dist, curv=None):
        """(score, gradient) of OPTIMIZE_3D's centered root gradients (kind 0
        log-rational, 1 its bottom-root form, 2 computeCenteredGradient)."""
        res, c, l, _ = self._g(grid)
        d = np.ascontiguousarray(dist, dtype=np.float64).reshape(-1)
        cv = None if curv is None else np.ascontiguousarray(curv, dtype=np.float64).reshape(-1)
        n = 4 * (rs.n_top + rs.n_bottom if kind == 0 else rs.n_bottom if kind == 1 else rs.n_top)
        grad = np.empty(n)
        sc = np.empty(1)
        with _quiet():
            self.L.ref_centered_gradient(C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c), _ptr(l),
                                         grid.slice, max_it, kind, _ptr(d), _ptr(cv), _ptr(grad),
                                         _ptr(sc))
        return float(sc[0]), grad

    def tanh_score_grad(self, rs, grid, wgrid, weights, max_it):
        res, c, l, _ = self._g(grid)
        wres, wc, wl, _ = self._g(wgrid)
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
        grad = np.empty(3 + rs.n_top + rs.n_bottom)
        field = np.empty(grid.n_voxels)
        sc = self.L.ref_tanh_score_grad(C.byref(_map_args(rs)), _ptr(res, _ip), _ptr(c), _ptr(l),
                                        grid.slice, max_it, _ptr(wres, _ip), _ptr(wc), _ptr(wl),
                                        _ptr(w), _ptr(grad), _ptr(field))
        return sc, grad, field.reshape(grid.res[::-1])


# ---------------------------------------------------------------------------
# The optimizer's set-up passes, restated with numpy (test infrastructure).

def inverted_distance(dist, normalized=False):
    """FIELD_3D::invertedDistance[Normalized] (FIELD_3D.cpp:5241-5352) of a
    (Z, Y, X) signed distance field: the 26-neighbour sign-change shells get
    1, every other cell the 6-neighbour breadth-first layer of the
    reference's sweep loop, then 1/v, negated inside, quartered outside."""
    d = np.asarray(dist, dtype=np.float64)
    Z, Y, X = d.shape
    n = d.size
    pad = np.pad(d, 1)
    flip = np.zeros(d.shape, dtype=bool)
    for k in (-1, 0, 1):
        for j in (-1, 0, 1):
            for i in (-1, 0, 1):
                if i == j == k == 0:
                    continue
                nb = pad[1 + k:1 + k + Z, 1 + j:1 + j + Y, 1 + i:1 + i + X]
                flip |= nb * d < 0
    final = flip.astype(np.float64)
    while True:
        zero = final <= 1e-5
        if not zero.any():
            break
        p = np.pad(final, 1)
        nbs = np.stack([p[1:-1, 1:-1, :-2], p[1:-1, 1:-1, 2:], p[1:-1, :-2, 1:-1],
                        p[1:-1, 2:, 1:-1], p[:-2, 1:-1, 1:-1], p[2:, 1:-1, 1:-1]])
        smallest = np.where(nbs > 1e-5, nbs, n + 1.0).min(axis=0)
        upd = zero & (smallest < n)
        if not upd.any():
            raise ValueError("no sign change reaches every cell")
        final = np.where(upd, smallest + 1.0, final)
    final = 1.0 / final
    final = np.where(d < 0, -final, final * 0.25)
    if normalized:
        final = final * (1.0 / np.abs(final).sum())
        inside = final[d < 0].sum()
        outside = final[d >= 0].sum()
        final = final * np.where(d < 0, 0.5 / abs(inside), 0.5 / abs(outside))
    return final


def cell_centers_ref(grid):
    """FIELD_3D::cellCenter of every cell of an unrotated grid, in the
    reference's operation order (FIELD_3D.cpp:818-841), x fastest."""
    axes = []
    for c in range(3):
        dx = grid.lengths[c] / grid.res[c]
        i = np.arange(grid.res[c], dtype=np.float64)
        f = grid.center[c] - grid.lengths[c] * 0.5
        f = f + i * dx
        f = f + dx * 0.5
        f = f - grid.center[c]
        axes.append(f + grid.center[c])
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return np.stack([x, y, z], axis=-1).reshape(-1, 3)


def conformal_radius(oracle, rs, grid, dgrid, dist, alpha=10.0):
    """OPTIMIZE_3D::estimateConformalRadius (OPTIMIZE_3D.cpp:4693-4772):
    returns (lowest score, threshold, exp(-threshold))."""
    import copy
    r1 = copy.deepcopy(rs)
    r1.sigma_top = r1.sigma_bottom = 1.0
    r1.scale = 1.0
    f = oracle.field(r1, grid, 1, 20.0)["field"].ravel().copy()
    inf = np.isinf(f)
    if inf.any():
        f[inf] = f[~inf].sum() / (~inf).sum()
    w_field = inverted_distance(np.asarray(dist).reshape(dgrid.res[::-1]))
    pts = cell_centers_ref(grid)
    w = np.array([oracle.trilinear(dgrid, w_field, p) for p in pts])
    lo, hi = f.min(), f.max()
    min_t, found = lo, np.finfo(np.float32).max
    for _ in range(4):
        inc = (hi - lo) / 100
        xs = []
        x = lo
        while x < hi:
            xs.append(x)
            x += inc
        found = np.finfo(np.float32).max
        for x in xs:
            s = np.sum(-np.tanh(alpha * (f - x)) * w)
            if s < found:
                found, min_t = s, x
        lo, hi = min_t - 5 * inc, min_t + 5 * inc
    return found, min_t, np.exp(-min_t)


def reweight_inside(md, fd, w):
    """buildReweightedInsideField's arithmetic (projects/toothOptimizer/
    toothOptimizer.cpp:302-381): (reweighted field, poor sum, well sum)."""
    md, fd, w = (np.asarray(a, dtype=np.float64).ravel() for a in (md, fd, w))
    inside = md < 0
    poor = inside & (fd > 0)
    well = inside & (fd < 0)
    poor_sum, well_sum = float(np.sum(w[poor])), float(np.sum(w[well]))
    total_worth, outside_worth, poor_fraction = 0.5, 0.5, 0.5
    outside = ((outside_worth * total_worth) / (1.0 - outside_worth)) / np.count_nonzero(md > 0)
    out = w.copy()
    out[poor] *= total_worth * poor_fraction / abs(poor_sum)
    out[well] *= total_worth * (1.0 - poor_fraction) / abs(well_sum)
    out[~inside] = outside
    return out, poor_sum, well_sum
