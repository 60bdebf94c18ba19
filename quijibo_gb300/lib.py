"""ctypes bindings of the C ABI in include/quijibo_gpu.h.

Loads the in-tree quijibo_gb300/_lib/libquijibo_gpu.so and raises when it is
missing: there is no CPU path behind these calls.
"""
import ctypes as C
import os

import numpy as np

from .rootsets import Grid, RootSet

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libquijibo_gpu.so")

QJG_OK, QJG_ERR_ARG, QJG_ERR_CUDA, QJG_ERR_NOMEM, QJG_ERR_HANDLE, QJG_ERR_CAPACITY = 0, -1, -2, -3, -4, -5
QJG_FP64, QJG_FP32, QJG_FP32_REFINE = 0, 1, 2
QJG_REFINE_POW, QJG_REFINE_INT = 0, 1
QJG_LIBM_DEVICE, QJG_LIBM_CR = 0, 1
CRM_FUNCTIONS = ("exp", "log", "sin", "cos", "acos")  # qjg_crmath_eval's fn order

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


class QjgGrid(C.Structure):
    _fields_ = [("res", C.c_int32 * 3), ("center", C.c_double * 3), ("lengths", C.c_double * 3),
                ("rot", C.c_double * 4), ("slice", C.c_double)]

    @classmethod
    def of(cls, g: Grid):
        s = cls()
        s.res[:] = [int(v) for v in g.res]
        s.center[:] = [float(v) for v in g.center]
        s.lengths[:] = [float(v) for v in g.lengths]
        s.rot[:] = [float(v) for v in g.rot]
        s.slice = float(g.slice)
        return s


class QjgIter(C.Structure):
    _fields_ = [("max_it", C.c_int32), ("precision", C.c_int32), ("refine_pow", C.c_int32),
                ("want_de", C.c_int32), ("escape", C.c_double), ("band_h", C.c_double),
                ("field_tol", C.c_double), ("rel_tol", C.c_double), ("form", C.c_int32),
                ("libm", C.c_int32)]


class QjgFieldStats(C.Structure):
    _fields_ = [("voxels", C.c_int64), ("voxel_iters", C.c_int64), ("root_terms", C.c_int64),
                ("refined", C.c_int64), ("refined_iters", C.c_int64), ("nonfinite", C.c_int64),
                ("lane_iters", C.c_int64), ("rerun", C.c_int64), ("rerun_iters", C.c_int64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class QjgO3dInfo(C.Structure):
    _fields_ = [("res", C.c_int32 * 3), ("center", C.c_double * 3), ("lengths", C.c_double * 3),
                ("n_top", C.c_int32), ("n_bot", C.c_int32), ("sigma_top", C.c_double),
                ("sigma_bot", C.c_double), ("exp_scaling", C.c_double), ("history", C.c_int32),
                ("field_res", (C.c_int32 * 3) * 3), ("field_center", (C.c_double * 3) * 3),
                ("field_lengths", (C.c_double * 3) * 3)]


QJG_EDGE_LINEAR, QJG_EDGE_BISECT = 0, 1


class QjgMeshStats(C.Structure):
    _fields_ = [("n_verts", C.c_int64), ("n_tris", C.c_int64), ("n_degenerate", C.c_int64),
                ("n_unbracketed", C.c_int64), ("map_evals", C.c_int64),
                ("map_evals_fp32", C.c_int64), ("map_evals_ff", C.c_int64), ("slabs", C.c_int64),
                ("field", QjgFieldStats), ("ms_field", C.c_double), ("ms_classify", C.c_double),
                ("ms_vertices", C.c_double), ("ms_triangles", C.c_double),
                ("ms_filter", C.c_double), ("ms_field_bulk", C.c_double)]

    def as_dict(self):
        d = {k: int(getattr(self, k)) for k, t in self._fields_
             if k != "field" and t is C.c_int64}
        d.update({k: float(getattr(self, k)) for k, t in self._fields_ if t is C.c_double})
        d["field"] = self.field.as_dict()
        return d


class QjgTanhStats(C.Structure):
    _fields_ = [("voxels", C.c_int64), ("overflowed", C.c_int64), ("bad_terms", C.c_int64),
                ("band_voxels", C.c_int64)]


class QjgEnergyItem(C.Structure):
    _fields_ = [("d_params", C.c_void_p), ("n_top", C.c_int32), ("n_bot", C.c_int32),
                ("n", C.c_int64), ("d_xyz", C.c_void_p), ("d_target", C.c_void_p),
                ("slice", C.c_double), ("max_it", C.c_int32), ("pad_", C.c_int32),
                ("escape", C.c_double), ("d_sat", C.c_double), ("d_grad", C.c_void_p),
                ("energy", C.c_double)]


class QjgFitStats(C.Structure):
    _fields_ = [("steps", C.c_int32), ("energy_evals", C.c_int32), ("gradient_evals", C.c_int32),
                ("energy0", C.c_double), ("energy", C.c_double)]


QJG_REQ_FIELD, QJG_REQ_MESH, QJG_REQ_ENERGY = 0, 1, 2
QJG_STATUS_QUEUED, QJG_STATUS_RUNNING, QJG_STATUS_DONE, QJG_STATUS_FAILED = 0, 1, 2, 3


class QjgRequest(C.Structure):
    _fields_ = [("kind", C.c_int32), ("precision", C.c_int32), ("n_top", C.c_int32),
                ("n_bot", C.c_int32), ("top_roots", _dp), ("top_powers", _dp), ("bot_roots", _dp),
                ("bot_powers", _dp), ("sigma_top", C.c_double), ("sigma_bot", C.c_double),
                ("scale", C.c_double), ("grid", QjgGrid), ("max_it", C.c_int32),
                ("escape", C.c_double), ("iso", C.c_double), ("vert_cap", C.c_int64),
                ("tri_cap", C.c_int64), ("params", _dp), ("d_sat", C.c_double),
                ("n_samples", C.c_int64), ("xyz", _dp),
                ("target", _dp), ("out_field", _dp), ("out_verts", _dp),
                ("out_tris", C.POINTER(C.c_int32)), ("out_grad", _dp), ("rel_tol", C.c_double)]


class QjgResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("error", C.c_int32), ("latency_ms", C.c_double),
                ("queue_ms", C.c_double), ("run_ms", C.c_double), ("t_admit_ms", C.c_double),
                ("t_done_ms", C.c_double), ("voxel_iters", C.c_int64), ("refined", C.c_int64),
                ("n_verts", C.c_int64), ("n_tris", C.c_int64), ("energy", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class QjgServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("failed", C.c_int64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("max_ms", C.c_double), ("span_s", C.c_double),
                ("in_use_bytes", C.c_int64), ("peak_in_use_bytes", C.c_int64),
                ("peak_running", C.c_int32), ("pad_", C.c_int32), ("batched", C.c_int64),
                ("batches", C.c_int64), ("max_batch", C.c_int64),
                ("energy_batched", C.c_int64), ("energy_batches", C.c_int64),
                ("max_energy_batch", C.c_int64), ("mesh_batched", C.c_int64)]


class QjgBlmvmSettings(C.Structure):
    _fields_ = [("max_it", C.c_int32), ("ls_max_funcs", C.c_int32), ("fatol", C.c_double),
                ("frtol", C.c_double), ("gatol", C.c_double), ("grtol", C.c_double),
                ("gttol", C.c_double)]


class QjgBlmvmStats(C.Structure):
    _fields_ = [("reason", C.c_int32), ("iterations", C.c_int32), ("evaluations", C.c_int32),
                ("grad_steps", C.c_int32), ("resets", C.c_int32), ("pad_", C.c_int32),
                ("f", C.c_double), ("gnorm", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


class QjgMapState(C.Structure):
    _fields_ = [("n_top", C.c_int32), ("n_bot", C.c_int32), ("top_roots", _dp),
                ("bot_roots", _dp), ("top_powers", _dp), ("bot_powers", _dp),
                ("sigma_top", C.c_double), ("sigma_bot", C.c_double), ("scale", C.c_double)]


QJG_FD_LOG_RATIONAL, QJG_FD_LOG_RATIONAL_BOTTOM, QJG_FD_POLYNOMIAL = 0, 1, 2
QJG_FIT_SCALED_ONLY = 0
QJG_FIT_SCALED = 1
OBJECTIVE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, _dp, _dp, _dp)
MONITOR_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.c_double, C.c_double, _dp)
SDF_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, _dp, C.c_int64, C.POINTER(C.c_int32), C.c_int64,
                     C.POINTER(QjgGrid), _dp)


class QjgToothConfig(C.Structure):
    _fields_ = [("input_path", C.c_char_p), ("checkpoint_path", C.c_char_p),
                ("output_prefix", C.c_char_p), ("fractal_radius", C.c_double),
                ("amp", C.c_double), ("n_levels", C.c_int32), ("levels", C.c_int32 * 8),
                ("pad_", C.c_int32), ("sdf", SDF_FN), ("sdf_user", C.c_void_p),
                ("settings", C.POINTER(QjgBlmvmSettings))]


class QjgToothLevel(C.Structure):
    _fields_ = [("res", C.c_int32), ("reweighted", C.c_int32), ("mesh_tris", C.c_int64),
                ("conformal_score", C.c_double), ("initial_score", C.c_double),
                ("max_score", C.c_double), ("final_score", C.c_double), ("poor_sum", C.c_double),
                ("well_sum", C.c_double), ("solve", QjgBlmvmStats * 4), ("ms", C.c_double),
                ("checkpoints", C.c_int32), ("pad_", C.c_int32)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("solve", "pad_")}
        d["solve"] = [self.solve[i].as_dict() for i in range(4)]
        return d


EXPORTS = {
    "qjg_create": ([C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "qjg_destroy": ([C.c_void_p], None),
    "qjg_last_error": ([C.c_void_p], C.c_char_p),
    "qjg_rootset_upload": ([C.c_void_p, C.c_int32, _dp, _dp, C.c_double, C.c_int32, _dp, _dp,
                            C.c_double, C.c_double, C.POINTER(C.c_int32)], C.c_int),
    "qjg_rootset_free": ([C.c_void_p, C.c_int32], C.c_int),
    "qjg_field": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.POINTER(QjgIter), C.c_int32,
                   C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "qjg_field_host": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.POINTER(QjgIter), _dp, _fp,
                        C.POINTER(QjgFieldStats)], C.c_int),
    "qjg_field_stats_read": ([C.c_void_p, C.c_void_p, C.POINTER(QjgFieldStats)], C.c_int),
    "qjg_field_noalloc": ([C.c_int32, _dp, _dp, C.c_double, C.c_int32, _dp, _dp, C.c_double,
                           C.c_double, C.POINTER(QjgGrid), C.POINTER(QjgIter), C.c_int32,
                           C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "qjg_mesh_field": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.POINTER(QjgIter), C.c_void_p,
                        C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                        C.c_void_p, C.c_int64, C.POINTER(QjgMeshStats), C.c_void_p], C.c_int),
    "qjg_mesh_stream": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.POINTER(QjgIter), C.c_double,
                         C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                         C.POINTER(QjgMeshStats), C.c_void_p], C.c_int),
    "qjg_mesh_prepare": ([C.c_void_p, C.POINTER(QjgGrid), C.c_int32, C.c_int64, C.c_int64],
                         C.c_int),
    "qjg_mesh_stream_async": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.POINTER(QjgIter),
                               C.c_double, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                               C.c_void_p, C.c_int64, C.c_void_p], C.c_int),
    "qjg_mesh_async_result": ([C.c_void_p, C.POINTER(QjgMeshStats)], C.c_int),
    "qjg_set_energy_pairs": ([C.c_int], C.c_int),
    "qjg_set_energy_adjoint_roots": ([C.c_int], C.c_int),
    "qjg_trim": ([C.c_void_p], C.c_int),
    "qjg_set_energy_fast": ([C.c_int], C.c_int),
    "qjg_set_energy_forward_blocks": ([C.c_int], C.c_int),
    "qjg_energy_backward_batch": ([C.c_void_p, C.c_int32, C.POINTER(QjgEnergyItem), C.c_void_p],
                                  C.c_int),
    "qjg_energy_last_work": ([C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
    "qjg_mesh_capture": ([C.c_void_p, C.c_int32], C.c_int),
    "qjg_mesh_edge_cache_write": ([C.c_void_p, C.c_char_p], C.c_int),
    "qjg_mesh_edge_cache_read": ([C.c_char_p, C.POINTER(C.c_int32), C.c_int64,
                                  C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int64,
                                  C.POINTER(C.c_int64)], C.c_int),
    "qjg_centered_gradient": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.c_int32, C.c_int32,
                               C.c_void_p, C.c_void_p, _dp, _dp, C.c_void_p], C.c_int),
    "qjg_tanh_score_grad": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.c_int32,
                             C.POINTER(QjgGrid), C.c_void_p, C.c_double, C.c_double, _dp, _dp,
                             C.c_void_p, C.POINTER(QjgTanhStats), C.c_void_p], C.c_int),
    "qjg_energy_forward": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                            C.c_void_p, C.c_double, C.c_int32, C.c_double, C.c_double, C.c_int32,
                            _dp, C.c_void_p, C.c_void_p], C.c_int),
    "qjg_energy_backward": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                             C.c_void_p, C.c_double, C.c_int32, C.c_double, C.c_double, C.c_int32,
                             _dp, C.c_void_p, C.c_void_p], C.c_int),
    "qjg_fit_lbfgs": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                       C.c_void_p, C.c_double, C.c_int32, C.c_double, C.c_double, C.c_int32,
                       C.c_int32, C.c_int32, _dp, C.POINTER(QjgFitStats), C.c_void_p], C.c_int),
    "qjg_inverted_distance": ([C.c_void_p, C.POINTER(C.c_int32), C.c_void_p, C.c_int32,
                               C.c_void_p, C.c_void_p], C.c_int),
    "qjg_conformal_radius": ([C.c_void_p, C.c_int32, C.POINTER(QjgGrid), C.POINTER(QjgGrid),
                              C.c_void_p, C.c_double, _dp, _dp, _dp, C.c_void_p], C.c_int),
    "qjg_blmvm_defaults": ([C.POINTER(QjgBlmvmSettings)], None),
    "qjg_blmvm": ([C.c_int32, _dp, _dp, _dp, OBJECTIVE_FN, C.c_void_p, MONITOR_FN, C.c_void_p,
                   C.POINTER(QjgBlmvmSettings), C.POINTER(QjgBlmvmStats)], C.c_int),
    "qjg_tanh_fit": ([C.c_void_p, C.c_int32, C.POINTER(QjgMapState), C.POINTER(QjgGrid),
                      C.c_int32, C.POINTER(QjgGrid), C.c_void_p, C.c_double, C.c_double,
                      C.POINTER(QjgBlmvmSettings), MONITOR_FN, C.c_void_p, C.c_void_p,
                      C.POINTER(QjgBlmvmStats), C.c_void_p], C.c_int),
    "qjg_tanh_max_score": ([C.c_void_p, C.POINTER(QjgGrid), C.POINTER(QjgGrid), C.c_void_p, _dp,
                            C.c_void_p], C.c_int),
    "qjg_reweight_inside": ([C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_void_p, _dp, _dp, C.c_void_p], C.c_int),
    "qjg_tooth_optimize": ([C.c_void_p, C.POINTER(QjgToothConfig), C.POINTER(QjgToothLevel),
                            C.c_void_p], C.c_int),
    "qjg_field3d_write": ([C.c_char_p, C.POINTER(C.c_int32), _dp, _dp, C.c_void_p], C.c_int),
    "qjg_field3d_read_header": ([C.c_char_p, C.POINTER(C.c_int32), _dp, _dp], C.c_int),
    "qjg_field3d_read": ([C.c_char_p, C.c_void_p, C.c_int64], C.c_int),
    "qjg_mesh_write_raw": ([C.c_char_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64], C.c_int),
    "qjg_mesh_write_obj": ([C.c_char_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64],
                           C.c_int),
    "qjg_o3d_read_info": ([C.c_char_p, C.POINTER(QjgO3dInfo)], C.c_int),
    "qjg_o3d_read": ([C.c_char_p] + [C.c_void_p] * 7, C.c_int),
    "qjg_o3d_write": ([C.c_char_p, C.POINTER(QjgO3dInfo)] + [C.c_void_p] * 7, C.c_int),
    "qjg_server_create": ([C.c_int, C.c_int32, C.c_int64, C.POINTER(C.c_void_p)], C.c_int),
    "qjg_server_destroy": ([C.c_void_p], None),
    "qjg_server_submit": ([C.c_void_p, C.POINTER(QjgRequest), C.POINTER(C.c_int64)], C.c_int),
    "qjg_server_poll": ([C.c_void_p, C.c_int64, C.POINTER(QjgResult)], C.c_int),
    "qjg_server_wait": ([C.c_void_p, C.c_int64, C.POINTER(QjgResult)], C.c_int),
    "qjg_server_drain": ([C.c_void_p], C.c_int),
    "qjg_server_read_stats": ([C.c_void_p, C.POINTER(QjgServerStats)], C.c_int),
    # measurement hooks (include/quijibo_gpu_bench.h)
    "qjg_set_timing": ([C.c_void_p, C.c_int], C.c_int),
    "qjg_last_timings": ([C.c_void_p, _fp, _fp], C.c_int),
    "qjg_launch_count": ([C.c_void_p], C.c_int64),
    "qjg_fma_probe": ([C.c_int, _dp], C.c_int),
    "qjg_crmath_eval": ([C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p], C.c_int),
    "qjg_set_field32_pairs": ([C.c_int], C.c_int),
}

_lib = None


def load():
    """Load the library (once); raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("CUDA library %s is missing: run `python -m quijibo_gb300.build`"
                               % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in EXPORTS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


class QjgError(RuntimeError):
    pass


def _addr(a):
    """Address of a host numpy array or of a device buffer given as an int."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.ctypes.data


def _io_check(rc, what):
    if rc != 0:
        raise QjgError("%s failed (%d)" % (what, rc))


def field3d_write(path, grid_res, center, lengths, field):
    """FIELD_3D binary file from a host array (Z, Y, X) or a device address."""
    res = (C.c_int32 * 3)(*[int(v) for v in grid_res])
    c = np.ascontiguousarray(center, dtype=np.float64)
    ln = np.ascontiguousarray(lengths, dtype=np.float64)
    if not isinstance(field, int):
        field = np.ascontiguousarray(field, dtype=np.float64)
    _io_check(load().qjg_field3d_write(str(path).encode(), res, c.ctypes.data_as(_dp),
                                       ln.ctypes.data_as(_dp), C.c_void_p(_addr(field))),
              "qjg_field3d_write")


def field3d_read(path):
    """(res (X, Y, Z), center, lengths, field[Z, Y, X]) of a FIELD_3D file."""
    res = (C.c_int32 * 3)()
    c = np.empty(3)
    ln = np.empty(3)
    L = load()
    _io_check(L.qjg_field3d_read_header(str(path).encode(), res, c.ctypes.data_as(_dp),
                                        ln.ctypes.data_as(_dp)), "qjg_field3d_read_header")
    X, Y, Z = res[0], res[1], res[2]
    f = np.empty((Z, Y, X))
    _io_check(L.qjg_field3d_read(str(path).encode(), C.c_void_p(f.ctypes.data), f.size),
              "qjg_field3d_read")
    return (X, Y, Z), c, ln, f


def mesh_write_raw(path, verts, tris, n_verts=None, n_tris=None):
    """TRIANGLE_MESH raw stream from FP64 vertices and int32 triangles (host
    arrays, or device addresses with explicit counts)."""
    if not isinstance(verts, int):
        verts = np.ascontiguousarray(verts, dtype=np.float64)
        n_verts = len(verts.reshape(-1, 3))
    if not isinstance(tris, int):
        tris = np.ascontiguousarray(tris, dtype=np.int32)
        n_tris = len(tris.reshape(-1, 3))
    _io_check(load().qjg_mesh_write_raw(str(path).encode(), C.c_void_p(_addr(verts)), n_verts,
                                        C.c_void_p(_addr(tris)), n_tris), "qjg_mesh_write_raw")


def mesh_write_obj(path, verts, tris, n_verts=None, n_tris=None, fp32=None):
    """OBJ as TRIANGLE_MESH::writeOBJ prints it.  Host arrays (float64 or
    float32 vertices) or device addresses (fp32 says which) with counts."""
    if not isinstance(verts, int):
        fp32 = verts.dtype == np.float32
        verts = np.ascontiguousarray(verts)
        n_verts = len(verts.reshape(-1, 3))
    if not isinstance(tris, int):
        tris = np.ascontiguousarray(tris, dtype=np.int32)
        n_tris = len(tris.reshape(-1, 3))
    v64 = None if fp32 else _addr(verts)
    v32 = _addr(verts) if fp32 else None
    _io_check(load().qjg_mesh_write_obj(str(path).encode(), C.c_void_p(v64), C.c_void_p(v32),
                                        n_verts, C.c_void_p(_addr(tris)), n_tris),
              "qjg_mesh_write_obj")


FIELD_NAMES = ("fractal", "distance", "curvature")


def o3d_read(path):
    """An optimizer state file: dict with the RootSet fields, the grid
    (res, center, lengths), exp scaling, history count and the three fields
    as (res, center, lengths, data[Z, Y, X])."""
    L = load()
    info = QjgO3dInfo()
    _io_check(L.qjg_o3d_read_info(str(path).encode(), C.byref(info)), "qjg_o3d_read_info")
    nt, nb = info.n_top, info.n_bot
    tr, tp = np.empty((nt, 4)), np.empty(nt)
    br, bp = np.empty((nb, 4)), np.empty(nb)
    fields = []
    for k in range(3):
        res = tuple(info.field_res[k])
        n = int(np.prod(res)) if min(res) > 0 else 0
        fields.append((res, tuple(info.field_center[k]), tuple(info.field_lengths[k]),
                       np.empty(res[::-1] if n else 0)))
    p = lambda a: C.c_void_p(a.ctypes.data if a.size else 0)  # noqa: E731
    _io_check(L.qjg_o3d_read(str(path).encode(), p(tr), p(tp), p(br), p(bp),
                             *[p(f[3]) for f in fields]), "qjg_o3d_read")
    return {"top_roots": tr, "top_powers": tp, "sigma_top": info.sigma_top,
            "bottom_roots": br, "bottom_powers": bp, "sigma_bottom": info.sigma_bot,
            "scale": info.exp_scaling, "res": tuple(info.res), "center": tuple(info.center),
            "lengths": tuple(info.lengths), "history": info.history,
            **{name: f for name, f in zip(FIELD_NAMES, fields)}}


def o3d_write(path, rs, grid_res, center, lengths, fields, history=0):
    """Write a state file; `fields` maps fractal / distance / curvature to
    (res, center, lengths, data) (missing ones are written empty)."""
    info = QjgO3dInfo()
    info.res[:] = [int(v) for v in grid_res]
    info.center[:] = list(center)
    info.lengths[:] = list(lengths)
    info.n_top, info.n_bot = rs.n_top, rs.n_bottom
    info.sigma_top, info.sigma_bot, info.exp_scaling = rs.sigma_top, rs.sigma_bottom, rs.scale
    info.history = history
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return C.c_void_p(a.ctypes.data if a.size else 0)

    data = []
    for k, name in enumerate(FIELD_NAMES):
        if name in fields:
            res, c, ln, d = fields[name]
            info.field_res[k][:] = [int(v) for v in res]
            info.field_center[k][:] = list(c)
            info.field_lengths[k][:] = list(ln)
            data.append(arr(d))
        else:
            data.append(C.c_void_p(0))
    _io_check(load().qjg_o3d_write(str(path).encode(), C.byref(info), arr(rs.top_roots),
                                   arr(rs.top_powers), arr(rs.bottom_roots), arr(rs.bottom_powers),
                                   *data), "qjg_o3d_write")


def mesh_edge_cache_read(path):
    """(edges [n, 2, 3] corner pairs, cubes [m, 4] (flag, x, y, z)) of an edge-cache file."""
    L = load()
    ne, nc = C.c_int64(), C.c_int64()
    rc = L.qjg_mesh_edge_cache_read(str(path).encode(), None, 0, C.byref(ne), None, 0, C.byref(nc))
    if rc:
        raise QjgError("qjg_mesh_edge_cache_read(%s) failed (%d)" % (path, rc))
    e = np.zeros(6 * ne.value, dtype=np.int32)
    c = np.zeros(4 * nc.value, dtype=np.int32)
    rc = L.qjg_mesh_edge_cache_read(str(path).encode(), e.ctypes.data_as(C.POINTER(C.c_int32)),
                                    ne.value, C.byref(ne), c.ctypes.data_as(C.POINTER(C.c_int32)),
                                    nc.value, C.byref(nc))
    if rc:
        raise QjgError("qjg_mesh_edge_cache_read(%s) failed (%d)" % (path, rc))
    return e.reshape(-1, 2, 3), c.reshape(-1, 4)


def set_energy_pairs(on):
    """Energy forward kernel: two samples per lane (True) or one (False)."""
    load().qjg_set_energy_pairs(int(bool(on)))


def set_energy_adjoint_roots(on):
    """FP32 adjoint: roots spread over a group of 16 lanes per sample (True,
    the default, for maps of at most 64 roots a side) or one lane per sample
    walking the roots (False)."""
    load().qjg_set_energy_adjoint_roots(int(bool(on)))


def set_energy_fast(on):
    """FP32 energy's polar power: fast hardware approximations (True, the
    default) or the accurate device functions (False)."""
    if load().qjg_set_energy_fast(int(bool(on))) != 0:
        raise QjgError("qjg_set_energy_fast failed")


def set_energy_forward_blocks(per_sm):
    """Energy forward kernel's blocks per SM (0: the sizing rule), for sweeps."""
    if load().qjg_set_energy_forward_blocks(int(per_sm)) != 0:
        raise QjgError("qjg_set_energy_forward_blocks(%d) failed" % per_sm)


def set_field32_pairs(on):
    """Process-wide FP32 bulk kernel form: True two voxels per lane (default)."""
    load().qjg_set_field32_pairs(int(bool(on)))


def crmath_eval(name, d_x, d_y, n, stream=None):
    """y[i] = f(x[i]) on the device with the correctly rounded FP64 function
    `name` (one of CRM_FUNCTIONS) of the QJG_LIBM_CR form; device pointers."""
    rc = load().qjg_crmath_eval(CRM_FUNCTIONS.index(name), C.c_void_p(d_x), C.c_void_p(d_y),
                                int(n), C.c_void_p(stream or 0))
    if rc != 0:
        raise QjgError("qjg_crmath_eval failed (%d)" % rc)


def fma_probe(device=0):
    """Achieved FP32 TFLOP/s of an FMA-chain probe kernel on every SM."""
    v = C.c_double()
    rc = load().qjg_fma_probe(device, C.byref(v))
    if rc != 0:
        raise QjgError("qjg_fma_probe failed (%d)" % rc)
    return v.value


def blmvm_settings(**kw):
    """The solver defaults (TAO's, with toothOptimizer's tolerances), with
    any field overridden by keyword."""
    st = QjgBlmvmSettings()
    load().qjg_blmvm_defaults(C.byref(st))
    for k, v in kw.items():
        setattr(st, k, v)
    return st


def _monitor_fn(monitor):
    if monitor is None:
        return MONITOR_FN(), None

    def cb(user, it, f, gnorm, x):
        try:
            return int(bool(monitor(it, f, gnorm, x)))
        except Exception:
            return 1
    fn = MONITOR_FN(cb)
    return fn, fn


def blmvm(fun, x0, lower, upper, settings=None, monitor=None):
    """Minimise fun(x) -> (f, grad) over lower <= x <= upper with the
    library's BLMVM (qjg_blmvm).  Returns (x, stats dict).  monitor(iter, f,
    gnorm, x_ptr) returning True ends the run."""
    x = np.array(x0, dtype=np.float64)
    lo = np.ascontiguousarray(lower, dtype=np.float64)
    hi = np.ascontiguousarray(upper, dtype=np.float64)
    n = len(x)
    err = []

    def cb(user, nn, xp, fp, gp):
        try:
            f, g = fun(np.ctypeslib.as_array(xp, (nn,)).copy())
            fp[0] = f
            gp_arr = np.ctypeslib.as_array(gp, (nn,))
            gp_arr[:] = g
            return 0
        except Exception as e:  # reported after the solver returns
            err.append(e)
            return 99
    fn = OBJECTIVE_FN(cb)
    mfn, _keep = _monitor_fn(monitor)
    st = QjgBlmvmStats()
    rc = load().qjg_blmvm(n, x.ctypes.data_as(_dp), lo.ctypes.data_as(_dp), hi.ctypes.data_as(_dp),
                          fn, None, mfn, None, C.byref(settings) if settings else None,
                          C.byref(st))
    if err:
        raise err[0]
    if rc != 0:
        raise QjgError("qjg_blmvm failed (%d)" % rc)
    return x, st.as_dict()


def _arr(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(shape) if shape else a


class Context:
    """One device context (qjg_create); root sets stay resident on it."""

    def __init__(self, device=0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.qjg_create(device, C.byref(h))
        if rc != 0:
            raise QjgError("qjg_create(%d) failed with %d" % (device, rc))
        self.h = h

    def close(self):
        if self.h:
            self.L.qjg_destroy(self.h)
            self.h = None

    def trim(self):
        """Return the device memory the context's pool keeps to the device."""
        self._check(self.L.qjg_trim(self.h), "qjg_trim")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise QjgError("%s failed (%d): %s" % (what, rc, self.L.qjg_last_error(self.h).decode()))

    def upload(self, rs: RootSet) -> int:
        tr, tp = _arr(rs.top_roots, (-1, 4)), _arr(rs.top_powers)
        br, bp = _arr(rs.bottom_roots, (-1, 4)), _arr(rs.bottom_powers)
        out = C.c_int32()
        p = lambda a: a.ctypes.data_as(_dp) if a.size else None
        self._check(self.L.qjg_rootset_upload(self.h, len(tp), p(tr), p(tp), float(rs.sigma_top),
                                              len(bp), p(br), p(bp), float(rs.sigma_bottom),
                                              float(rs.scale), C.byref(out)), "qjg_rootset_upload")
        return out.value

    def free(self, handle):
        self._check(self.L.qjg_rootset_free(self.h, handle), "qjg_rootset_free")

    @staticmethod
    def iter_params(max_it, escape, precision=QJG_FP64, refine_pow=QJG_REFINE_POW, want_de=False,
                    band_h=2.0, field_tol=1e-3, rel_tol=0.0, lagrange=False,
                    libm=QJG_LIBM_DEVICE):
        return QjgIter(int(max_it), int(precision), int(refine_pow), int(bool(want_de)),
                       float(escape), float(band_h), float(field_tol), float(rel_tol),
                       int(bool(lagrange)), int(libm))

    def field(self, handle, grid: Grid, it: QjgIter, d_field, d_de=None, z0=0, z1=None,
              stream=None):
        """Device-pointer call: d_field / d_de are CUDA device addresses (ints)."""
        z1 = grid.res[2] if z1 is None else z1
        self._check(self.L.qjg_field(self.h, handle, C.byref(QjgGrid.of(grid)), C.byref(it), z0, z1,
                                     C.c_void_p(d_field), C.c_void_p(d_de or 0),
                                     C.c_void_p(stream or 0)), "qjg_field")

    def stats(self, stream=None):
        st = QjgFieldStats()
        self._check(self.L.qjg_field_stats_read(self.h, C.c_void_p(stream or 0), C.byref(st)),
                    "qjg_field_stats_read")
        return st.as_dict()

    def inverted_distance(self, res, d_dist, normalized, d_out, stream=None):
        """FIELD_3D::invertedDistance[Normalized] on device buffers."""
        r = (C.c_int32 * 3)(*[int(v) for v in res])
        self._check(self.L.qjg_inverted_distance(self.h, r, C.c_void_p(d_dist), int(normalized),
                                                 C.c_void_p(d_out), C.c_void_p(stream or 0)),
                    "qjg_inverted_distance")

    def conformal_radius(self, handle, grid: Grid, dist_grid: Grid, d_dist, alpha=10.0,
                         stream=None):
        """estimateConformalRadius: (lowest score, threshold, exp(-threshold))."""
        sc, th, es = C.c_double(), C.c_double(), C.c_double()
        self._check(self.L.qjg_conformal_radius(self.h, handle, C.byref(QjgGrid.of(grid)),
                                                C.byref(QjgGrid.of(dist_grid)), C.c_void_p(d_dist),
                                                float(alpha), C.byref(sc), C.byref(th), C.byref(es),
                                                C.c_void_p(stream or 0)), "qjg_conformal_radius")
        return sc.value, th.value, es.value

    def set_timing(self, on=True):
        self._check(self.L.qjg_set_timing(self.h, int(on)), "qjg_set_timing")

    def last_timings(self):
        a, b = C.c_float(), C.c_float()
        self._check(self.L.qjg_last_timings(self.h, C.byref(a), C.byref(b)), "qjg_last_timings")
        return a.value, b.value

    def launch_count(self):
        return int(self.L.qjg_launch_count(self.h))

    def field_host(self, handle, grid: Grid, it: QjgIter, de=False, out=None, de_out=None):
        """Host-buffer call; returns (field[Z,Y,X] float64, de or None, stats)."""
        X, Y, Z = grid.res
        f = out if out is not None else np.empty((Z, Y, X))
        d = (de_out if de_out is not None else np.empty((Z, Y, X), dtype=np.float32)) if de else None
        st = QjgFieldStats()
        self._check(self.L.qjg_field_host(self.h, handle, C.byref(QjgGrid.of(grid)), C.byref(it),
                                          f.ctypes.data_as(_dp),
                                          d.ctypes.data_as(_fp) if d is not None else None,
                                          C.byref(st)), "qjg_field_host")
        return f, d, st.as_dict()

    def mesh_field(self, handle, grid: Grid, it, d_field, edge_mode, iso=0.0, slab_nz=0,
                   d_verts64=0, d_verts32=0, vert_cap=0, d_tris=0, tri_cap=0, stream=None,
                   check=True):
        """Stored-field mesher on device buffers; returns (rc, stats dict)."""
        st = QjgMeshStats()
        rc = self.L.qjg_mesh_field(self.h, handle if handle is not None else -1,
                                   C.byref(QjgGrid.of(grid)), C.byref(it) if it is not None else None,
                                   C.c_void_p(d_field), int(edge_mode), float(iso), int(slab_nz),
                                   C.c_void_p(d_verts64), C.c_void_p(d_verts32), int(vert_cap),
                                   C.c_void_p(d_tris), int(tri_cap), C.byref(st),
                                   C.c_void_p(stream or 0))
        if check:
            self._check(rc, "qjg_mesh_field")
        return rc, st.as_dict()

    def mesh_stream(self, handle, grid: Grid, it, iso=0.0, slab_nz=0, d_verts64=0, d_verts32=0,
                    vert_cap=0, d_tris=0, tri_cap=0, stream=None, check=True):
        """Streaming mesher (field computed per slab); returns (rc, stats dict)."""
        st = QjgMeshStats()
        rc = self.L.qjg_mesh_stream(self.h, handle, C.byref(QjgGrid.of(grid)), C.byref(it),
                                    float(iso), int(slab_nz), C.c_void_p(d_verts64),
                                    C.c_void_p(d_verts32), int(vert_cap), C.c_void_p(d_tris),
                                    int(tri_cap), C.byref(st), C.c_void_p(stream or 0))
        if check:
            self._check(rc, "qjg_mesh_stream")
        return rc, st.as_dict()

    def mesh_prepare(self, grid: Grid, vert_cap, tri_cap, slab_nz=0):
        """Size the context for qjg_mesh_stream_async (device allocations)."""
        self._check(self.L.qjg_mesh_prepare(self.h, C.byref(QjgGrid.of(grid)), int(slab_nz),
                                            int(vert_cap), int(tri_cap)), "qjg_mesh_prepare")

    def mesh_stream_async(self, handle, grid: Grid, it, iso=0.0, slab_nz=0, d_verts64=0,
                          d_verts32=0, vert_cap=0, d_tris=0, tri_cap=0, stream=None):
        """Enqueue the streaming mesher as a fixed launch sequence (no host
        wait inside; capturable); read the stats with mesh_async_result."""
        self._check(self.L.qjg_mesh_stream_async(self.h, handle, C.byref(QjgGrid.of(grid)),
                                                 C.byref(it), float(iso), int(slab_nz),
                                                 C.c_void_p(d_verts64), C.c_void_p(d_verts32),
                                                 int(vert_cap), C.c_void_p(d_tris), int(tri_cap),
                                                 C.c_void_p(stream or 0)),
                    "qjg_mesh_stream_async")

    def mesh_async_result(self, check=True):
        """(rc, stats dict) of the last mesh_stream_async run (after its stream ran)."""
        st = QjgMeshStats()
        rc = self.L.qjg_mesh_async_result(self.h, C.byref(st))
        if check:
            self._check(rc, "qjg_mesh_async_result")
        return rc, st.as_dict()

    def energy_batch(self, items, stream=None):
        """qjg_energy_backward_batch over dicts with d_params, n_top, n_bot, n,
        d_xyz, d_target, max_it, escape, d_sat, slice, d_grad (device
        addresses as ints); returns the energies."""
        arr = (QjgEnergyItem * len(items))()
        for a, it in zip(arr, items):
            a.d_params, a.n_top, a.n_bot, a.n = it["d_params"], it["n_top"], it["n_bot"], it["n"]
            a.d_xyz, a.d_target, a.slice = it["d_xyz"], it["d_target"], it.get("slice", 0.0)
            a.max_it, a.escape, a.d_sat = it["max_it"], it["escape"], it.get("d_sat", 1.0)
            a.d_grad = it["d_grad"]
        self._check(self.L.qjg_energy_backward_batch(self.h, len(items), arr, C.c_void_p(stream or 0)),
                    "qjg_energy_backward_batch")
        return [a.energy for a in arr]

    def energy_last_work(self):
        """(forward map applications, adjoint orbit steps) of the last energy call."""
        a, b = C.c_int64(), C.c_int64()
        self._check(self.L.qjg_energy_last_work(self.h, C.byref(a), C.byref(b)),
                    "qjg_energy_last_work")
        return a.value, b.value

    def mesh_capture(self, on=True):
        """Keep each mesher call's edge-cache lists (qjg_mesh_capture)."""
        self._check(self.L.qjg_mesh_capture(self.h, int(bool(on))), "qjg_mesh_capture")

    def mesh_edge_cache_write(self, path):
        """The last captured mesher call as the reference's edge-cache file."""
        self._check(self.L.qjg_mesh_edge_cache_write(self.h, str(path).encode()),
                    "qjg_mesh_edge_cache_write")

    def centered_gradient(self, handle, grid: Grid, max_it, kind, d_dist, n_entries, d_curv=0,
                          stream=None):
        """OPTIMIZE_3D's central-difference root gradients (QJG_FD_*): (score
        of the unmoved map, gradient of n_entries = 4 x the moved roots)."""
        score = C.c_double()
        grad = np.empty(n_entries)
        self._check(self.L.qjg_centered_gradient(self.h, handle, C.byref(QjgGrid.of(grid)),
                                                 int(max_it), int(kind), C.c_void_p(d_dist),
                                                 C.c_void_p(d_curv or 0), grad.ctypes.data_as(_dp),
                                                 C.byref(score), C.c_void_p(stream or 0)),
                    "qjg_centered_gradient")
        return score.value, grad

    def tanh_score_grad(self, handle, grid: Grid, max_it, wgrid: Grid, d_weights, n_params,
                        alpha=10.0, threshold=0.0, d_field=0, stream=None):
        """(score, grad [log s, bottom exps, top exps, sigma_t, sigma_b], stats)."""
        score = C.c_double()
        grad = np.empty(n_params)
        st = QjgTanhStats()
        self._check(self.L.qjg_tanh_score_grad(self.h, handle, C.byref(QjgGrid.of(grid)),
                                               int(max_it), C.byref(QjgGrid.of(wgrid)),
                                               C.c_void_p(d_weights), float(alpha),
                                               float(threshold), C.byref(score),
                                               grad.ctypes.data_as(_dp), C.c_void_p(d_field),
                                               C.byref(st), C.c_void_p(stream or 0)),
                    "qjg_tanh_score_grad")
        return score.value, grad, {k: int(getattr(st, k)) for k, _ in st._fields_}

    def tanh_fit(self, mode, rs: RootSet, grid: Grid, max_it, wgrid: Grid, d_weights,
                 alpha=10.0, threshold=0.0, settings=None, monitor=None, d_field=0, stream=None):
        """One BLMVM solve of toothOptimizer (QJG_FIT_SCALED_ONLY or
        QJG_FIT_SCALED); rs's exponents, power scalars and scale are updated
        in place.  Returns the solver stats."""
        tr, br = _arr(rs.top_roots, (-1, 4)), _arr(rs.bottom_roots, (-1, 4))
        tp, bp = _arr(rs.top_powers).copy(), _arr(rs.bottom_powers).copy()
        p = lambda a: a.ctypes.data_as(_dp) if a.size else None
        ms = QjgMapState(len(tp), len(bp), p(tr), p(br), p(tp), p(bp), float(rs.sigma_top),
                         float(rs.sigma_bottom), float(rs.scale))
        mfn, _keep = _monitor_fn(monitor)
        st = QjgBlmvmStats()
        self._check(self.L.qjg_tanh_fit(self.h, int(mode), C.byref(ms), C.byref(QjgGrid.of(grid)),
                                        int(max_it), C.byref(QjgGrid.of(wgrid)),
                                        C.c_void_p(d_weights), float(alpha), float(threshold),
                                        C.byref(settings) if settings else None, mfn, None,
                                        C.c_void_p(d_field), C.byref(st), C.c_void_p(stream or 0)),
                    "qjg_tanh_fit")
        rs.top_powers, rs.bottom_powers = tp, bp
        rs.sigma_top, rs.sigma_bottom, rs.scale = ms.sigma_top, ms.sigma_bot, ms.scale
        return st.as_dict()

    def tanh_max_score(self, grid: Grid, wgrid: Grid, d_weights, stream=None):
        """sum |w| at the cell centres (computeMaximumScaledPowerRationalScore)."""
        out = C.c_double()
        self._check(self.L.qjg_tanh_max_score(self.h, C.byref(QjgGrid.of(grid)),
                                              C.byref(QjgGrid.of(wgrid)), C.c_void_p(d_weights),
                                              C.byref(out), C.c_void_p(stream or 0)),
                    "qjg_tanh_max_score")
        return out.value

    def reweight_inside(self, n, d_md, d_fd, d_w, d_out, stream=None):
        """buildReweightedInsideField's arithmetic; returns (poor_sum, well_sum)."""
        poor, well = C.c_double(), C.c_double()
        self._check(self.L.qjg_reweight_inside(self.h, int(n), C.c_void_p(d_md), C.c_void_p(d_fd),
                                               C.c_void_p(d_w), C.c_void_p(d_out),
                                               C.byref(poor), C.byref(well),
                                               C.c_void_p(stream or 0)), "qjg_reweight_inside")
        return poor.value, well.value

    def tooth_optimize(self, input_path, levels=(25, 50, 97), fractal_radius=4.0, amp=-1.0,
                       output_prefix=None, checkpoint_path=None, sdf=None, settings=None,
                       stream=None):
        """toothOptimizer's run (qjg_tooth_optimize); per-level stats.
        sdf(verts (V,3), tris (T,3), grid) -> signed distance on grid
        (x fastest) enables the reweighted solve."""
        cfg = QjgToothConfig()
        enc = lambda p: str(p).encode() if p is not None else None  # noqa: E731
        cfg.input_path = enc(input_path)
        cfg.checkpoint_path = enc(checkpoint_path)
        cfg.output_prefix = enc(output_prefix)
        cfg.fractal_radius = float(fractal_radius)
        cfg.amp = float(amp)
        cfg.n_levels = len(levels)
        for i, r in enumerate(levels):
            cfg.levels[i] = int(r)
        err = []
        if sdf is not None:
            def cb(user, vp, nv, tp, nt, gp, out):
                try:
                    v = np.ctypeslib.as_array(vp, (int(nv), 3)).copy() if nv else np.zeros((0, 3))
                    t = (np.ctypeslib.as_array(tp, (int(nt), 3)).copy() if nt
                         else np.zeros((0, 3), dtype=np.int32))
                    gr = gp.contents
                    n = gr.res[0] * gr.res[1] * gr.res[2]
                    np.ctypeslib.as_array(out, (n,))[:] = np.asarray(sdf(v, t, gr)).ravel()
                    return 0
                except Exception as e:
                    err.append(e)
                    return 1
            cfg.sdf = SDF_FN(cb)
        if settings is not None:
            cfg.settings = C.pointer(settings)
        out = (QjgToothLevel * len(levels))()
        rc = self.L.qjg_tooth_optimize(self.h, C.byref(cfg), out, C.c_void_p(stream or 0))
        if err:
            raise err[0]
        self._check(rc, "qjg_tooth_optimize")
        return [out[i].as_dict() for i in range(len(levels))]

    def energy(self, d_params, n_top, n_bot, n, d_xyz, d_target, max_it, escape, slice_=0.0,
               precision=QJG_FP64, d_grad=0, d_iters=0, d_sat=1.0, stream=None):
        """Squared-error energy (and, with d_grad, its gradient into d_grad)."""
        e = C.c_double()
        if d_grad:
            rc = self.L.qjg_energy_backward(self.h, C.c_void_p(d_params), n_top, n_bot, int(n),
                                            C.c_void_p(d_xyz), C.c_void_p(d_target), float(slice_),
                                            int(max_it), float(escape), float(d_sat),
                                            int(precision), C.byref(e), C.c_void_p(d_grad),
                                            C.c_void_p(stream or 0))
            self._check(rc, "qjg_energy_backward")
        else:
            rc = self.L.qjg_energy_forward(self.h, C.c_void_p(d_params), n_top, n_bot, int(n),
                                           C.c_void_p(d_xyz), C.c_void_p(d_target), float(slice_),
                                           int(max_it), float(escape), float(d_sat),
                                           int(precision), C.byref(e), C.c_void_p(d_iters),
                                           C.c_void_p(stream or 0))
            self._check(rc, "qjg_energy_forward")
        return e.value


def _fit(self, d_params, n_top, n_bot, n, d_xyz, d_target, max_it, escape, steps, history=8,
         slice_=0.0, precision=QJG_FP32, d_sat=1.0, stream=None):
    """Device L-BFGS fit; returns (energies per step, stats dict)."""
    en = np.zeros(steps + 1)
    st = QjgFitStats()
    self._check(self.L.qjg_fit_lbfgs(self.h, C.c_void_p(d_params), n_top, n_bot, int(n),
                                     C.c_void_p(d_xyz), C.c_void_p(d_target), float(slice_),
                                     int(max_it), float(escape), float(d_sat), int(precision),
                                     int(steps),
                                     int(history), en.ctypes.data_as(_dp), C.byref(st),
                                     C.c_void_p(stream or 0)), "qjg_fit_lbfgs")
    d = {k: getattr(st, k) for k, _ in st._fields_}
    return en[:st.steps + 1], d


Context.fit_lbfgs = _fit


def params_of(rs: RootSet):
    """The energy parameter vector [top roots | bottom roots | top exps |
    bottom exps | log s] of a root set (effective exponents sigma * e)."""
    return np.concatenate([np.asarray(rs.top_roots, dtype=np.float64).reshape(-1),
                           np.asarray(rs.bottom_roots, dtype=np.float64).reshape(-1),
                           rs.sigma_top * np.asarray(rs.top_powers, dtype=np.float64),
                           rs.sigma_bottom * np.asarray(rs.bottom_powers, dtype=np.float64),
                           [np.log(rs.scale)]])


def rootset_of(params, n_top, n_bot):
    """Inverse of params_of (sigma = 1)."""
    p = np.asarray(params, dtype=np.float64)
    nr = n_top + n_bot
    r = p[:4 * nr].reshape(nr, 4)
    e = p[4 * nr:5 * nr]
    return RootSet(top_roots=r[:n_top].copy(), top_powers=e[:n_top].copy(),
                   bottom_roots=r[n_top:].copy(), bottom_powers=e[n_top:].copy(),
                   scale=float(np.exp(p[5 * nr])))


class Server:
    """Continuous-batching request server (qjg_server_*)."""

    def __init__(self, device=0, workers=8, hbm_budget=64 << 30):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.qjg_server_create(device, workers, int(hbm_budget), C.byref(h))
        if rc != 0:
            raise QjgError("qjg_server_create failed (%d)" % rc)
        self.h = h
        self._keep = {}

    def close(self):
        if self.h:
            self.L.qjg_server_destroy(self.h)
            self.h = None

    def submit(self, kind, rs=None, grid=None, max_it=20, escape=2.0, precision=QJG_FP32_REFINE,
               iso=0.0, vert_cap=0, tri_cap=0, params=None, xyz=None, target=None,
               out_field=None, out_verts=None, out_tris=None, out_grad=None, d_sat=1.0,
               rel_tol=0.0):
        r = QjgRequest()
        r.kind, r.precision, r.max_it, r.escape, r.iso = kind, precision, max_it, escape, iso
        r.d_sat, r.rel_tol = d_sat, rel_tol
        keep = []

        def arr(a, shape=None):
            a = _arr(a, shape)
            keep.append(a)
            return a.ctypes.data_as(_dp) if a.size else None

        if rs is not None:
            r.n_top, r.n_bot = rs.n_top, rs.n_bottom
            r.top_roots, r.top_powers = arr(rs.top_roots, (-1, 4)), arr(rs.top_powers)
            r.bot_roots, r.bot_powers = arr(rs.bottom_roots, (-1, 4)), arr(rs.bottom_powers)
            r.sigma_top, r.sigma_bot, r.scale = rs.sigma_top, rs.sigma_bottom, rs.scale
        if grid is not None:
            r.grid = QjgGrid.of(grid)
        r.vert_cap, r.tri_cap = int(vert_cap), int(tri_cap)
        if params is not None:
            r.params = arr(params)
            r.n_samples = len(target)
            r.xyz, r.target = arr(xyz, (-1, 3)), arr(target)
        for name, a in (("out_field", out_field), ("out_verts", out_verts), ("out_grad", out_grad)):
            if a is not None:
                keep.append(a)
                setattr(r, name, a.ctypes.data_as(_dp))
        if out_tris is not None:
            keep.append(out_tris)
            r.out_tris = out_tris.ctypes.data_as(C.POINTER(C.c_int32))
        t = C.c_int64()
        rc = self.L.qjg_server_submit(self.h, C.byref(r), C.byref(t))
        if rc != 0:
            raise QjgError("qjg_server_submit failed (%d)" % rc)
        self._keep[t.value] = keep
        return t.value

    def wait(self, ticket):
        res = QjgResult()
        rc = self.L.qjg_server_wait(self.h, ticket, C.byref(res))
        if rc != 0:
            raise QjgError("qjg_server_wait failed (%d)" % rc)
        self._keep.pop(ticket, None)
        return res.as_dict()

    def drain(self):
        self.L.qjg_server_drain(self.h)

    def stats(self):
        st = QjgServerStats()
        self.L.qjg_server_read_stats(self.h, C.byref(st))
        return {k: getattr(st, k) for k, _ in st._fields_}
