"""ctypes loader for the FP64 k-Shape oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py as the checker / timed CPU baseline.  The product never
imports it.  See oracle.h for what each function restates.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

MODE_COMPAT, MODE_CANONICAL, MODE_PYREF = 0, 1, 2

_i64 = ctypes.c_int64
_int = ctypes.c_int
_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_fp = ctypes.POINTER(ctypes.c_float)


class OrJob(ctypes.Structure):
    _fields_ = [("data", _fp), ("n", _i64), ("m", _int), ("k", _int), ("mode", _int),
                ("init_chose", _int), ("init_labels", _i32p), ("seed", ctypes.c_uint32),
                ("max_iter", _int), ("restart", _int)]


class OrResult(ctypes.Structure):
    _fields_ = [("labels", _i32p), ("centroids", _dp), ("iterations", _int), ("sum_class", _int),
                ("restarted", _int), ("inertia", ctypes.c_double), ("min_margin", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import importlib.util
            spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
            b = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(b)
            b.build_oracle()
        L = ctypes.CDLL(LIB_PATH)
        L.or_fft_size.restype = _int
        L.or_fft_size.argtypes = [_int, _int]
        L.or_znorm.argtypes = [_dp, _i64, _int, _int]
        L.or_ncc.argtypes = [_dp, _dp, _int, _int, _dp]
        L.or_ncc_naive.argtypes = [_dp, _dp, _int, _int, _dp]
        L.or_align.restype = _int
        L.or_align.argtypes = [_dp, _dp, _int, _int, _dp]
        L.or_shift_row.argtypes = [_dp, _int, _int, _dp]
        L.or_assign.argtypes = [_dp, _dp, _i64, _int, _int, _int, _int, _i32p, _dp, _i32p, _dp]
        L.or_extract.restype = _int
        L.or_extract.argtypes = [_dp, _i32p, _dp, _i64, _int, _int, _int, _int, _i32p]
        L.or_top_eig_jacobi.restype = ctypes.c_double
        L.or_top_eig_jacobi.argtypes = [_dp, _int, _dp]
        L.or_random_select.argtypes = [_i64, _int, ctypes.c_uint32, _i32p]
        L.or_kshape.restype = _int
        L.or_kshape.argtypes = [ctypes.POINTER(OrJob), ctypes.POINTER(OrResult)]
        L.or_ari.restype = ctypes.c_double
        L.or_ari.argtypes = [_i32p, _i32p, _i64]
        L.or_k_from_labels.restype = _int
        L.or_k_from_labels.argtypes = [_i32p, _i64]
        L.or_generate.restype = _int
        L.or_generate.argtypes = [_i64, _int, _int, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                  _fp, _i32p]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_i32p)


def fft_size(m, mode):
    return lib().or_fft_size(int(m), int(mode))


def znorm(x, ddof=1):
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    n, m = x.shape
    lib().or_znorm(_d(x), n, m, ddof)
    return x


def ncc(x, y, F, naive=False):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    m = x.shape[0]
    out = np.zeros(2 * m - 1)
    (lib().or_ncc_naive if naive else lib().or_ncc)(_d(x), _d(y), m, F, _d(out))
    return out


def align(center, member, F):
    c = np.ascontiguousarray(center, dtype=np.float64)
    x = np.ascontiguousarray(member, dtype=np.float64)
    out = np.zeros_like(x)
    s = lib().or_align(_d(c), _d(x), x.shape[0], F, _d(out))
    return s, out


def shift_row(x, shift):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    lib().or_shift_row(_d(x), x.shape[0], int(shift), _d(out))
    return out


def assign(X, C, F, clamp2=True):
    X = np.ascontiguousarray(X, dtype=np.float64)
    C = np.ascontiguousarray(C, dtype=np.float64)
    n, m = X.shape
    k = C.shape[0]
    labels = np.zeros(n, np.int32)
    dist = np.zeros(n)
    shift = np.zeros(n, np.int32)
    margin = np.zeros(n)
    lib().or_assign(_d(X), _d(C), n, m, k, F, int(clamp2), _i(labels), _d(dist), _i(shift), _d(margin))
    return labels, dist, shift, margin


def extract(X, labels, C, mode, cal_select=0):
    X = np.ascontiguousarray(X, dtype=np.float64)
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    C = np.ascontiguousarray(C, dtype=np.float64).copy()
    n, m = X.shape
    k = C.shape[0]
    counts = np.zeros(k, np.int32)
    sc = lib().or_extract(_d(X), _i(labels), _d(C), n, m, k, mode, cal_select, _i(counts))
    return C, counts, sc


def top_eig(A):
    A = np.ascontiguousarray(A, dtype=np.float64)
    v = np.zeros(A.shape[0])
    lam = lib().or_top_eig_jacobi(_d(A), A.shape[0], _d(v))
    return lam, v


def random_select(n, k, seed):
    out = np.zeros(k, np.int32)
    lib().or_random_select(n, k, seed, _i(out))
    return out


def k_from_labels(labels):
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    return lib().or_k_from_labels(_i(labels), labels.shape[0])


def ari(a, b):
    a = np.ascontiguousarray(a, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.int32)
    return lib().or_ari(_i(a), _i(b), a.shape[0])


def kshape(data, k, mode, init_labels, init_chose=0, seed=0, max_iter=10, restart=True):
    """Run the whole loop.  data: n x m raw values (float32 as parsed)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, m = data.shape
    init = np.ascontiguousarray(init_labels, dtype=np.int32)
    labels = np.zeros(n, np.int32)
    cents = np.zeros((k, m))
    job = OrJob(data.ctypes.data_as(_fp), n, m, k, mode, init_chose, _i(init), seed, max_iter, int(restart))
    res = OrResult(_i(labels), _d(cents), 0, 0, 0, 0.0, 0.0)
    rc = lib().or_kshape(ctypes.byref(job), ctypes.byref(res))
    if rc != 0:
        raise ValueError("oracle kshape rejected the job")
    return dict(labels=labels, centroids=cents, iterations=res.iterations, sum_class=res.sum_class,
                restarted=res.restarted, inertia=res.inertia, min_margin=res.min_margin)


def generate(n, m, classes, noise=0.2, dirichlet=0.0, seed=0):
    """The engine's synthetic series (n x m float32) and class labels, made by the
    oracle library from the same generator source, without the engine's library."""
    data = np.empty((n, m), np.float32)
    labels = np.empty(n, np.int32)
    if lib().or_generate(n, m, classes, noise, dirichlet, seed, data.ctypes.data_as(_fp), _i(labels)) != 0:
        raise ValueError("generate: invalid parameters")
    return data, labels
