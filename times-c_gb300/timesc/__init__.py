"""Python binding of the GB300 k-Shape engine's C ABI (include/timesc.h).

The compute path is libtimesc.so (hand-written sm_103a kernels); this module
only marshals pointers.  Device buffers are torch CUDA tensors (torch is used
for device memory and streams).  There is no CPU fallback: if the library is
missing, importing a compute entry point raises.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libtimesc.so")
CLI_PATH = os.path.join(PKG, "bin", "test")

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_IO, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_REJECTED = range(8)
MODE_COMPAT, MODE_CANONICAL = 0, 1
PREC_FP32, PREC_BF16, PREC_TF32 = 0, 1, 2

_i64, _int, _u32 = ctypes.c_int64, ctypes.c_int, ctypes.c_uint32
_vp = ctypes.c_void_p
_fp = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)


class TimescError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("timesc error %d: %s" % (code, msg))
        self.code = code


class Job(ctypes.Structure):
    _fields_ = [("h_data", _vp), ("d_data", _vp), ("n", _i64), ("m", _int), ("k", _int), ("mode", _int),
                ("precision", _int), ("init_chose", _int), ("seed", _u32), ("max_iter", _int),
                ("restart", _int), ("h_init_labels", _vp)]


class Result(ctypes.Structure):
    _fields_ = [("h_labels", _vp), ("h_centroids", _vp), ("iterations", _int), ("sum_class", _int),
                ("restarted", _int), ("inertia", ctypes.c_double), ("seconds", ctypes.c_double)]


class PoolOpts(ctypes.Structure):
    _fields_ = [("workers", _int), ("hbm_budget_bytes", ctypes.c_uint64)]


class GenSpec(ctypes.Structure):
    _fields_ = [("n", _i64), ("m", _int), ("classes", _int), ("noise", ctypes.c_double),
                ("dirichlet", ctypes.c_double), ("seed", ctypes.c_uint64)]


# exported names and argument types, kept in the order of include/timesc.h
SIGNATURES = {
    "tc_version": (_int, []),
    "tc_create": (_int, [_int, ctypes.POINTER(_vp)]),
    "tc_destroy": (_int, [_vp]),
    "tc_last_error": (ctypes.c_char_p, [_vp]),
    "tc_launch_count": (ctypes.c_uint64, []),
    "tc_fft_size": (_int, [_int, _int]),
    "tc_znorm": (_int, [_vp, _vp, _i64, _int, _int, _vp]),
    "tc_init_labels": (_int, [_vp, _vp, _i64, _int, _vp]),
    "tc_sbd_assign": (_int, [_vp, _vp, _vp, _i64, _int, _int, _int, _int, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "tc_prepare_series": (_int, [_vp, _vp, _i64, _int, _vp]),
    "tc_assign_stats": (_int, [_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                               ctypes.POINTER(ctypes.c_uint64)]),
    "tc_extract_stats": (_int, [_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                ctypes.POINTER(ctypes.c_uint64)]),
    "tc_loop_stats": (_int, [_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(ctypes.c_uint64)]),
    "tc_sbd_assign_noalloc": (_int, [_vp, _vp, _i64, _int, _int, _int, _vp, _vp, _vp, ctypes.c_char_p, _int]),
    "tc_extract_shapes": (_int, [_vp, _vp, _vp, _vp, _vp, _i64, _int, _int, _int, _int, _int, _vp,
                                 ctypes.POINTER(_int), _vp]),
    "tc_kshape_run": (_int, [_vp, ctypes.POINTER(Job), ctypes.POINTER(Result)]),
    "tc_pool_create": (_int, [_int, ctypes.POINTER(PoolOpts), ctypes.POINTER(_vp)]),
    "tc_pool_destroy": (_int, [_vp]),
    "tc_job_footprint": (ctypes.c_uint64, [ctypes.POINTER(Job)]),
    "tc_pool_run_batch": (_int, [_vp, _vp, _int, _vp, _vp]),
    "tc_pool_submit": (_int, [_vp, ctypes.POINTER(Job), ctypes.POINTER(Result), ctypes.POINTER(ctypes.c_uint64)]),
    "tc_pool_wait": (_int, [_vp, ctypes.c_uint64, ctypes.POINTER(_int), ctypes.POINTER(ctypes.c_double),
                            ctypes.POINTER(ctypes.c_double)]),
    "tc_pool_stats": (_int, [_vp, ctypes.POINTER(_int), ctypes.POINTER(_int), ctypes.POINTER(ctypes.c_uint64)]),
    "tc_read_file": (_int, [ctypes.c_char_p, _int, ctypes.POINTER(_fp), ctypes.POINTER(_i32p),
                            ctypes.POINTER(_i64), ctypes.POINTER(_int), ctypes.c_char_p, _int]),
    "tc_free_host": (None, [_vp]),
    "tc_write_labels": (_int, [ctypes.c_char_p, _vp, _i64]),
    "tc_write_centroids": (_int, [ctypes.c_char_p, _vp, _int, _int]),
    "tc_random_select": (_int, [_i64, _int, _u32, _vp]),
    "tc_k_from_labels": (_int, [_vp, _i64]),
    "tc_generate": (_int, [ctypes.POINTER(GenSpec), _vp, _vp]),
}

_lib = None


def lib():
    """Load libtimesc.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libtimesc.so not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(t):
    """Device/host address of a torch tensor or numpy array (None -> NULL)."""
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def _stream(stream):
    if stream is not None:
        return stream
    import torch
    return torch.cuda.current_stream().cuda_stream


def fft_size(m, mode=MODE_COMPAT):
    return lib().tc_fft_size(int(m), int(mode))


class Context:
    """One engine context on one GPU (owns the reusable scratch)."""

    def __init__(self, device=0):
        h = _vp()
        rc = lib().tc_create(int(device), ctypes.byref(h))
        if rc != OK:
            raise TimescError(rc, "tc_create(%d) failed" % device)
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            lib().tc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != OK:
            msg = lib().tc_last_error(self.h)
            raise TimescError(rc, msg.decode() if msg else "")

    # ---- stages (torch CUDA tensors)
    def znorm(self, x, ddof=1, stream=None):
        n, m = x.shape
        self._check(lib().tc_znorm(self.h, _ptr(x), n, m, ddof, _stream(stream)))

    def init_labels(self, labels, k, stream=None):
        self._check(lib().tc_init_labels(self.h, _ptr(labels), labels.shape[0], k, _stream(stream)))

    def sbd_assign(self, x, C, mode=MODE_COMPAT, precision=PREC_FP32, labels=None, dist=None, shift=None,
                   old_labels=None, changed=None, dist_sum=None, stream=None):
        n, m = x.shape
        k = C.shape[0]
        self._check(lib().tc_sbd_assign(self.h, _ptr(x), _ptr(C), n, m, k, mode, precision, _ptr(labels),
                                        _ptr(dist), _ptr(shift), _ptr(old_labels), _ptr(changed),
                                        _ptr(dist_sum), _stream(stream)))

    def assign_stats(self):
        """(screened, bounded, bounded_pairs): assignments that built distance bounds,
        that used them, and the (series, centroid) pairs the bounded ones evaluated."""
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(lib().tc_assign_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def extract_stats(self):
        """(extractions, clusters, reused): extractions that compared their clusters with
        the previous call's, the clusters they covered, and those whose output was
        reused unchanged (synchronises the device)."""
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(lib().tc_extract_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def loop_stats(self):
        """(device_iterations, host_iterations, graphs_built): kshape_run iterations on
        this context that ran inside the loop graph and on the host, and loop graphs built."""
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(lib().tc_loop_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def prepare_series(self, x, stream=None):
        """Keep a BF16 copy of x for TC_PREC_BF16 assignments on the same tensor."""
        n, m = x.shape
        self._check(lib().tc_prepare_series(self.h, _ptr(x), n, m, _stream(stream)))

    def extract_shapes(self, x, labels, C, shift=None, mode=MODE_COMPAT, cal_select=0, precision=PREC_FP32,
                       counts=None, stream=None):
        n, m = x.shape
        k = C.shape[0]
        sc = _int(0)
        self._check(lib().tc_extract_shapes(self.h, _ptr(x), _ptr(labels), _ptr(shift), _ptr(C), n, m, k, mode,
                                            cal_select, precision, _ptr(counts), ctypes.byref(sc),
                                            _stream(stream)))
        return sc.value

    # ---- whole loop (host buffers)
    def kshape_run(self, data, k, mode=MODE_COMPAT, precision=PREC_FP32, init_chose=0, seed=0, max_iter=20,
                   restart=True, init_labels=None, d_data=None):
        if d_data is not None:
            n, m = d_data.shape
        else:
            data = np.ascontiguousarray(data, dtype=np.float32)
            n, m = data.shape
        labels = np.zeros(n, np.int32)
        cents = np.zeros((k, m), np.float32)
        il = None if init_labels is None else np.ascontiguousarray(init_labels, dtype=np.int32)
        job = Job(None if d_data is not None else data.ctypes.data, _ptr(d_data), n, m, k, mode, precision,
                  init_chose, seed, max_iter, int(restart), None if il is None else il.ctypes.data)
        res = Result(labels.ctypes.data, cents.ctypes.data, 0, 0, 0, 0.0, 0.0)
        self._check(lib().tc_kshape_run(self.h, ctypes.byref(job), ctypes.byref(res)))
        return dict(labels=labels, centroids=cents, iterations=res.iterations, sum_class=res.sum_class,
                    restarted=res.restarted, inertia=res.inertia, seconds=res.seconds)


class JobSpec:
    """One job for a Pool: host data (n x m float32) and the tc_kshape_run options.
    Keeps the arrays the C side points at alive until the job is collected."""

    def __init__(self, data, k, mode=MODE_COMPAT, precision=PREC_FP32, init_chose=0, seed=0, max_iter=20,
                 restart=True, init_labels=None):
        self.data = np.ascontiguousarray(data, dtype=np.float32)
        n, m = self.data.shape
        self.k = k
        self.labels = np.zeros(n, np.int32)
        self.centroids = np.zeros((k, m), np.float32)
        self.init = None if init_labels is None else np.ascontiguousarray(init_labels, dtype=np.int32)
        self.job = Job(self.data.ctypes.data, None, n, m, k, mode, precision, init_chose, seed, max_iter,
                       int(restart), None if self.init is None else self.init.ctypes.data)
        self.res = Result(self.labels.ctypes.data, self.centroids.ctypes.data, 0, 0, 0, 0.0, 0.0)

    def footprint(self):
        return int(lib().tc_job_footprint(ctypes.byref(self.job)))

    def result(self):
        r = self.res
        return dict(labels=self.labels, centroids=self.centroids, iterations=r.iterations, sum_class=r.sum_class,
                    restarted=r.restarted, inertia=r.inertia, seconds=r.seconds)


class Pool:
    """Workers (contexts + host threads) running many jobs concurrently on one GPU:
    run_batch for a fixed set, submit/wait for continuous serving."""

    def __init__(self, device=0, workers=8, hbm_budget_bytes=0):
        h = _vp()
        opts = PoolOpts(workers, hbm_budget_bytes)
        rc = lib().tc_pool_create(device, ctypes.byref(opts), ctypes.byref(h))
        if rc != OK:
            raise TimescError(rc, "tc_pool_create failed")
        self.h = h
        self._live = {}

    def close(self):
        if self.h:
            lib().tc_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def run_batch(self, specs):
        """Runs JobSpecs to completion; returns their tc_status codes."""
        n = len(specs)
        jobs = (Job * n)(*[s.job for s in specs])
        results = (Result * n)(*[s.res for s in specs])
        st = (_int * n)()
        lib().tc_pool_run_batch(self.h, jobs, n, results, st)
        for i, s in enumerate(specs):
            s.res = results[i]
        return list(st)

    def submit(self, spec):
        t = ctypes.c_uint64()
        rc = lib().tc_pool_submit(self.h, ctypes.byref(spec.job), ctypes.byref(spec.res), ctypes.byref(t))
        if rc != OK:
            raise TimescError(rc, "job rejected" if rc == ERR_REJECTED else "submit failed")
        self._live[t.value] = spec
        return t.value

    def wait(self, ticket):
        """(status, queued seconds, latency seconds) of a submitted job."""
        st, q, lat = _int(), ctypes.c_double(), ctypes.c_double()
        rc = lib().tc_pool_wait(self.h, ticket, ctypes.byref(st), ctypes.byref(q), ctypes.byref(lat))
        if rc != OK:
            raise TimescError(rc, "unknown ticket")
        self._live.pop(ticket, None)
        return st.value, q.value, lat.value

    def stats(self):
        r, q, b = _int(), _int(), ctypes.c_uint64()
        lib().tc_pool_stats(self.h, ctypes.byref(r), ctypes.byref(q), ctypes.byref(b))
        return dict(running=r.value, queued=q.value, held_bytes=b.value)


def sbd_assign_noalloc(x, C, labels, dist=None, mode=MODE_COMPAT, stream=None):
    """Allocation-free SBD assignment (no context; scratch in a static device
    array).  For callers that must not allocate device memory on the call path."""
    n, m = x.shape
    k = C.shape[0]
    err = ctypes.create_string_buffer(256)
    rc = lib().tc_sbd_assign_noalloc(_ptr(x), _ptr(C), n, m, k, mode, _ptr(labels), _ptr(dist), _stream(stream),
                                     err, 256)
    if rc != OK:
        raise TimescError(rc, err.value.decode())


# ---- host helpers
def read_file(path, labeled):
    d = _fp()
    lab = _i32p()
    n = _i64()
    m = _int()
    err = ctypes.create_string_buffer(512)
    rc = lib().tc_read_file(path.encode(), int(bool(labeled)), ctypes.byref(d),
                            ctypes.byref(lab) if labeled else None, ctypes.byref(n), ctypes.byref(m), err, 512)
    if rc != OK:
        raise TimescError(rc, err.value.decode())
    data = np.ctypeslib.as_array(d, shape=(n.value, m.value)).copy()
    lib().tc_free_host(ctypes.cast(d, _vp))
    labels = None
    if labeled:
        labels = np.ctypeslib.as_array(lab, shape=(n.value,)).copy()
        lib().tc_free_host(ctypes.cast(lab, _vp))
    return data, labels


def write_labels(path, labels):
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    rc = lib().tc_write_labels(path.encode(), labels.ctypes.data, labels.shape[0])
    if rc != OK:
        raise TimescError(rc, "cannot write " + path)


def write_centroids(path, C):
    C = np.ascontiguousarray(C, dtype=np.float32)
    rc = lib().tc_write_centroids(path.encode(), C.ctypes.data, C.shape[0], C.shape[1])
    if rc != OK:
        raise TimescError(rc, "cannot write " + path)


def random_select(n, k, seed):
    out = np.zeros(k, np.int32)
    rc = lib().tc_random_select(n, k, seed, out.ctypes.data)
    if rc != OK:
        raise TimescError(rc, "random_select(%d, %d)" % (n, k))
    return out


def k_from_labels(labels):
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    return lib().tc_k_from_labels(labels.ctypes.data, labels.shape[0])


def generate(n, m, classes, noise=0.2, dirichlet=0.0, seed=0):
    """Synthetic series (n x m float32) and their class labels (0-based)."""
    data = np.empty((n, m), np.float32)
    labels = np.empty(n, np.int32)
    spec = GenSpec(n, m, classes, noise, dirichlet, seed)
    rc = lib().tc_generate(ctypes.byref(spec), data.ctypes.data, labels.ctypes.data)
    if rc != OK:
        raise TimescError(rc, "generate")
    return data, labels
