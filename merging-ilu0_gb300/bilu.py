"""Python binding of the bilu C ABI (include/bilu.h) over ctypes.

Device memory is passed as torch CUDA tensors (any object with .data_ptr()
works); host arrays as numpy.  The library must have been built
(merging-ilu0_gb300/bilu_build.py); importing this module without it raises.
The binding adds no computation of its own: every operation is a call into
libbilu.so.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libbilu.so")

# ---------------------------------------------------------------- constants
OK = 0
ERR_INVALID, ERR_PATTERN, ERR_CAPACITY, ERR_CUDA, ERR_NO_DEVICE, ERR_ALLOC = 1, 2, 3, 4, 5, 6

SYS_CONVERGED, SYS_MAX_ITER, SYS_BREAKDOWN_RHO, SYS_NONFINITE, SYS_ZERO_RHS, SYS_INITIAL_OK = 1, -1, -2, -3, 2, 3

(PRECOND_ILU0, PRECOND_ILU0_SPLIT, PRECOND_PARILU0, PRECOND_ILU0_ISAI, PRECOND_PARILU0_ISAI, PRECOND_NONE,
 PRECOND_GENERAL_ISAI) = range(7)
TOL_ABS, TOL_REL = 0, 1
FP64, FP32 = 0, 1
REDUCE_REF, REDUCE_FAST = 0, 1

EXPORTED = [
    "bilu_default_options", "bilu_plan_create", "bilu_plan_destroy", "bilu_plan_get_info",
    "bilu_plan_get_pattern", "bilu_expand_values", "bilu_solve", "bilu_solve_warm", "bilu_ilu0",
    "bilu_parilu0", "bilu_split_lu", "bilu_isai", "bilu_true_residual", "bilu_last_error",
    "bilu_version", "bilu_device_count", "bilu_gen_stencil", "bilu_gen_stencil_range", "bilu_gen_uneven",
    "bilu_plan_enable_timing",
    "bilu_plan_last_timing", "bilu_plan_autotune", "bilu_solve_noalloc", "bilu_uneven_plan_create", "bilu_uneven_plan_destroy",
    "bilu_uneven_autotune", "bilu_uneven_solve", "bilu_uneven_get_info", "bilu_uneven_set_config", "bilu_forward_error",
    "bilu_mlp_create", "bilu_mlp_destroy", "bilu_mlp_param_count", "bilu_mlp_get_params", "bilu_mlp_set_params",
    "bilu_mlp_train", "bilu_mlp_loss_grad", "bilu_mlp_eval", "bilu_mlp_warm_start", "bilu_mlp_save", "bilu_mlp_load",
    "bilu_probe_fp64_rate",
    "bilu_check_integer_fp",
]


class Options(C.Structure):
    _fields_ = [
        ("precond", C.c_int), ("ilu_approach", C.c_int), ("parilu_sweeps", C.c_int), ("isai_power", C.c_int),
        ("tol_mode", C.c_int), ("tol", C.c_double), ("max_iter", C.c_int), ("factor_precision", C.c_int),
        ("reduction", C.c_int), ("compute_true_residual", C.c_int), ("threads_per_system", C.c_int),
        ("parilu_res_tol", C.c_double),
        ("isai_lower_diag", C.c_int),
        ("smem_staging", C.c_int),
    ]


class Results(C.Structure):
    _fields_ = [("iter_counts", C.c_void_p), ("conv_flags", C.c_void_p), ("iter_res_norms", C.c_void_p),
                ("true_res_norms", C.c_void_p), ("status", C.c_void_p), ("parilu_sweeps", C.c_void_p),
                ("ilu_residual", C.c_void_p)]


class PlanInfo(C.Structure):
    _fields_ = [(k, C.c_int) for k in (
        "n", "nnz", "nnz_in", "missing_diag", "nnz_L", "nnz_U", "nnz_isai_L", "nnz_isai_U", "levels_lower",
        "levels_upper", "max_row_len", "threads", "smem_bytes", "operands_in_smem", "solver_kernel")]


class Timing(C.Structure):
    _fields_ = [("setup_ms", C.c_float), ("solve_ms", C.c_float), ("total_ms", C.c_float)]


class BiluError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"bilu error {code}: {msg}")
        self.code = code


_lib = None


def lib():
    """The loaded libbilu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBPATH} is missing: run merging-ilu0_gb300/bilu_build.py (or __graft_entry__.build())")
        L = C.CDLL(LIBPATH)
        vp, ip, i, d = C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_double
        L.bilu_last_error.restype = C.c_char_p
        L.bilu_version.restype = C.c_char_p
        L.bilu_device_count.restype = i
        L.bilu_default_options.argtypes = [C.POINTER(Options)]
        L.bilu_plan_create.argtypes = [C.POINTER(vp), i, i, ip, ip, C.POINTER(Options)]
        L.bilu_plan_destroy.argtypes = [vp]
        L.bilu_plan_get_info.argtypes = [vp, C.POINTER(PlanInfo)]
        L.bilu_plan_get_pattern.argtypes = [vp, i, ip, ip, ip, ip]
        L.bilu_expand_values.argtypes = [vp, i, vp, vp, vp]
        L.bilu_solve.argtypes = [vp, i, vp, vp, vp, C.POINTER(Results), vp]
        L.bilu_solve_warm.argtypes = [vp, i, vp, vp, vp, vp, C.POINTER(Results), vp]
        L.bilu_ilu0.argtypes = [vp, i, vp, vp, i, vp]
        L.bilu_parilu0.argtypes = [vp, i, vp, vp, vp, i, vp]
        L.bilu_split_lu.argtypes = [vp, i, vp, vp, vp, vp]
        L.bilu_isai.argtypes = [vp, i, vp, vp, vp, vp]
        L.bilu_true_residual.argtypes = [vp, i, vp, vp, vp, vp, vp]
        L.bilu_solve_noalloc.argtypes = [vp, i, vp, vp, vp, C.POINTER(Results), vp]
        L.bilu_uneven_plan_create.argtypes = [C.POINTER(vp), i, ip, ip, ip, ip, C.POINTER(Options)]
        L.bilu_uneven_plan_destroy.argtypes = [vp]
        L.bilu_uneven_autotune.argtypes = [vp, vp, vp, vp, vp]
        L.bilu_uneven_solve.argtypes = [vp, vp, vp, vp, C.POINTER(Results), vp]
        L.bilu_uneven_get_info.argtypes = [vp, i, ip, ip, ip, ip, ip, ip, C.POINTER(C.c_float)]
        L.bilu_uneven_set_config.argtypes = [vp, i, i, i]
        L.bilu_forward_error.argtypes = [vp, i, ip, vp, vp, vp, C.POINTER(d), vp, vp]
        fp = C.POINTER(C.c_float)
        L.bilu_mlp_create.argtypes = [C.POINTER(vp), C.c_uint64]
        L.bilu_mlp_destroy.argtypes = [vp]
        L.bilu_mlp_param_count.restype = i
        L.bilu_mlp_get_params.argtypes = [vp, fp]
        L.bilu_mlp_set_params.argtypes = [vp, fp]
        L.bilu_mlp_train.argtypes = [vp, vp, i, vp, vp, i, i, C.c_float, C.c_uint64, fp, vp]
        L.bilu_mlp_loss_grad.argtypes = [vp, vp, i, vp, vp, i, ip, fp, fp, vp]
        L.bilu_mlp_eval.argtypes = [vp, vp, i, vp, i, ip, fp, fp, C.POINTER(d), vp]
        L.bilu_mlp_warm_start.argtypes = [vp, vp, i, vp, vp, d, vp, vp, vp]
        L.bilu_mlp_save.argtypes = [vp, C.c_char_p]
        L.bilu_mlp_load.argtypes = [vp, C.c_char_p]
        L.bilu_probe_fp64_rate.argtypes = [C.POINTER(d), C.POINTER(d), vp]
        L.bilu_check_integer_fp.argtypes = [i, C.c_uint64, C.POINTER(C.c_ulonglong), vp]
        L.bilu_plan_enable_timing.argtypes = [vp, i]
        L.bilu_plan_last_timing.argtypes = [vp, C.POINTER(Timing)]
        L.bilu_gen_uneven.argtypes = [i, C.c_uint64, i, i, i, i, ip, ip, ip, ip, C.POINTER(d), C.POINTER(d)]
        L.bilu_gen_stencil.argtypes = [i, i, i, i, i, C.c_uint64, ip, ip, ip, ip, C.POINTER(d), C.POINTER(d)]
        L.bilu_gen_stencil_range.argtypes = [i, i, i, i, C.c_longlong, i, C.c_uint64, ip, ip, ip, ip, C.POINTER(d),
                                             C.POINTER(d)]
        _lib = L
    return _lib


def _check(code):
    if code != OK:
        raise BiluError(code, lib().bilu_last_error().decode())


def _iptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


def _dptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _dev(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(s):
    if s is None:
        return None
    return C.c_void_p(s.cuda_stream if hasattr(s, "cuda_stream") else int(s))


def default_options(**kw):
    o = Options()
    lib().bilu_default_options(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def device_count():
    return lib().bilu_device_count()


def version():
    return lib().bilu_version().decode()


def probe_fp64_rate(stream=None):
    """(FP64 FMA throughput of the current device in GFLOP/s, SM clock during the measurement in MHz);
    bilu_probe_fp64_rate."""
    g, m = C.c_double(), C.c_double()
    _check(lib().bilu_probe_fp64_rate(C.byref(g), C.byref(m), _stream(stream)))
    return g.value, m.value


def check_integer_fp(n_per_thread=1024, seed=1, stream=None):
    """(roundings, widenings, reciprocals) of the kernels' integer FP64 operations that differ from the
    hardware's on n_per_thread bit patterns per thread; bilu_check_integer_fp."""
    out = (C.c_ulonglong * 3)()
    _check(lib().bilu_check_integer_fp(n_per_thread, seed, out, _stream(stream)))
    return int(out[0]), int(out[1]), int(out[2])


# ---------------------------------------------------------------- generators
def gen_stencil(kind, gx, gy, gz, nsys, seed=20261203, first=0):
    """Seeded batch of a stencil workload: returns (row_ptrs, col_idxs, values[nsys, nnz], b[nsys, n]).
    first > 0: systems first .. first+nsys-1 of the same seeded stream (a rank's slab of a global batch)."""
    n, nnz = C.c_int(), C.c_int()
    _check(lib().bilu_gen_stencil(kind, gx, gy, gz, 0, seed, C.byref(n), C.byref(nnz), None, None, None, None))
    rp = np.zeros(n.value + 1, np.int32)
    ci = np.zeros(nnz.value, np.int32)
    vals = np.zeros((nsys, nnz.value), np.float64)
    b = np.zeros((nsys, n.value), np.float64)
    _check(lib().bilu_gen_stencil_range(kind, gx, gy, gz, int(first), nsys, seed, C.byref(n), C.byref(nnz),
                                        _iptr(rp), _iptr(ci), _dptr(vals), _dptr(b)))
    return rp, ci, vals, b


def gen_uneven(nsys, seed=20261203, nmin=64, nmax=1024, kmin=5, kmax=12):
    """Seeded uneven batch: returns (sys_n, sys_nnz, row_ptrs, col_idxs, values, b), systems back to back."""
    sn = np.zeros(nsys, np.int32)
    sz = np.zeros(nsys, np.int32)
    _check(lib().bilu_gen_uneven(nsys, seed, nmin, nmax, kmin, kmax, _iptr(sn), _iptr(sz), None, None, None, None))
    rp = np.zeros(int(sn.sum()) + nsys, np.int32)
    ci = np.zeros(int(sz.sum()), np.int32)
    v = np.zeros(int(sz.sum()))
    b = np.zeros(int(sn.sum()))
    _check(lib().bilu_gen_uneven(nsys, seed, nmin, nmax, kmin, kmax, _iptr(sn), _iptr(sz), _iptr(rp), _iptr(ci),
                                 _dptr(v), _dptr(b)))
    return sn, sz, rp, ci, v, b


class UnevenPlan:
    """bilu_uneven_plan: systems with their own sizes and patterns in one graph-launched solve."""

    def __init__(self, sys_n, sys_nnz, row_ptrs, col_idxs, options=None, **kw):
        self.sys_n = np.ascontiguousarray(sys_n, np.int32)
        self.sys_nnz = np.ascontiguousarray(sys_nnz, np.int32)
        self.row_ptrs = np.ascontiguousarray(row_ptrs, np.int32)
        self.col_idxs = np.ascontiguousarray(col_idxs, np.int32)
        self.options = options if options is not None else default_options(**kw)
        self.nsys = len(self.sys_n)
        h = C.c_void_p()
        _check(lib().bilu_uneven_plan_create(C.byref(h), self.nsys, _iptr(self.sys_n), _iptr(self.sys_nnz),
                                             _iptr(self.row_ptrs), _iptr(self.col_idxs), C.byref(self.options)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().bilu_uneven_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def autotune(self, values, b, x, stream=None):
        _check(lib().bilu_uneven_autotune(self.h, _dev(values), _dev(b), _dev(x), _stream(stream)))

    def solve(self, values, b, x, iters=None, conv=None, res=None, true_res=None, status=None, stream=None):
        R = Results(*(C.c_void_p(t.data_ptr()) if t is not None else None
                      for t in (iters, conv, res, true_res, status)))
        _check(lib().bilu_uneven_solve(self.h, _dev(values), _dev(b), _dev(x), C.byref(R), _stream(stream)))

    def set_config(self, bucket, threads=0, grid=0):
        """Pins a bucket's CTA size and grid (bilu_uneven_set_config; grid below the bucket's systems: persistent
        CTAs over its work queue)."""
        _check(lib().bilu_uneven_set_config(self.h, bucket, threads, grid))

    def info(self):
        """Per size bucket: n range, systems, CTA size, grid, shared memory, autotuned time."""
        out = []
        while True:
            v = [C.c_int() for _ in range(6)]
            t = C.c_float()
            rc = lib().bilu_uneven_get_info(self.h, len(out), *[C.byref(q) for q in v], C.byref(t))
            if rc == ERR_INVALID and out:
                return out  # past the last bucket
            _check(rc)
            out.append(dict(n_lo=v[0].value, n_hi=v[1].value, systems=v[2].value, threads=v[3].value,
                            grid=v[4].value, smem_bytes=v[5].value, tuned_ms=t.value))


# ---------------------------------------------------------------- plans
class Plan:
    """A pattern plan (bilu_plan_create); use as a context manager or call close()."""

    def __init__(self, row_ptrs, col_idxs, options=None, **kw):
        self.row_ptrs = np.ascontiguousarray(row_ptrs, np.int32)
        self.col_idxs = np.ascontiguousarray(col_idxs, np.int32)
        self.options = options if options is not None else default_options(**kw)
        self.n = len(self.row_ptrs) - 1
        self.nnz_in = len(self.col_idxs)
        h = C.c_void_p()
        _check(lib().bilu_plan_create(C.byref(h), self.n, self.nnz_in, _iptr(self.row_ptrs), _iptr(self.col_idxs),
                                      C.byref(self.options)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().bilu_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        i = PlanInfo()
        _check(lib().bilu_plan_get_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in PlanInfo._fields_}

    def pattern(self, which):
        n, nnz = C.c_int(), C.c_int()
        _check(lib().bilu_plan_get_pattern(self.h, which, C.byref(n), C.byref(nnz), None, None))
        rp = np.zeros(n.value + 1, np.int32)
        ci = np.zeros(max(nnz.value, 1), np.int32)
        _check(lib().bilu_plan_get_pattern(self.h, which, C.byref(n), C.byref(nnz), _iptr(rp), _iptr(ci)))
        return rp, ci[: nnz.value]

    def solve(self, values, b, x, iters=None, conv=None, res=None, true_res=None, status=None, stream=None,
              lu_init=None, sweeps=None, ilu_res=None):
        """All arguments are CUDA tensors (values nsys*nnz_in f64, b/x nsys*n f64, iters f32, conv/status i32,
        res/true_res f64, sweeps i32, ilu_res f64); returns immediately (stream ordered)."""
        nsys = b.shape[0] if b.dim() > 1 else b.numel() // self.n
        R = Results(*(C.c_void_p(t.data_ptr()) if t is not None else None
                      for t in (iters, conv, res, true_res, status, sweeps, ilu_res)))
        if lu_init is None:
            _check(lib().bilu_solve(self.h, nsys, _dev(values), _dev(b), _dev(x), C.byref(R), _stream(stream)))
        else:
            _check(lib().bilu_solve_warm(self.h, nsys, _dev(values), _dev(lu_init), _dev(b), _dev(x), C.byref(R),
                                         _stream(stream)))

    def solve_noalloc(self, values, b, x, iters=None, conv=None, res=None, true_res=None, status=None,
                      stream=None):
        """bilu_solve_noalloc: same results as solve(), scratch in the library's fixed device array."""
        nsys = b.shape[0] if b.dim() > 1 else b.numel() // self.n
        R = Results(*(C.c_void_p(t.data_ptr()) if t is not None else None
                      for t in (iters, conv, res, true_res, status)))
        _check(lib().bilu_solve_noalloc(self.h, nsys, _dev(values), _dev(b), _dev(x), C.byref(R),
                                        _stream(stream)))

    def enable_timing(self, enable=True):
        _check(lib().bilu_plan_enable_timing(self.h, 1 if enable else 0))

    def autotune(self, values, b, x, stream=None):
        """Keeps the fastest register-resident solver configuration for this batch (x is overwritten)."""
        nsys = b.shape[0] if b.dim() > 1 else b.numel() // self.n
        _check(lib().bilu_plan_autotune(self.h, nsys, _dev(values), _dev(b), _dev(x), _stream(stream)))
        return self.info()

    def last_timing(self):
        t = Timing()
        _check(lib().bilu_plan_last_timing(self.h, C.byref(t)))
        return {"setup_ms": t.setup_ms, "solve_ms": t.solve_ms, "total_ms": t.total_ms}

    def ilu0(self, values, lu, approach=1, stream=None):
        nsys = values.shape[0]
        _check(lib().bilu_ilu0(self.h, nsys, _dev(values), _dev(lu), approach, _stream(stream)))

    def parilu0(self, values, lu, sweeps, init=None, stream=None):  # noqa: D401
        nsys = values.shape[0]
        _check(lib().bilu_parilu0(self.h, nsys, _dev(values), _dev(init), _dev(lu), sweeps, _stream(stream)))

    def split_lu(self, lu, L, U, stream=None):
        _check(lib().bilu_split_lu(self.h, lu.shape[0], _dev(lu), _dev(L), _dev(U), _stream(stream)))

    def isai(self, lu, ail, aiu, stream=None):
        _check(lib().bilu_isai(self.h, lu.shape[0], _dev(lu), _dev(ail), _dev(aiu), _stream(stream)))

    def true_residual(self, values, b, x, out, stream=None):
        _check(lib().bilu_true_residual(self.h, b.shape[0], _dev(values), _dev(b), _dev(x), _dev(out),
                                        _stream(stream)))

    def forward_error(self, values, b, x, sys_ids, x_dense=None, stream=None):
        """||x_s - x_dense||_2 / ||x_dense||_2 for the sampled systems (FP64 dense LU on the GPU)."""
        ids = np.ascontiguousarray(sys_ids, np.int32)
        out = np.zeros(len(ids))
        _check(lib().bilu_forward_error(self.h, len(ids), _iptr(ids), _dev(values), _dev(b), _dev(x), _dptr(out),
                                        _dev(x_dense), _stream(stream)))
        return out

    def expand_values(self, vin, vout, stream=None):
        _check(lib().bilu_expand_values(self.h, vin.shape[0], _dev(vin), _dev(vout), _stream(stream)))


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


class Mlp:
    """The learned ParILU warm start (bilu_mlp_*)."""

    def __init__(self, seed=1):
        h = C.c_void_p()
        _check(lib().bilu_mlp_create(C.byref(h), seed))
        self.h = h
        self.nparams = lib().bilu_mlp_param_count()

    def close(self):
        if getattr(self, "h", None):
            lib().bilu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def params(self):
        p = np.zeros(self.nparams, np.float32)
        _check(lib().bilu_mlp_get_params(self.h, _fptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _check(lib().bilu_mlp_set_params(self.h, _fptr(p)))

    def train(self, plan, values, lu_target, steps, batch, lr, seed=0, stream=None):
        losses = np.zeros(max(steps, 1), np.float32)
        _check(lib().bilu_mlp_train(self.h, plan.h, values.shape[0], _dev(values), _dev(lu_target), steps, batch,
                                    C.c_float(lr), seed, _fptr(losses), _stream(stream)))
        return losses[:steps]

    def loss_grad(self, plan, values, lu_target, idx, stream=None):
        idx = np.ascontiguousarray(idx, np.int32)
        loss = np.zeros(1, np.float32)
        grad = np.zeros(self.nparams, np.float32)
        _check(lib().bilu_mlp_loss_grad(self.h, plan.h, values.shape[0], _dev(values), _dev(lu_target), len(idx),
                                        _iptr(idx), _fptr(loss), _fptr(grad), _stream(stream)))
        return float(loss[0]), grad

    def eval(self, plan, values, idx, stream=None):
        idx = np.ascontiguousarray(idx, np.int32)
        feat = np.zeros((len(idx), 9), np.float32)
        out = np.zeros(len(idx), np.float32)
        base = np.zeros(len(idx))
        _check(lib().bilu_mlp_eval(self.h, plan.h, values.shape[0], _dev(values), len(idx), _iptr(idx), _fptr(feat),
                                   _fptr(out), _dptr(base), _stream(stream)))
        return feat, out, base

    def warm_start(self, plan, values, lu0, threshold=1e-3, ilu_res=None, used=None, stream=None):
        _check(lib().bilu_mlp_warm_start(self.h, plan.h, values.shape[0], _dev(values), _dev(lu0),
                                         C.c_double(threshold), _dev(ilu_res), _dev(used), _stream(stream)))

    def save(self, path):
        _check(lib().bilu_mlp_save(self.h, path.encode()))

    def load(self, path):
        _check(lib().bilu_mlp_load(self.h, path.encode()))

