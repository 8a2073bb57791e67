"""Python binding of the kg_b200 C ABI (include/kg_b200.h) over ctypes.

The library is the in-tree build/libkg_b200.so of this package; there is no
fallback: if it is missing or no sm_103 GPU is present, calls raise.
Device memory is plain pointers (e.g. ``torch.Tensor.data_ptr()``).
"""
import ctypes
import os
import subprocess

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_DIR = os.path.dirname(PKG_DIR)
# KG_B200_LIB selects another build of the same library (e.g. one compiled
# with different engine options); the default is the in-tree build.
LIB_PATH = os.environ.get("KG_B200_LIB") or os.path.join(PKG_DIR, "build", "libkg_b200.so")
HEADER = os.path.join(REPO_DIR, "include", "kg_b200.h")

STENCILS = ["laplacian", "divergence", "gradient", "uxx1", "wave13pt", "tricubic",
            "tricubic2", "jacobi", "lapgsrb", "gaussblur", "gameoflife"]
STENCIL_ID = {s: i for i, s in enumerate(STENCILS)}
IS2D = {"jacobi", "gaussblur", "gameoflife"}

KG_F64, KG_F64_FMA, KG_F32, KG_BF16, KG_F16, KG_U8, KG_F64_FF, KG_F64_MIX = range(8)
DTYPES = {"f64": KG_F64, "f64fma": KG_F64_FMA, "f32": KG_F32, "bf16": KG_BF16,
          "f16": KG_F16, "u8": KG_U8, "f64ff": KG_F64_FF, "f64mix": KG_F64_MIX}
DTYPE_SIZE = {KG_F64: 8, KG_F64_FMA: 8, KG_F32: 4, KG_BF16: 2, KG_F16: 2, KG_U8: 1, KG_F64_FF: 8, KG_F64_MIX: 8}
STATUS = ["KG_OK", "KG_EINVAL", "KG_ECUDA", "KG_ENOMEM", "KG_ETIMEOUT", "KG_ENOTSUP", "KG_ENODEV"]

# Every extern "C" symbol the header declares (checked by the CPU tests).
EXPORTS = [
    "kg_laplacian", "kg_divergence", "kg_gradient", "kg_uxx1", "kg_wave13pt", "kg_tricubic",
    "kg_tricubic2", "kg_jacobi", "kg_lapgsrb", "kg_gaussblur", "kg_gameoflife",
    "kg_stencil_narrays", "kg_stencil_ncoefs", "kg_stencil_is2d", "kg_stencil_outputs",
    "kg_sweep", "kg_checksum", "kg_error_stats", "kg_convert", "kg_program_run",
    "kg_plan_create", "kg_plan_launch", "kg_plan_final_roles", "kg_plan_destroy",
    "kg_kernel_regcount", "kg_sweep_launches", "kg_status_string", "kg_last_error",
    "kg_device_check", "kg_version", "kg_measure_peaks", "kg_checksum_noalloc",
    "kg_batch_create", "kg_batch_step", "kg_batch_capture", "kg_batch_launch", "kg_batch_tune",
    "kg_batch_set_config", "kg_batch_get_config", "kg_batch_set_step", "kg_batch_final_roles",
    "kg_batch_destroy", "kg_poisson_solve", "kg_engine_status",
    "kg_vecadd", "kg_matvec", "kg_matmul", "kg_matmul_tc", "kg_sincos", "kg_whispering", "kg_extra_regcount",
    "kg_plan_kernels", "kg_exact_arith", "kg_set_tma_wait_limit",
]
EXTRA_TESTS = ["vecadd", "matvec", "matmul", "sincos", "whispering"]
KG_ENGINE_AUTO, KG_ENGINE_DIRECT, KG_ENGINE_STAGED, KG_ENGINE_TMA, KG_ENGINE_TMA_VEC = 0, 1, 2, 3, 4
KG_ARITH_ADD, KG_ARITH_MUL, KG_ARITH_DIV, KG_ARITH_NATIVE_ADD, KG_ARITH_NATIVE_MUL, KG_ARITH_NATIVE_DIV = range(6)
ENGINES = {"auto": KG_ENGINE_AUTO, "direct": KG_ENGINE_DIRECT, "staged": KG_ENGINE_STAGED, "tma": KG_ENGINE_TMA,
           "tmavec": KG_ENGINE_TMA_VEC}
KG_SOLVE_SOR_F64, KG_SOLVE_IR_SOR_F32, KG_SOLVE_IR_JACOBI_F32 = 0, 1, 2


class KgError(RuntimeError):
    def __init__(self, status, msg):
        self.status = status
        name = STATUS[status] if 0 <= status < len(STATUS) else str(status)
        super().__init__("%s: %s" % (name, msg))


class KgProblem(ctypes.Structure):
    _fields_ = [("stencil", ctypes.c_int32), ("dtype", ctypes.c_int32),
                ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("ns", ctypes.c_int32),
                ("engine", ctypes.c_int32), ("coef", ctypes.c_double * 6),
                ("arr", ctypes.c_void_p * 6)]


class KgPeaks(ctypes.Structure):
    _fields_ = [("fp64_ops", ctypes.c_double), ("fp32_ops", ctypes.c_double),
                ("int32_ops", ctypes.c_double), ("sms", ctypes.c_int), ("reserved", ctypes.c_int)]


class KgBatchConfig(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int), ("bx", ctypes.c_int), ("by", ctypes.c_int), ("kc", ctypes.c_int),
                ("ctas_per_sm", ctypes.c_int), ("tiles", ctypes.c_int), ("nshapes", ctypes.c_int),
                ("temporal", ctypes.c_int), ("staged", ctypes.c_int), ("reserved", ctypes.c_int),
                ("steps_done", ctypes.c_longlong)]


class KgSolveOpts(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("sweeps_per_check", ctypes.c_int), ("omega", ctypes.c_double),
                ("rtol", ctypes.c_double), ("max_sweeps", ctypes.c_longlong)]


class KgSolveReport(ctypes.Structure):
    _fields_ = [("sweeps", ctypes.c_longlong), ("outer", ctypes.c_int), ("nhistory", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("fnorm", ctypes.c_double), ("seconds", ctypes.c_double),
                ("history_sweeps", ctypes.c_longlong * 256), ("history_rel", ctypes.c_double * 256)]


class KgTimings(ctypes.Structure):
    _fields_ = [("alloc", ctypes.c_double), ("load", ctypes.c_double),
                ("compute", ctypes.c_double), ("save", ctypes.c_double),
                ("free_", ctypes.c_double), ("kernel_avg", ctypes.c_double),
                ("kernel_min", ctypes.c_double), ("nregs", ctypes.c_int),
                ("weights_once", ctypes.c_int)]


def build(jobs=8, drivers=True, quiet=True):
    """Compile build/libkg_b200.so (sm_103a) and the b200 target programs."""
    targets = ["all"] + (["drivers"] if drivers else [])
    out = subprocess.run(["make", "-j%d" % jobs, "-C", PKG_DIR] + targets,
                         capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("build of %s failed:\n%s\n%s" % (PKG_DIR, out.stdout, out.stderr))


_lib = None


def _sig(lib):
    P, I, D, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    sig = {
        "kg_laplacian": [I, I, I, I, D, D, P, P, P],
        "kg_divergence": [I, I, I, I, D, D, D, P, P, P, P, P],
        "kg_gradient": [I, I, I, I, D, D, D, P, P, P, P, P],
        "kg_uxx1": [I, I, I, I, D, D, P, P, P, P, P, P, P],
        "kg_wave13pt": [I, I, I, I, D, D, D, P, P, P, P],
        "kg_tricubic": [I, I, I, I, P, P, P, P, P, P],
        "kg_tricubic2": [I, I, I, I, P, P, P, P, P, P],
        "kg_jacobi": [I, I, I, D, D, D, P, P, P],
        "kg_lapgsrb": [I, I, I, I, D, D, D, D, P, P, P],
        "kg_gaussblur": [I, I, I, D, D, D, D, D, D, P, P, P],
        "kg_gameoflife": [I, I, I, P, P, P],
        "kg_sweep": [ctypes.POINTER(KgProblem), P],
        "kg_engine_status": [P],
        "kg_set_tma_wait_limit": [ctypes.c_longlong],
        "kg_vecadd": [I, I, I, I, P, P, P, P],
        "kg_matvec": [I, I, I, P, P, P, P],
        "kg_matmul": [I, I, I, I, P, P, P, P],
        "kg_matmul_tc": [I, I, I, P, P, P, P],
        "kg_sincos": [I, I, I, I, P, P, P, P],
        "kg_whispering": [I, I, I, D, D] + [P] * 9 + [P],
        "kg_extra_regcount": [ctypes.c_char_p, I, ctypes.POINTER(I)],
        "kg_checksum": [I, S, I, ctypes.POINTER(ctypes.c_void_p), P, P],
        "kg_checksum_noalloc": [I, S, I, ctypes.POINTER(ctypes.c_void_p), P, P],
        "kg_error_stats": [I, S, P, P, P, P],
        "kg_convert": [I, P, I, P, S, P],
        "kg_program_run": [ctypes.POINTER(KgProblem), I, I, ctypes.POINTER(KgTimings), P],
        "kg_plan_create": [ctypes.POINTER(P), ctypes.POINTER(KgProblem), I],
        "kg_plan_launch": [P, P],
        "kg_plan_final_roles": [P, ctypes.POINTER(KgProblem)],
        "kg_plan_destroy": [P],
        "kg_plan_kernels": [P],
        "kg_exact_arith": [I, S, P, P, P, P],
        "kg_kernel_regcount": [I, I, ctypes.POINTER(I)],
        "kg_device_check": [],
        "kg_measure_peaks": [ctypes.POINTER(KgPeaks), P],
        "kg_batch_create": [ctypes.POINTER(P), ctypes.POINTER(KgProblem), I],
        "kg_batch_step": [P, I, P],
        "kg_batch_capture": [P, I],
        "kg_batch_launch": [P, P],
        "kg_batch_tune": [P, ctypes.c_char_p, P],
        "kg_batch_set_config": [P, I, I],
        "kg_batch_get_config": [P, ctypes.POINTER(KgBatchConfig)],
        "kg_batch_set_step": [P, ctypes.c_longlong],
        "kg_batch_final_roles": [P, I, ctypes.POINTER(KgProblem)],
        "kg_batch_destroy": [P],
        "kg_poisson_solve": [I, I, I, P, P, ctypes.POINTER(KgSolveOpts), ctypes.POINTER(KgSolveReport), P],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    for name in ("kg_stencil_narrays", "kg_stencil_ncoefs", "kg_stencil_is2d", "kg_stencil_outputs"):
        getattr(lib, name).argtypes = [I]
        getattr(lib, name).restype = I
    lib.kg_sweep_launches.argtypes = [I, I]
    lib.kg_sweep_launches.restype = I
    for name in ("kg_status_string",):
        getattr(lib, name).argtypes = [I]
        getattr(lib, name).restype = ctypes.c_char_p
    lib.kg_last_error.argtypes = []
    lib.kg_last_error.restype = ctypes.c_char_p
    lib.kg_version.argtypes = []
    lib.kg_version.restype = ctypes.c_char_p


def load():
    """Load the in-tree library (no GPU needed to load it)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("%s is missing: run __graft_entry__.build()" % LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        _sig(lib)
        _lib = lib
    return _lib


def check(status):
    if status != 0:
        raise KgError(status, load().kg_last_error().decode())


def stream_ptr(stream):
    """A torch.cuda.Stream (or None for the default stream) as kg_stream_t."""
    if stream is None:
        return None
    return ctypes.c_void_p(stream.cuda_stream)


def problem(stencil, dtype, shape, coef, arrays, engine=KG_ENGINE_AUTO):
    """kg_problem from a stencil name, dtype id, shape, coefficients and device
    pointers; `engine` a KG_ENGINE_* id (or its name)."""
    p = KgProblem()
    p.engine = ENGINES[engine] if isinstance(engine, str) else int(engine)
    p.stencil = STENCIL_ID[stencil] if isinstance(stencil, str) else int(stencil)
    p.dtype = dtype
    if len(shape) == 2:
        p.nx, p.ny, p.ns = shape[0], shape[1], 1
    else:
        p.nx, p.ny, p.ns = shape
    for q, c in enumerate(coef):
        p.coef[q] = c
    for q, a in enumerate(arrays):
        p.arr[q] = a
    return p


def sweep(p, stream=None):
    check(load().kg_sweep(ctypes.byref(p), stream_ptr(stream)))


def extra_step(test, dtype, args, ptrs, coef=(), stream=None):
    """One call of kg_<test> (vecadd, matvec, matmul, sincos, whispering) on
    device pointers; args are the sizes of its command line (without nt)."""
    lib = load()
    st = stream_ptr(stream)
    if test == "vecadd":
        check(lib.kg_vecadd(dtype, *args, *ptrs, st))
    elif test == "sincos":
        check(lib.kg_sincos(dtype, *args, *ptrs, st))
    elif test == "matvec":
        check(lib.kg_matvec(dtype, *args, *ptrs, st))
    elif test == "matmul":
        check(lib.kg_matmul(dtype, *args, *ptrs, st))
    elif test == "whispering":
        check(lib.kg_whispering(dtype, args[0], args[1], coef[0], coef[1], *ptrs, st))
    else:
        raise ValueError(test)


def extra_rotate(test, ptrs):
    """The reference main()'s pointer rotation after one step."""
    p = list(ptrs)
    if test == "vecadd":
        return [p[1], p[2], p[0]]
    if test == "whispering":   # e, h0, h1, u_em0, u_em1, ...
        p[1], p[2] = p[2], p[1]
        p[3], p[4] = p[4], p[3]
    return p


def engine_status(stream=None):
    """kg_engine_status: raises KgError(KG_ETIMEOUT) if a TMA sweep's wait gave up."""
    check(load().kg_engine_status(stream_ptr(stream)))


def checksum(dtype, n, arrays, out_ptr, stream=None):
    arr = (ctypes.c_void_p * len(arrays))(*arrays)
    check(load().kg_checksum(dtype, n, len(arrays), arr, out_ptr, stream_ptr(stream)))


def error_stats(dtype, n, x_ptr, ref_ptr, out_ptr, stream=None):
    check(load().kg_error_stats(dtype, n, x_ptr, ref_ptr, out_ptr, stream_ptr(stream)))


def convert(dst_t, dst, src_t, src, n, stream=None):
    check(load().kg_convert(dst_t, dst, src_t, src, n, stream_ptr(stream)))


def regcount(stencil, dtype):
    r = ctypes.c_int(0)
    check(load().kg_kernel_regcount(STENCIL_ID.get(stencil, stencil), dtype, ctypes.byref(r)))
    return r.value


def rotate(stencil, arrays):
    """The reference's pointer rotation after one sweep."""
    a = list(arrays)
    if stencil in ("divergence", "gradient"):
        return a
    if stencil == "wave13pt":
        return [a[1], a[2], a[0]] + a[3:]
    return [a[1], a[0]] + a[2:]


class Plan:
    """nt sweeps with the reference's rotation, captured as one CUDA graph."""

    def __init__(self, p, nt):
        self.h = ctypes.c_void_p()
        check(load().kg_plan_create(ctypes.byref(self.h), ctypes.byref(p), nt))

    def launch(self, stream=None):
        check(load().kg_plan_launch(self.h, stream_ptr(stream)))

    def final_roles(self):
        p = KgProblem()
        check(load().kg_plan_final_roles(self.h, ctypes.byref(p)))
        return p

    def kernels(self):
        """Kernel launches in one replay."""
        return load().kg_plan_kernels(self.h)

    def close(self):
        if self.h:
            load().kg_plan_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def measure_peaks(stream=None):
    """Measured FP64/FP32/INT32 issue rates of the current device (ops/s)."""
    r = KgPeaks()
    check(load().kg_measure_peaks(ctypes.byref(r), stream_ptr(stream)))
    return r


class Batch:
    """kg_batch: many problems (list of KgProblem, device pointers) stepped together."""

    def __init__(self, problems):
        arr = (KgProblem * len(problems))(*problems)
        self.n = len(problems)
        self.h = ctypes.c_void_p()
        check(load().kg_batch_create(ctypes.byref(self.h), arr, len(problems)))

    def step(self, nsteps=1, stream=None):
        check(load().kg_batch_step(self.h, nsteps, stream_ptr(stream)))

    def capture(self, nsteps):
        check(load().kg_batch_capture(self.h, nsteps))

    def launch(self, stream=None):
        check(load().kg_batch_launch(self.h, stream_ptr(stream)))

    def tune(self, cache_path=None, stream=None):
        check(load().kg_batch_tune(self.h, cache_path.encode() if cache_path else None, stream_ptr(stream)))

    def set_config(self, shape, ctas):
        check(load().kg_batch_set_config(self.h, shape, ctas))

    def config(self):
        c = KgBatchConfig()
        check(load().kg_batch_get_config(self.h, ctypes.byref(c)))
        return c

    def set_step(self, step):
        check(load().kg_batch_set_step(self.h, step))

    def final_roles(self, q):
        p = KgProblem()
        check(load().kg_batch_final_roles(self.h, q, ctypes.byref(p)))
        return p

    def close(self):
        if self.h:
            load().kg_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_solve(shape, f_ptr, u_ptr, kind, omega=1.8, rtol=1e-10, sweeps_per_check=100,
                  max_sweeps=10**7, stream=None, raise_on_timeout=True):
    """kg_poisson_solve; returns (status, KgSolveReport)."""
    o = KgSolveOpts(kind, sweeps_per_check, omega, rtol, max_sweeps)
    r = KgSolveReport()
    nx, ny, ns = shape
    st = load().kg_poisson_solve(nx, ny, ns, f_ptr, u_ptr, ctypes.byref(o), ctypes.byref(r), stream_ptr(stream))
    if st != 0 and (raise_on_timeout or st != 4):
        check(st)
    return st, r


def program_run(p, nt, copy_back_mask, stream=None):
    """kg_program_run on host pointers; returns KgTimings (p.arr permuted in place)."""
    t = KgTimings()
    check(load().kg_program_run(ctypes.byref(p), nt, copy_back_mask, ctypes.byref(t), stream_ptr(stream)))
    return t
