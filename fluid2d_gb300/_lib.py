"""Build and load libfluid2d_gb300.so (the sm_103a kernels behind a C ABI).

Two variants are built from the same sources:

* ``libfluid2d_gb300.so``        -- the product build (nvcc may contract a*b+c
  into FMA);
* ``libfluid2d_gb300_exact.so``  -- ``-DF2D_EXACT -fmad=false``: every
  operation rounded separately, for bit-for-bit comparison with the CPU
  oracle in the parity tests.

There is no CPU fallback: ``lib()`` raises if the library cannot be loaded.
"""
import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

_HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(_HERE, "csrc")
BUILD = os.path.join(_HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(_HERE), "include")
SOURCES = ["api.cu", "kernels_adv.cu", "kernels_ops.cu", "kernels_mg.cu", "engine.cu",
           "kernels_fused.cu", "noalloc.cu", "kernels_mixed.cu", "timeloop.cu", "fluxdiag.cu",
           "kernels_walls.cu", "batch.cu", "peaks.cu"]
HEADERS = ["f2d_common.cuh", "f2d_kernels.cuh", "f2d_fused.cuh", "f2d_adv.cuh", "f2d_mixed.cuh",
           "f2d_loop.cuh", "f2d_flux.cuh", "f2d_walls.cuh",
           "f2d_tri.cuh", "f2d_batch.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-fvisibility=hidden"]
VARIANTS = {
    "product": ("libfluid2d_gb300.so", []),
    "exact": ("libfluid2d_gb300_exact.so", ["-DF2D_EXACT", "-fmad=false"]),
}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _deps():
    files = [os.path.join(CSRC, s) for s in _sources()]
    files += [os.path.join(CSRC, h) for h in HEADERS if os.path.exists(os.path.join(CSRC, h))]
    files.append(os.path.join(INCLUDE, "fluid2d_gb300.h"))
    return files


def so_path(variant="product"):
    return os.path.join(BUILD, VARIANTS[variant][0])


def _stale(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(variants=("product", "exact"), force=False, verbose=False):
    """Compile every variant (all translation units in parallel)."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for var in variants:
        so, extra = VARIANTS[var]
        target = os.path.join(BUILD, so)
        if not force and not _stale(target):
            continue
        objs = []
        for src in _sources():
            obj = os.path.join(BUILD, "%s.%s.o" % (src[:-3], var))
            cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ["-I", INCLUDE, "-c",
                                                        os.path.join(CSRC, src), "-o", obj]
            jobs.append(cmd)
            objs.append(obj)
        jobs.append(("link", target, objs))

    compile_jobs = [j for j in jobs if not isinstance(j, tuple)]
    link_jobs = [j for j in jobs if isinstance(j, tuple)]

    def run(cmd):
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
        return r.stdout

    with ThreadPoolExecutor(max_workers=max(2, min(16, os.cpu_count() or 4))) as ex:
        list(ex.map(run, compile_jobs))
    for _, target, objs in link_jobs:
        tmp = target + ".tmp%d" % os.getpid()
        run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, target)
    return [so_path(v) for v in variants]


_libs = {}
_lock = threading.Lock()


def lib(variant="product"):
    """The loaded library (building it first if it is missing or stale)."""
    with _lock:
        if variant not in _libs:
            path = so_path(variant)
            if _stale(path):
                build(variants=(variant,))
            L = ctypes.CDLL(path)
            _declare(L)
            _libs[variant] = L
        return _libs[variant]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double

# name -> argtypes (all return int status)
SIGNATURES = {
    "f2d_adv_upwind": [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P],
    "f2d_adv_centered": [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P],
    "f2d_flx_adv_upwind": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P],
    "f2d_flx_adv_centered": [_P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P],
    "f2d_computeorthogradient": [_P, _P, _D, _D, _I, _I, _I, _P, _P, _P],
    "f2d_celltocorner": [_P, _P, _I, _I, _P],
    "f2d_cornertocell": [_P, _P, _I, _I, _P],
    "f2d_add_diffusion": [_P, _P, _D, _I, _D, _P, _I, _I, _P],
    "f2d_add_torque": [_P, _P, _D, _I, _D, _P, _I, _I, _P],
    "f2d_computenoslipsourceterm": [_P, _P, _P, _D, _D, _I, _I, _I, _P, _P],
    "f2d_computedotprod": [_P, _P, _P, _I, _I, _I, _P, _P],
    "f2d_computemax": [_P, _P, _I, _I, _I, _P, _P],
    "f2d_computesum": [_P, _P, _I, _I, _I, _P, _P],
    "f2d_computesumandnorm": [_P, _P, _I, _I, _I, _P, _P],
    "f2d_computenormmaxu": [_P, _P, _I, _I, _I, _P, _P],
    "f2d_computekemaxu": [_P, _P, _P, _I, _I, _I, _P, _P],
    "f2d_computekemaxuv": [_P, _P, _P, _I, _I, _I, _P, _P],
    "f2d_computekewithpsi": [_P, _P, _P, _I, _I, _I, _P, _P],
    "f2d_smoothtwicewitha": [_P, _P, _P, _P, _D, _I, _I, _P],
    "f2d_smoothtwicewitha_noalloc": [_P, _P, _P, _P, _D, _I, _I, _P],
    "f2d_computeresidualwitha": [_P, _P, _P, _P, _P, _I, _I, _P],
    "f2d_smoothtridiag": [_P, _P, _P, _P, _I, _I, _P],
    "f2d_fillhalo": [_P, _I, _I, _I, _P],
    "f2d_interpolate": [_P, _P, _P, _I, _I, _I, _I, _I, _P, _P],
    "f2d_restrict": [_P, _P, _I, _I, _I, _I, _I, _P, _P],
    "f2d_coarsenmatrix": [_P, _P, _P, _I, _I, _I, _I, _I, _P, _P],
    "f2d_computenorm": [_P, _P, _I, _I, _I, _P, _P],
    "f2d_computeinner": [_P, _P, _P, _I, _I, _I, _P, _P],
}
_PP = ctypes.POINTER(ctypes.c_void_p)
_PI = ctypes.POINTER(ctypes.c_int)
_PDd = ctypes.POINTER(ctypes.c_double)
_PPD = ctypes.POINTER(ctypes.POINTER(ctypes.c_double))


class ModelDesc(ctypes.Structure):
    """f2d_model_desc of include/fluid2d_gb300.h"""
    _fields_ = [("model", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("perio", ctypes.c_int),
                ("order", ctypes.c_int), ("flux_method", ctypes.c_int),
                ("aparab", ctypes.c_double), ("gravity", ctypes.c_double),
                ("Rd", ctypes.c_double), ("beta", ctypes.c_double),
                ("hydroepsilon", ctypes.c_double), ("adaptable_dt", ctypes.c_int),
                ("dt", ctypes.c_double), ("cfl", ctypes.c_double), ("dtmax", ctypes.c_double),
                ("precision", ctypes.c_int), ("diffusion", ctypes.c_int),
                ("Kdiff", ctypes.c_double * 2)]


class LoopDesc(ctypes.Structure):
    """f2d_loop_desc of include/fluid2d_gb300.h"""
    _fields_ = [("tend", ctypes.c_double), ("freq_his", ctypes.c_double),
                ("freq_diag", ctypes.c_double), ("exacthistime", ctypes.c_int),
                ("rescaledtime", ctypes.c_int), ("nsave", ctypes.c_int),
                ("save", ctypes.c_int * 8), ("his_cap", ctypes.c_int), ("diag_cap", ctypes.c_int),
                ("t", ctypes.c_double), ("tnexthis", ctypes.c_double),
                ("tnextdiag", ctypes.c_double), ("kt", ctypes.c_int),
                ("diag_fluxes", ctypes.c_int)]


class LoopState(ctypes.Structure):
    """f2d_loop_state of include/fluid2d_gb300.h"""
    _fields_ = [("t", ctypes.c_double), ("dt", ctypes.c_double), ("tnexthis", ctypes.c_double),
                ("tnextdiag", ctypes.c_double), ("kt", ctypes.c_int), ("status", ctypes.c_int),
                ("nhis", ctypes.c_int), ("ndiag", ctypes.c_int)]


SIGNATURES.update({
    "f2d_gmg_create": [_P, _I, _I, _D, _D, _D, _I, _D, _PP],
    "f2d_gmg_destroy": [_P],
    "f2d_gmg_levels": [_P, _PI, _PI, _PI, _PI],
    "f2d_gmg_twovcycle": [_P, _P, _P, _P],
    "f2d_gmg_solve": [_P, _P, _P, _I, _D, _P],
    "f2d_gmg_solve_stats": [_P, _PI, _PDd, _PI],
    "f2d_gmg_vcycle": [_P, _I, _P],
    "f2d_gmg_fcycle": [_P, _I, _P],
    "f2d_model_create": [ctypes.POINTER(ModelDesc), _P, _PP],
    "f2d_model_destroy": [_P],
    "f2d_model_info": [_P, _PI, _PI, _PI, _PI, _PI, _PPD, _PPD],
    "f2d_model_set_psi": [_P, _P],
    "f2d_model_diagnostics": [_P, _P],
    "f2d_model_step": [_P, _I, _P],
    "f2d_model_step_graph": [_P, _I, _P],
    "f2d_model_step_host": [_P, _I, ctypes.c_void_p, ctypes.c_void_p],
    "f2d_model_set_dt": [_P, _D],
    "f2d_model_solve_stats": [_P, _PI, _PDd, _PI],
    "f2d_model_status": [_P, _I, _PI, _P],
    "f2d_models_status": [ctypes.POINTER(ctypes.c_void_p), _I, _I, _PI, _P],
    "f2d_model_probe": [_P, _I, _PI, _PDd],
    "f2d_model_bytes": [_P, ctypes.POINTER(ctypes.c_size_t)],
    "f2d_model_graph_kernels": [_P, _PI],
    "f2d_model_coarse_level": [_P, _I, _PI, _PI, _PI],
    "f2d_model_coarse_op": [_P, _I, _PI],
    "f2d_model_cluster_level": [_P, _PI],
    "f2d_model_reset_graphs": [_P],
    "f2d_batch_create": [ctypes.POINTER(ctypes.c_void_p), _I, _I, _PP],
    "f2d_batch_step": [_P, _I, _P],
    "f2d_batch_info": [_P, _PI, _PI],
    "f2d_batch_destroy": [_P],
    "f2d_model_noslip": [_P, _P, _P],
    "f2d_model_islands": [_P, _P, _P, _P],
    "f2d_model_flux_setup": [_P, _P],
    "f2d_model_diag_fluxes": [_P, _P],
    "f2d_model_flux_info": [_P, _PI, _PPD],
    "f2d_model_loop_setup": [_P, ctypes.POINTER(LoopDesc), _P],
    "f2d_model_loop_start": [_P, _P],
    "f2d_model_loop_run": [_P, _I, _P],
    "f2d_model_loop_state": [_P, ctypes.POINTER(LoopState), _P],
    "f2d_model_loop_drain": [_P, _P, _P, _P, _P, _P, _PI, _PI, _P],
})

EXTRA = {
    "f2d_gmg_level_ptr": ([_P, _I, ctypes.c_char_p], _P),
    "f2d_model_varname": ([_P, _I], ctypes.c_char_p),
    "f2d_model_diagname": ([_P, _I], ctypes.c_char_p),
    "f2d_model_buffer": ([_P, ctypes.c_char_p], _P),
    "f2d_model_flux_name": ([_P, _I], ctypes.c_char_p),
    "f2d_version": ([], _I),
    "f2d_set_pdl": ([_I], _I),
    "f2d_set_level_tiles": ([_I], _I),
    "f2d_set_level_threads": ([_I], _I),
    "f2d_set_separable": ([_I], _I),
    "f2d_set_cluster": ([_I], _I),
    "f2d_set_l2_persist": ([_I], _I),
    "f2d_fp64_peak": ([ctypes.POINTER(ctypes.c_double)], _I),
    "f2d_last_error": ([], ctypes.c_char_p),
    "f2d_exact_arithmetic": ([], _I),
}


def _declare(L):
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _I
    for name, (args, res) in EXTRA.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    try:
        from . import _abi_ext
        _abi_ext.declare(L)
    except ImportError:
        pass


class F2DError(RuntimeError):
    """A nonzero status returned by the library (message from f2d_last_error)."""

    def __init__(self, name, code, msg):
        RuntimeError.__init__(self, "%s failed (status %d): %s" % (name, code, msg))
        self.code = code


def call(name, *args, variant="product"):
    L = lib(variant)
    rc = getattr(L, name)(*args)
    if rc != 0:
        raise F2DError(name, rc, L.f2d_last_error().decode(errors="replace"))
    return rc
