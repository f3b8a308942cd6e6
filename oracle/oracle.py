"""ctypes view of the C oracle with the f2py calling conventions of Fluid2d.

TEST INFRASTRUCTURE ONLY: the oracle is what the GB300 kernels of
``fluid2d_gb300`` are compared against.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline / reference arm of ``bench.py`` may import this module.

Each function keeps the Python signature that f2py generates for the Fortran
routine it restates (dimension arguments inferred from the arrays, ``intent
(out)`` scalars returned, ``intent(inplace)`` arrays updated in place):

* ``fortran_advection``: ``adv_upwind``, ``adv_centered``
  (core/fortran_advection.f90:2,169)
* ``fortran_fluxes``: ``adv_upwind_flux``, ``adv_centered_flux``
  (core/fortran_fluxes.f90:2,174 -- exported there under the plain names)
* ``fortran_operators``: ``computeorthogradient``, ``celltocorner``,
  ``cornertocell``, ``add_diffusion``, ``add_torque``,
  ``computenoslipsourceterm`` (core/fortran_operators.f90)
* ``fortran_diag``: ``computedotprod``, ``computemax``, ``computesum``,
  ``computesumandnorm``, ``computenormmaxu``, ``computekemaxu``,
  ``computekemaxuv``, ``computekewithpsi`` (core/fortran_diag.f90)
* ``gmg.fortran_multigrid``: ``smoothtwicewitha``, ``smoothoncewitha``,
  ``smoothtridiag``, ``computeresidualwitha``, ``fillhalo``,
  ``interpolate``, ``restrict``, ``coarsenmatrix``, ``computenorm``,
  ``computeinner`` (core/gmg/fortran_multigrid.f90)

An in-place argument that is not a C-contiguous float64/int8 array is copied
into a contiguous buffer for the call and copied back afterwards; f2py's
``intent(inplace)`` has the same visible effect on the array's values.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "f2d_oracle.c")
_BUILD = os.path.join(_HERE, "_build")

# parity: -ffp-contract=off, no fused multiply-add, so every product and sum
# is rounded as the Fortran statement writes it.
CFLAGS = ["-O3", "-ffp-contract=off", "-fPIC", "-shared", "-fno-math-errno"]
# timing (the CPU baseline): what the reference's own build does for speed
# (build.py:13, -O3 -march=native): full optimisation with multiply-adds
# contracted into FMA.  -march=native itself is not used: the host code
# builds the same on the x86-64 and aarch64 machines, and FMA is part of the
# aarch64 base instruction set.
TIMING_CFLAGS = ["-O3", "-ffp-contract=fast", "-funroll-loops", "-fPIC", "-shared",
                 "-fno-math-errno"]
VARIANTS = {"parity": ("liboracle.so", CFLAGS),
            "timing": ("liboracle_timing.so", TIMING_CFLAGS)}
_SO = os.path.join(_BUILD, VARIANTS["parity"][0])


def variant():
    """The build this process loads: 'parity' unless F2D_ORACLE_VARIANT says
    'timing' (set by bench.py's CPU-baseline workers before they load it)."""
    v = os.environ.get("F2D_ORACLE_VARIANT", "parity")
    return v if v in VARIANTS else "parity"


def build(force=False, variants=("parity", "timing")):
    """Compile the oracle shared libraries (gcc, a second or two each)."""
    os.makedirs(_BUILD, exist_ok=True)
    for v in variants:
        so, flags = VARIANTS[v]
        so = os.path.join(_BUILD, so)
        if (not force and os.path.exists(so)
                and os.path.getmtime(so) >= os.path.getmtime(_SRC)):
            continue
        tmp = so + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc"] + flags + ["-o", tmp, _SRC, "-lm"])
        os.replace(tmp, so)
    return _SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        v = variant()
        build(variants=(v,))
        _lib = ctypes.CDLL(os.path.join(_BUILD, VARIANTS[v][0]))
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_PD = ctypes.POINTER(ctypes.c_double)


def _declare(L):
    sig = {
        "adv_upwind": (_I, [_P] * 6 + [_I] * 5),
        "adv_centered": (_I, [_P] * 6 + [_I] * 5),
        "adv_upwind_flux": (_I, [_P] * 8 + [_I] * 5),
        "adv_centered_flux": (_I, [_P] * 8 + [_I] * 5),
        "computeorthogradient": (None, [_P, _P, _D, _D, _I, _I, _I, _P, _P]),
        "celltocorner": (None, [_P, _P, _I, _I]),
        "cornertocell": (None, [_P, _P, _I, _I]),
        "add_diffusion": (None, [_P, _P, _D, _I, _D, _P, _I, _I]),
        "add_torque": (None, [_P, _P, _D, _I, _D, _P, _I, _I]),
        "computenoslipsourceterm": (_D, [_P, _P, _P, _D, _D, _I, _I, _I]),
        "computedotprod": (_D, [_P, _P, _P, _I, _I, _I]),
        "computemax": (_D, [_P, _P, _I, _I, _I]),
        "computesum": (_D, [_P, _P, _I, _I, _I]),
        "computesumandnorm": (None, [_P, _P, _I, _I, _I, _PD, _PD]),
        "computenormmaxu": (None, [_P, _P, _I, _I, _I, _PD, _PD]),
        "computekemaxu": (None, [_P, _P, _P, _I, _I, _I, _PD, _PD]),
        "computekemaxuv": (None, [_P, _P, _P, _I, _I, _I, _PD, _PD, _PD]),
        "computekewithpsi": (_D, [_P, _P, _P, _I, _I, _I]),
        "smoothtwicewitha": (None, [_P, _P, _P, _P, _D, _I, _I, _P]),
        "smoothoncewitha": (None, [_P, _P, _P, _P, _D, _I, _I]),
        "smoothtridiag": (_I, [_P, _P, _P, _P, _I, _I]),
        "computeresidualwitha": (None, [_P, _P, _P, _P, _P, _I, _I]),
        "fillhalo": (None, [_P, _I, _I, _I]),
        "interpolate": (_I, [_P, _P, _P, _I, _I, _I, _I, _I, _P]),
        "restrict_": (None, [_P, _P, _I, _I, _I, _I, _I, _P]),
        "coarsenmatrix": (None, [_P, _P, _P, _P, _I, _I, _I, _I, _I]),
        "computenorm": (_D, [_P, _P, _I, _I, _I]),
        "computeinner": (_D, [_P, _P, _P, _I, _I, _I]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


class _Arg:
    """Contiguous buffer for one array argument, copied back if needed."""

    def __init__(self, a, dtype, writeback):
        if not isinstance(a, np.ndarray):
            raise TypeError("expected a numpy array, got %r" % type(a))
        self.orig = a
        self.writeback = writeback
        if a.dtype == dtype and a.flags["C_CONTIGUOUS"]:
            self.buf = a
            self.copied = False
        else:
            self.buf = np.ascontiguousarray(a, dtype=dtype)
            self.copied = True

    @property
    def ptr(self):
        return self.buf.ctypes.data

    def done(self):
        if self.copied and self.writeback:
            self.orig[...] = self.buf


def _f64(a, wb=False):
    return _Arg(a, np.float64, wb)


def _i8(a):
    if a.dtype != np.int8:
        raise TypeError("mask arrays are int8 (integer*1), got %s" % a.dtype)
    return _Arg(a, np.int8, False)


def _mn(a):
    if a.ndim < 2:
        raise ValueError("expected a 2D (m, n) array")
    return int(a.shape[0]), int(a.shape[1])


def _check(a, b):
    if a.shape[:2] != b.shape[:2]:
        raise ValueError("shape mismatch %s vs %s" % (a.shape, b.shape))


# ---------------------------------------------------------------- advection
def _adv(name, msk, x, y, u, v, cst, nh, method, order, xflx=None, yflx=None):
    for a in (x, y, u, v):
        _check(msk, a)
    m, n = _mn(msk)
    M, X, U, V = _i8(msk), _f64(x), _f64(u), _f64(v)
    Y = _f64(y, True)
    C = _f64(np.asarray(cst, dtype=np.float64).reshape(5))
    args = [M.ptr, X.ptr, Y.ptr, U.ptr, V.ptr]
    outs = [Y]
    if xflx is not None:
        XF, YF = _f64(xflx, True), _f64(yflx, True)
        args += [XF.ptr, YF.ptr]
        outs += [XF, YF]
    rc = getattr(lib(), name)(*args, C.ptr, int(nh), int(method), int(order), m, n)
    if rc == 1:
        raise RuntimeError("NHALO = 3 is compulsory with UP5")
    if rc:
        raise RuntimeError("%s: grid too wide for the oracle scratch" % name)
    for o in outs:
        o.done()


def adv_upwind(msk, x, y, u, v, cst, nh, method, order):
    """core/fortran_advection.f90:2-165"""
    _adv("adv_upwind", msk, x, y, u, v, cst, nh, method, order)


def adv_centered(msk, x, y, u, v, cst, nh, method, order):
    """core/fortran_advection.f90:169-284"""
    _adv("adv_centered", msk, x, y, u, v, cst, nh, method, order)


def adv_upwind_flux(msk, x, y, u, v, xflx, yflx, cst, nh, method, order):
    """core/fortran_fluxes.f90:2-170 (fortran_fluxes.adv_upwind)"""
    _adv("adv_upwind_flux", msk, x, y, u, v, cst, nh, method, order, xflx, yflx)


def adv_centered_flux(msk, x, y, u, v, xflx, yflx, cst, nh, method, order):
    """core/fortran_fluxes.f90:174-279 (fortran_fluxes.adv_centered)"""
    _adv("adv_centered_flux", msk, x, y, u, v, cst, nh, method, order, xflx, yflx)


# ---------------------------------------------------------------- operators
def computeorthogradient(msk, psi, dx, dy, nh, u, v):
    """core/fortran_operators.f90:2-39"""
    m, n = _mn(msk)
    M, P, U, V = _i8(msk), _f64(psi), _f64(u, True), _f64(v, True)
    lib().computeorthogradient(M.ptr, P.ptr, float(dx), float(dy), int(nh), m, n, U.ptr, V.ptr)
    U.done()
    V.done()


def celltocorner(xr, xp):
    """core/fortran_operators.f90:44-64"""
    m, n = _mn(xr)
    R, P = _f64(xr), _f64(xp, True)
    lib().celltocorner(R.ptr, P.ptr, m, n)
    P.done()


def cornertocell(xp, xr):
    """core/fortran_operators.f90:102-122"""
    m, n = _mn(xp)
    P, R = _f64(xp), _f64(xr, True)
    lib().cornertocell(P.ptr, R.ptr, m, n)
    R.done()


def add_diffusion(msk, trac, dx, nh, Kdiff, dtrac):
    """core/fortran_operators.f90:125-156"""
    m, n = _mn(msk)
    M, T, D = _i8(msk), _f64(trac), _f64(dtrac, True)
    lib().add_diffusion(M.ptr, T.ptr, float(dx), int(nh), float(Kdiff), D.ptr, m, n)
    D.done()


def add_torque(msk, buoy, dx, nh, gravity, domega):
    """core/fortran_operators.f90:330-381"""
    m, n = _mn(msk)
    M, B, W = _i8(msk), _f64(buoy), _f64(domega, True)
    lib().add_torque(M.ptr, B.ptr, float(dx), int(nh), float(gravity), W.ptr, m, n)
    W.done()


def computenoslipsourceterm(msk, x, y, dx, dy, nh):
    """core/fortran_operators.f90:221-277; returns ``total``"""
    m, n = _mn(msk)
    M, X, Y = _i8(msk), _f64(x), _f64(y, True)
    t = lib().computenoslipsourceterm(M.ptr, X.ptr, Y.ptr, float(dx), float(dy), int(nh), m, n)
    Y.done()
    return t


# ---------------------------------------------------------------- diagnostics
def computedotprod(msk, x, y, nh):
    """core/fortran_diag.f90:3-30"""
    m, n = _mn(msk)
    return lib().computedotprod(_i8(msk).ptr, _f64(x).ptr, _f64(y).ptr, int(nh), m, n)


def computemax(msk, x, nh):
    """core/fortran_diag.f90:33-60"""
    m, n = _mn(msk)
    return lib().computemax(_i8(msk).ptr, _f64(x).ptr, int(nh), m, n)


def computesum(msk, x, nh):
    """core/fortran_diag.f90:63-90"""
    m, n = _mn(msk)
    return lib().computesum(_i8(msk).ptr, _f64(x).ptr, int(nh), m, n)


def computesumandnorm(msk, x, nh):
    """core/fortran_diag.f90:93-120; returns ``(y, y2)``"""
    m, n = _mn(msk)
    a, b = ctypes.c_double(), ctypes.c_double()
    M, X = _i8(msk), _f64(x)
    lib().computesumandnorm(M.ptr, X.ptr, int(nh), m, n, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def computenormmaxu(msk, x, nh):
    """core/fortran_diag.f90:123-152; returns ``(y, ymax)``"""
    m, n = _mn(msk)
    a, b = ctypes.c_double(), ctypes.c_double()
    M, X = _i8(msk), _f64(x)
    lib().computenormmaxu(M.ptr, X.ptr, int(nh), m, n, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def computekemaxu(msk, u, v, nh):
    """core/fortran_diag.f90:155-195; returns ``(ke, maxu)``"""
    m, n = _mn(msk)
    a, b = ctypes.c_double(), ctypes.c_double()
    M, U, V = _i8(msk), _f64(u), _f64(v)
    lib().computekemaxu(M.ptr, U.ptr, V.ptr, int(nh), m, n, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def computekemaxuv(msk, u, v, nh):
    """core/fortran_diag.f90:198-236; returns ``(ke, maxu, maxv)``"""
    m, n = _mn(msk)
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    M, U, V = _i8(msk), _f64(u), _f64(v)
    lib().computekemaxuv(M.ptr, U.ptr, V.ptr, int(nh), m, n, ctypes.byref(a),
                         ctypes.byref(b), ctypes.byref(c))
    return a.value, b.value, c.value


def computekewithpsi(msk, omega, psi, nh):
    """core/fortran_diag.f90:239-267"""
    m, n = _mn(msk)
    return lib().computekewithpsi(_i8(msk).ptr, _f64(omega).ptr, _f64(psi).ptr, int(nh), m, n)


# ---------------------------------------------------------------- multigrid
def _a5(A):
    if A.ndim != 3 or A.shape[2] < 5:
        raise ValueError("A must be (m, n, 5)")
    return _f64(np.ascontiguousarray(A[:, :, :5]))


def smoothtwicewitha(msk, A, x, b, coef, yo):
    """core/gmg/fortran_multigrid.f90:2-127"""
    m, n = _mn(msk)
    M, AA, X, B, Y = _i8(msk), _a5(A), _f64(x, True), _f64(b), _f64(yo, True)
    if Y.buf.shape != (3, n):
        raise ValueError("yo must be (3, n)")
    lib().smoothtwicewitha(M.ptr, AA.ptr, X.ptr, B.ptr, float(coef), m, n, Y.ptr)
    X.done()
    Y.done()


def smoothoncewitha(msk, A, x, b, coef, yo=None):
    """core/gmg/fortran_multigrid.f90:130-212"""
    m, n = _mn(msk)
    M, AA, X, B = _i8(msk), _a5(A), _f64(x, True), _f64(b)
    lib().smoothoncewitha(M.ptr, AA.ptr, X.ptr, B.ptr, float(coef), m, n)
    X.done()


def smoothtridiag(msk, A, x, b):
    """core/gmg/fortran_multigrid.f90:215-288"""
    m, n = _mn(msk)
    M, AA, X, B = _i8(msk), _a5(A), _f64(x, True), _f64(b)
    if lib().smoothtridiag(M.ptr, AA.ptr, X.ptr, B.ptr, m, n):
        raise RuntimeError("smoothtridiag: grid too tall for the oracle scratch")
    X.done()


def computeresidualwitha(msk, A, x, b, y):
    """core/gmg/fortran_multigrid.f90:320-362"""
    m, n = _mn(msk)
    M, AA, X, B, Y = _i8(msk), _a5(A), _f64(x), _f64(b), _f64(y, True)
    lib().computeresidualwitha(M.ptr, AA.ptr, X.ptr, B.ptr, Y.ptr, m, n)
    Y.done()


def fillhalo(x, nh):
    """core/gmg/fortran_multigrid.f90:365-412"""
    m, n = _mn(x)
    X = _f64(x, True)
    lib().fillhalo(X.ptr, int(nh), m, n)
    X.done()


def interpolate(msk1, msk2, x2, nh, x1):
    """core/gmg/fortran_multigrid.f90:415-498"""
    m1, n1 = _mn(msk1)
    m2, n2 = _mn(msk2)
    M1, M2, X2, X1 = _i8(msk1), _i8(msk2), _f64(x2), _f64(x1, True)
    if lib().interpolate(M1.ptr, M2.ptr, X2.ptr, int(nh), m2, n2, m1, n1, X1.ptr):
        raise ValueError("interpolate: nh must be 2 or 3")
    X1.done()


def restrict(msk2, x1, nh, x2):
    """core/gmg/fortran_multigrid.f90:501-546"""
    m2, n2 = _mn(msk2)
    m1, n1 = _mn(x1)
    M2, X1, X2 = _i8(msk2), _f64(x1), _f64(x2, True)
    lib().restrict_(M2.ptr, X1.ptr, int(nh), m2, n2, m1, n1, X2.ptr)
    X2.done()


def coarsenmatrix(Afine, msk1, msk2, nh):
    """core/gmg/fortran_multigrid.f90:706-811; returns Acoarse (m2, n2, 9)

    The returned array is zero where the Fortran leaves Acoarse unwritten
    (outside coarse rows/columns nh..m2-nh), as f2py's zero-initialised
    intent(out) buffer would be.
    """
    m1, n1 = _mn(msk1)
    m2, n2 = _mn(msk2)
    AF = _f64(np.ascontiguousarray(Afine[:, :, :9]))
    out = np.zeros((m2, n2, 9))
    lib().coarsenmatrix(AF.ptr, out.ctypes.data, _i8(msk1).ptr, _i8(msk2).ptr,
                        int(nh), m1, n1, m2, n2)
    return out


def computenorm(msk, x, nh):
    """core/gmg/fortran_multigrid.f90:813-839"""
    m, n = _mn(msk)
    return lib().computenorm(_i8(msk).ptr, _f64(x).ptr, int(nh), m, n)


def computeinner(msk, x, y, nh):
    """core/gmg/fortran_multigrid.f90:841-867"""
    m, n = _mn(msk)
    return lib().computeinner(_i8(msk).ptr, _f64(x).ptr, _f64(y).ptr, int(nh), m, n)
