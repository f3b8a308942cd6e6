"""The reference's f2py kernel modules, backed by the GB300 kernels.

Every function keeps the Python signature f2py generates for the Fortran
routine it replaces (dimension arguments inferred from the arrays,
``intent(out)`` scalars returned, ``intent(inplace)`` arrays updated in
place), so Fluid2d's callers need no change:

* fortran_advection: adv_upwind, adv_centered   (core/fortran_advection.f90)
* fortran_fluxes:    flx_adv_upwind, flx_adv_centered
                     (core/fortran_fluxes.f90, exported there as adv_upwind,
                     adv_centered -- see fluid2d_gb300/f2py_compat)
* fortran_operators: computeorthogradient, celltocorner, cornertocell,
                     add_diffusion, add_torque, computenoslipsourceterm
                     (core/fortran_operators.f90)
* fortran_diag:      computedotprod, computemax, computesum,
                     computesumandnorm, computenormmaxu, computekemaxu,
                     computekemaxuv, computekewithpsi  (core/fortran_diag.f90)
* gmg.fortran_multigrid: smoothtwicewitha, computeresidualwitha, fillhalo,
                     interpolate, restrict, coarsenmatrix, computenorm,
                     computeinner  (core/gmg/fortran_multigrid.f90)

Arrays may be CUDA tensors (used in place, no copy when contiguous) or
numpy arrays (copied to the GPU for the call and back afterwards -- the
reference-facing host-buffer path).  Errors raise ``F2DError`` instead of
stopping the process.  ``use_variant('exact')`` switches to the build that
rounds every operation separately.
"""
import numpy as np
import torch

from . import _lib

_variant = "product"


def use_variant(name):
    """Select 'product' or 'exact' for the following calls; returns the old one."""
    global _variant
    if name not in _lib.VARIANTS:
        raise ValueError(name)
    old, _variant = _variant, name
    return old


def device():
    if not torch.cuda.is_available():
        raise RuntimeError("fluid2d_gb300 needs a CUDA device (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle():
    return ctypes_stream(torch.cuda.current_stream())


def ctypes_stream(s):
    return s.cuda_stream


_TORCH = {np.float64: torch.float64, np.int8: torch.int8, np.float32: torch.float32}


class Arg(object):
    """One array argument bound to a contiguous CUDA buffer."""

    def __init__(self, a, dtype, out=False):
        self.orig = a
        self.out = out
        tdt = _TORCH[dtype]
        if isinstance(a, torch.Tensor):
            if a.device.type != "cuda":
                raise TypeError("tensor arguments must live on the GPU")
            if a.dtype == tdt and a.is_contiguous():
                self.t, self.copy = a, False
            else:
                self.t, self.copy = a.to(dtype=tdt).contiguous(), True
        elif isinstance(a, np.ndarray):
            if dtype is np.int8 and a.dtype != np.int8:
                raise TypeError("mask arrays are int8 (integer*1), got %s" % a.dtype)
            h = np.ascontiguousarray(a, dtype=dtype)
            self.t = torch.from_numpy(h).to(device())
            self.copy = True
        else:
            raise TypeError("expected a torch tensor or numpy array, got %r" % type(a))

    @property
    def ptr(self):
        return self.t.data_ptr()

    @property
    def shape(self):
        return tuple(self.t.shape)

    def done(self):
        if not (self.out and self.copy):
            return
        if isinstance(self.orig, torch.Tensor):
            self.orig.copy_(self.t)
        else:
            self.orig[...] = self.t.cpu().numpy()


def _f64(a, out=False):
    return Arg(a, np.float64, out)


def _i8(a):
    return Arg(a, np.int8)


def _mn(a):
    s = a.shape
    if len(s) < 2:
        raise ValueError("expected a 2D (m, n) array")
    return int(s[0]), int(s[1])


def _same(msk, *arrs):
    for a in arrs:
        if a is not None and tuple(a.shape[:2]) != tuple(msk.shape[:2]):
            raise ValueError("shape mismatch %s vs %s" % (tuple(a.shape), tuple(msk.shape)))


def _planes(A, k):
    """A stencil array as a planar (k, m, n) CUDA float64 tensor.

    Accepts the reference layout (m, n, >=k) from numpy or torch, or an
    already planar (k, m, n) CUDA tensor.
    """
    if isinstance(A, torch.Tensor) and A.device.type == "cuda":
        if A.dim() == 3 and A.shape[0] == k and A.shape[2] != k:
            return A.to(torch.float64).contiguous()
        return A[:, :, :k].permute(2, 0, 1).to(torch.float64).contiguous()
    a = np.asarray(A)
    if a.ndim != 3 or a.shape[2] < k:
        raise ValueError("A must be (m, n, %d)" % k)
    h = np.ascontiguousarray(np.moveaxis(a[:, :, :k], 2, 0), dtype=np.float64)
    return torch.from_numpy(h).to(device())


def _call(name, *args):
    _lib.call(name, *args, variant=_variant)


def _scalars(k):
    return torch.zeros(k, dtype=torch.float64, device=device())


def _host(t):
    v = t.cpu().numpy().tolist()
    return v


# ---------------------------------------------------------------- advection
def _cst(cst):
    if isinstance(cst, torch.Tensor) and cst.device.type == "cuda":
        return _f64(cst.reshape(5))
    return _f64(np.asarray(cst, dtype=np.float64).reshape(5))


def _adv(name, msk, x, y, u, v, cst, nh, method, order, xflx=None, yflx=None):
    _same(msk, x, y, u, v, xflx, yflx)
    m, n = _mn(msk)
    M, X, U, V, C = _i8(msk), _f64(x), _f64(u), _f64(v), _cst(cst)
    Y = _f64(y, True)
    outs = [Y]
    if xflx is not None:
        XF, YF = _f64(xflx, True), _f64(yflx, True)
        outs += [XF, YF]
        _call(name, M.ptr, X.ptr, Y.ptr, U.ptr, V.ptr, XF.ptr, YF.ptr, C.ptr, int(nh),
              int(method), int(order), m, n, stream_handle())
    else:
        _call(name, M.ptr, X.ptr, Y.ptr, U.ptr, V.ptr, C.ptr, int(nh), int(method), int(order),
              m, n, stream_handle())
    for o in outs:
        o.done()


def adv_upwind(msk, x, y, u, v, cst, nh, method, order):
    """core/fortran_advection.f90:2-165"""
    _adv("f2d_adv_upwind", msk, x, y, u, v, cst, nh, method, order)


def adv_centered(msk, x, y, u, v, cst, nh, method, order):
    """core/fortran_advection.f90:169-284"""
    _adv("f2d_adv_centered", msk, x, y, u, v, cst, nh, method, order)


def flx_adv_upwind(msk, x, y, u, v, xflx, yflx, cst, nh, method, order):
    """core/fortran_fluxes.f90:2-170 (fortran_fluxes.adv_upwind)"""
    _adv("f2d_flx_adv_upwind", msk, x, y, u, v, cst, nh, method, order, xflx, yflx)


def flx_adv_centered(msk, x, y, u, v, xflx, yflx, cst, nh, method, order):
    """core/fortran_fluxes.f90:174-279 (fortran_fluxes.adv_centered)"""
    _adv("f2d_flx_adv_centered", msk, x, y, u, v, cst, nh, method, order, xflx, yflx)


# ---------------------------------------------------------------- operators
def computeorthogradient(msk, psi, dx, dy, nh, u, v):
    """core/fortran_operators.f90:2-39"""
    _same(msk, psi, u, v)
    m, n = _mn(msk)
    M, P, U, V = _i8(msk), _f64(psi), _f64(u, True), _f64(v, True)
    _call("f2d_computeorthogradient", M.ptr, P.ptr, float(dx), float(dy), int(nh), m, n, U.ptr,
          V.ptr, stream_handle())
    U.done()
    V.done()


def celltocorner(xr, xp):
    """core/fortran_operators.f90:44-64"""
    _same(xr, xp)
    m, n = _mn(xr)
    R, P = _f64(xr), _f64(xp, True)
    _call("f2d_celltocorner", R.ptr, P.ptr, m, n, stream_handle())
    P.done()


def cornertocell(xp, xr):
    """core/fortran_operators.f90:102-122"""
    _same(xp, xr)
    m, n = _mn(xp)
    P, R = _f64(xp), _f64(xr, True)
    _call("f2d_cornertocell", P.ptr, R.ptr, m, n, stream_handle())
    R.done()


def add_diffusion(msk, trac, dx, nh, Kdiff, dtrac):
    """core/fortran_operators.f90:125-156"""
    _same(msk, trac, dtrac)
    m, n = _mn(msk)
    M, T, D = _i8(msk), _f64(trac), _f64(dtrac, True)
    _call("f2d_add_diffusion", M.ptr, T.ptr, float(dx), int(nh), float(Kdiff), D.ptr, m, n,
          stream_handle())
    D.done()


def add_torque(msk, buoy, dx, nh, gravity, domega):
    """core/fortran_operators.f90:330-381"""
    _same(msk, buoy, domega)
    m, n = _mn(msk)
    M, B, W = _i8(msk), _f64(buoy), _f64(domega, True)
    _call("f2d_add_torque", M.ptr, B.ptr, float(dx), int(nh), float(gravity), W.ptr, m, n,
          stream_handle())
    W.done()


def computenoslipsourceterm(msk, x, y, dx, dy, nh):
    """core/fortran_operators.f90:221-277 -> total (y updated in place)"""
    _same(msk, x, y)
    m, n = _mn(msk)
    M, X, Y = _i8(msk), _f64(x), _f64(y, True)
    out = _scalars(1)
    _call("f2d_computenoslipsourceterm", M.ptr, X.ptr, Y.ptr, float(dx), float(dy), int(nh), m,
          n, out.data_ptr(), stream_handle())
    Y.done()
    return _host(out)[0]


# ---------------------------------------------------------------- diagnostics
def _reduce(name, k, msk, x, y, nh):
    _same(msk, x, y)
    m, n = _mn(msk)
    M, X = _i8(msk), _f64(x)
    out = _scalars(k)
    if y is None:
        _call(name, M.ptr, X.ptr, int(nh), m, n, out.data_ptr(), stream_handle())
    else:
        Y = _f64(y)
        _call(name, M.ptr, X.ptr, Y.ptr, int(nh), m, n, out.data_ptr(), stream_handle())
    vals = _host(out)
    return vals[0] if k == 1 else tuple(vals)


def computedotprod(msk, x, y, nh):
    """core/fortran_diag.f90:3-30"""
    return _reduce("f2d_computedotprod", 1, msk, x, y, nh)


def computemax(msk, x, nh):
    """core/fortran_diag.f90:33-60"""
    return _reduce("f2d_computemax", 1, msk, x, None, nh)


def computesum(msk, x, nh):
    """core/fortran_diag.f90:63-90"""
    return _reduce("f2d_computesum", 1, msk, x, None, nh)


def computesumandnorm(msk, x, nh):
    """core/fortran_diag.f90:93-120 -> (y, y2)"""
    return _reduce("f2d_computesumandnorm", 2, msk, x, None, nh)


def computenormmaxu(msk, x, nh):
    """core/fortran_diag.f90:123-152 -> (y, ymax)"""
    return _reduce("f2d_computenormmaxu", 2, msk, x, None, nh)


def computekemaxu(msk, u, v, nh):
    """core/fortran_diag.f90:155-195 -> (ke, maxu)"""
    return _reduce("f2d_computekemaxu", 2, msk, u, v, nh)


def computekemaxuv(msk, u, v, nh):
    """core/fortran_diag.f90:198-236 -> (ke, maxu, maxv)"""
    return _reduce("f2d_computekemaxuv", 3, msk, u, v, nh)


def computekewithpsi(msk, omega, psi, nh):
    """core/fortran_diag.f90:239-267"""
    return _reduce("f2d_computekewithpsi", 1, msk, omega, psi, nh)


# ---------------------------------------------------------------- multigrid
def smoothtwicewitha(msk, A, x, b, coef, yo=None):
    """core/gmg/fortran_multigrid.f90:2-127 (yo is accepted and ignored:
    the 3-row buffer of the Fortran is a library scratch array here)"""
    _same(msk, x, b)
    m, n = _mn(msk)
    M, X, B = _i8(msk), _f64(x, True), _f64(b)
    AP = _planes(A, 5)
    _call("f2d_smoothtwicewitha", M.ptr, AP.data_ptr(), X.ptr, B.ptr, float(coef), m, n,
          stream_handle())
    X.done()


def smoothtridiag(msk, A, x, b):
    """core/gmg/fortran_multigrid.f90:215-317 (one vertical line-relaxation sweep)"""
    _same(msk, x, b)
    m, n = _mn(msk)
    M, X, B = _i8(msk), _f64(x, True), _f64(b)
    AP = _planes(A, 5)
    _call("f2d_smoothtridiag", M.ptr, AP.data_ptr(), X.ptr, B.ptr, m, n, stream_handle())
    X.done()


def computeresidualwitha(msk, A, x, b, y):
    """core/gmg/fortran_multigrid.f90:320-362"""
    _same(msk, x, b, y)
    m, n = _mn(msk)
    M, X, B, Y = _i8(msk), _f64(x), _f64(b), _f64(y, True)
    AP = _planes(A, 5)
    _call("f2d_computeresidualwitha", M.ptr, AP.data_ptr(), X.ptr, B.ptr, Y.ptr, m, n,
          stream_handle())
    Y.done()


def fillhalo(x, nh):
    """core/gmg/fortran_multigrid.f90:365-412"""
    m, n = _mn(x)
    X = _f64(x, True)
    _call("f2d_fillhalo", X.ptr, int(nh), m, n, stream_handle())
    X.done()


def interpolate(msk1, msk2, x2, nh, x1):
    """core/gmg/fortran_multigrid.f90:415-498"""
    _same(msk1, x1)
    _same(msk2, x2)
    m1, n1 = _mn(msk1)
    m2, n2 = _mn(msk2)
    M1, M2, X2, X1 = _i8(msk1), _i8(msk2), _f64(x2), _f64(x1, True)
    _call("f2d_interpolate", M1.ptr, M2.ptr, X2.ptr, int(nh), m2, n2, m1, n1, X1.ptr,
          stream_handle())
    X1.done()


def restrict(msk2, x1, nh, x2):
    """core/gmg/fortran_multigrid.f90:501-546"""
    _same(msk2, x2)
    m2, n2 = _mn(msk2)
    m1, n1 = _mn(x1)
    M2, X1, X2 = _i8(msk2), _f64(x1), _f64(x2, True)
    _call("f2d_restrict", M2.ptr, X1.ptr, int(nh), m2, n2, m1, n1, X2.ptr, stream_handle())
    X2.done()


def coarsenmatrix(Afine, msk1, msk2, nh):
    """core/gmg/fortran_multigrid.f90:706-811 -> Acoarse (m2, n2, 9)

    Returned in the reference layout: a C-ordered numpy array for numpy
    inputs, else a CUDA tensor view (m2, n2, 9).  Cells the Fortran does not
    write are 0.
    """
    m1, n1 = _mn(msk1)
    m2, n2 = _mn(msk2)
    AF = _planes(Afine, 9)
    M1, M2 = _i8(msk1), _i8(msk2)
    out = torch.zeros((9, m2, n2), dtype=torch.float64, device=device())
    _call("f2d_coarsenmatrix", AF.data_ptr(), M1.ptr, M2.ptr, int(nh), m1, n1, m2, n2,
          out.data_ptr(), stream_handle())
    res = out.permute(1, 2, 0)
    if isinstance(msk2, np.ndarray):
        return np.ascontiguousarray(res.cpu().numpy())
    return res


def computenorm(msk, x, nh):
    """core/gmg/fortran_multigrid.f90:813-839"""
    return _reduce("f2d_computenorm", 1, msk, x, None, nh)


def computeinner(msk, x, y, nh):
    """core/gmg/fortran_multigrid.f90:841-867"""
    return _reduce("f2d_computeinner", 1, msk, x, y, nh)
