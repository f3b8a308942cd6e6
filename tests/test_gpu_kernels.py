"""Per-routine parity: each GB300 kernel against the C oracle of the Fortran.

With the exact build (every operation rounded separately) the full output
arrays, halos included, must be bit-identical to the oracle's for every
routine except the reductions (whose summation order differs; maxima stay
exact).  With the product build (FMA contraction allowed) values agree to a
relative 1e-12 and every cell the routine must not touch is unchanged.
"""
import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu

SHAPES = [(22, 22), (38, 70), (71, 39), (134, 134)]
GEOMS = ["closed", "perio", "xchannel"]
VARIANTS = ["exact", "product"]


@pytest.fixture(scope="module")
def gk():
    import torch
    from fluid2d_gb300 import kernels
    assert torch.cuda.is_available()
    return kernels


@pytest.fixture(params=VARIANTS)
def variant(request, gk):
    old = gk.use_variant(request.param)
    yield request.param
    gk.use_variant(old)


def K():
    from oracle import oracle
    return oracle


def cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def check(got, ref, variant, rtol=1e-12):
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    if variant == "exact":
        assert np.array_equal(got, ref, equal_nan=True), "max |diff| %g" % np.nanmax(
            np.abs(got - ref))
    else:
        scale = max(1e-300, np.nanmax(np.abs(ref)))
        d = np.nanmax(np.abs(got - ref))
        assert d <= rtol * scale, "max rel diff %g" % (d / scale)


def cases():
    out = []
    for k, (m, n) in enumerate(SHAPES):
        for g in GEOMS:
            out.append((m, n, g, k % 4, 100 * k + GEOMS.index(g)))
    return out


@pytest.mark.parametrize("m,n,geom,islands,seed", cases())
@pytest.mark.parametrize("method,order", [(1, 5), (0, 5), (1, 3), (0, 1)])
def test_adv_upwind(gk, variant, m, n, geom, islands, seed, method, order):
    msk = C.mask(m, n, geom, islands, seed)
    x, u, v = C.field(m, n, seed + 1), C.field(m, n, seed + 2, 0.3), C.field(m, n, seed + 3, 0.3)
    cst = np.array([1. / (n - 6), 1. / (m - 6), 0.05, 0.9, 0.05])
    y0 = C.field(m, n, seed + 4)  # halo content must survive
    yr = y0.copy()
    K().adv_upwind(msk, x, yr, u, v, cst, 3, method, order)
    yg = cuda(y0)
    gk.adv_upwind(cuda(msk), cuda(x), yg, cuda(u), cuda(v), cuda(cst), 3, method, order)
    check(host(yg), yr, variant)


@pytest.mark.parametrize("m,n,geom,islands,seed", cases()[:6])
@pytest.mark.parametrize("order", [2, 4, 6])
def test_adv_centered_and_fluxes(gk, variant, m, n, geom, islands, seed, order):
    msk = C.mask(m, n, geom, islands, seed)
    x, u, v = C.field(m, n, seed + 1), C.field(m, n, seed + 2), C.field(m, n, seed + 3)
    cst = np.array([0.1, 0.2, 0.05, 0., 0.])
    y0 = C.field(m, n, seed + 4)
    yr = y0.copy()
    K().adv_centered(msk, x, yr, u, v, cst, 3, 0, order)
    yg = cuda(y0)
    gk.adv_centered(cuda(msk), cuda(x), yg, cuda(u), cuda(v), cuda(cst), 3, 0, order)
    check(host(yg), yr, variant)
    # fortran_fluxes variants: y plus the edge fluxes
    for up in (True, False):
        yr, xf, yf = y0.copy(), C.field(m, n, 7), C.field(m, n, 8)
        yg, xfg, yfg = cuda(y0), cuda(xf), cuda(yf)
        if up:
            K().adv_upwind_flux(msk, x, yr, u, v, xf, yf, np.array([0.1, 0.2, 0.05, 1., 0.05]),
                                3, 1, 5)
            gk.flx_adv_upwind(cuda(msk), cuda(x), yg, cuda(u), cuda(v), xfg, yfg,
                              cuda(np.array([0.1, 0.2, 0.05, 1., 0.05])), 3, 1, 5)
        else:
            K().adv_centered_flux(msk, x, yr, u, v, xf, yf, cst, 3, 0, min(order, 4))
            gk.flx_adv_centered(cuda(msk), cuda(x), yg, cuda(u), cuda(v), xfg, yfg, cuda(cst),
                                3, 0, min(order, 4))
        check(host(yg), yr, variant)
        check(host(xfg), xf, variant)
        check(host(yfg), yf, variant)


def test_adv_nh_error(gk):
    from fluid2d_gb300._lib import F2DError
    m, n = 22, 22
    msk = C.mask(m, n)
    x = C.field(m, n)
    with pytest.raises(F2DError) as e:
        gk.adv_upwind(cuda(msk), cuda(x), cuda(x.copy()), cuda(x), cuda(x),
                      cuda(np.ones(5)), 2, 1, 5)
    assert e.value.code == 1


@pytest.mark.parametrize("m,n,geom,islands,seed", cases())
def test_operators(gk, variant, m, n, geom, islands, seed):
    msk = C.mask(m, n, geom, islands, seed)
    psi, w, b = C.field(m, n, seed), C.field(m, n, seed + 1), C.field(m, n, seed + 2)
    dx, dy = 1. / (n - 6), 1.3 / (m - 6)
    # computeorthogradient: untouched outer ring keeps its content
    u0, v0 = C.field(m, n, 11), C.field(m, n, 12)
    ur, vr = u0.copy(), v0.copy()
    K().computeorthogradient(msk, psi, dx, dy, 3, ur, vr)
    ug, vg = cuda(u0), cuda(v0)
    gk.computeorthogradient(cuda(msk), cuda(psi), dx, dy, 3, ug, vg)
    check(host(ug), ur, variant)
    check(host(vg), vr, variant)
    # celltocorner / cornertocell
    xr = C.field(m, n, 13)
    for fn in ("celltocorner", "cornertocell"):
        xp0 = C.field(m, n, 14)
        ref = xp0.copy()
        getattr(K(), fn)(xr, ref)
        g = cuda(xp0)
        getattr(gk, fn)(cuda(xr), g)
        check(host(g), ref, variant)
    # add_diffusion / add_torque accumulate into the tendency
    ref = w.copy()
    K().add_diffusion(msk, psi, dx, 3, 0.37, ref)
    g = cuda(w)
    gk.add_diffusion(cuda(msk), cuda(psi), dx, 3, 0.37, g)
    check(host(g), ref, variant)
    ref = w.copy()
    K().add_torque(msk, b, dx, 3, 5.0, ref)
    g = cuda(w)
    gk.add_torque(cuda(msk), cuda(b), dx, 3, 5.0, g)
    check(host(g), ref, variant)


@pytest.mark.parametrize("m,n,geom,islands,seed", cases())
def test_computenoslipsourceterm(gk, variant, m, n, geom, islands, seed):
    """core/fortran_operators.f90:221-277 as core/operators.py:256 calls it:
    the whole output array (the cells its loop writes, its scatters into row
    and column nh, the untouched rest) and the returned total, which the
    Fortran sums in loop order (bit-identical in the exact build)."""
    msk = C.mask(m, n, geom, islands + 1, seed)
    psi = C.field(m, n, seed + 5)
    dx, dy = 1. / (n - 6), 1.3 / (m - 6)
    y0 = C.field(m, n, seed + 6)
    yr = y0.copy()
    tr = K().computenoslipsourceterm(msk, psi, yr, dx, dy, 3)
    yg = cuda(y0)
    tg = gk.computenoslipsourceterm(cuda(msk), cuda(psi), yg, dx, dy, 3)
    check(host(yg), yr, variant)
    if variant == "exact":
        assert tg == tr
    else:
        assert abs(tg - tr) <= 1e-12 * max(np.abs(yr).sum(), 1e-300)
    # numpy arrays (the reference's own call) take the host-buffer path
    yh = y0.copy()
    th = gk.computenoslipsourceterm(msk, psi, yh, dx, dy, 3)
    check(yh, yr, variant)
    assert th == tg


@pytest.mark.parametrize("m,n,geom,islands,seed", cases())
def test_diagnostics(gk, variant, m, n, geom, islands, seed):
    msk = C.mask(m, n, geom, islands, seed)
    u, v, x = C.field(m, n, seed), C.field(m, n, seed + 1), C.field(m, n, seed + 2)
    M = cuda(msk)
    U, V, X = cuda(u), cuda(v), cuda(x)

    def close(a, b, exact_max=()):
        a, b = np.atleast_1d(a), np.atleast_1d(b)
        for k in range(len(a)):
            if k in exact_max:
                assert a[k] == b[k]
            else:
                assert abs(a[k] - b[k]) <= 1e-12 * max(1., abs(b[k])), (k, a, b)

    close(gk.computekemaxu(M, U, V, 3), K().computekemaxu(msk, u, v, 3), exact_max=(1,))
    # maxu/maxv of computekemaxuv are maxima of u^2+u'^2, which FMA contraction
    # may round differently: exact only in the exact build
    close(gk.computekemaxuv(M, U, V, 3), K().computekemaxuv(msk, u, v, 3),
          exact_max=(1, 2) if variant == "exact" else ())
    close(gk.computesumandnorm(M, X, 3), K().computesumandnorm(msk, x, 3))
    close(gk.computenormmaxu(M, X, 3), K().computenormmaxu(msk, x, 3), exact_max=(1,))
    close(gk.computedotprod(M, X, U, 3), K().computedotprod(msk, x, u, 3))
    close(gk.computesum(M, X, 3), K().computesum(msk, x, 3))
    close(gk.computemax(M, X, 3), K().computemax(msk, x, 3), exact_max=(0,))
    close(gk.computekewithpsi(M, X, U, 3), K().computekewithpsi(msk, x, u, 3))
    close(gk.computenorm(M, X, 3), K().computenorm(msk, x, 3))
    close(gk.computeinner(M, X, V, 3), K().computeinner(msk, x, v, 3))


def _hierarchy(m, n, geom, islands, seed, dx=None, dy=None):
    """Oracle levels with their 9-plane operators (before ninetofive)."""
    from oracle import stepper
    msk = C.corner_mask(C.mask(m, n, geom, islands, seed))
    dx = dx or 1. / (n - 6)
    dy = dy or dx
    info = stepper.gridinfo(n - 6, m - 6, dx, dy)
    levs = [stepper.Level(inf, 3, 8. / 9., 1., 'default') for inf in info]
    levs[0].set_finest(msk)
    for k in range(1, len(levs)):
        levs[k].set_coarser(levs[k - 1])
    return levs


HSHAPES = [(38, 38, "closed", 2, 1), (70, 38, "perio", 0, 2), (134, 70, "xchannel", 3, 3)]


@pytest.mark.parametrize("m,n,geom,islands,seed", HSHAPES)
def test_multigrid_kernels(gk, variant, m, n, geom, islands, seed):
    levs = _hierarchy(m, n, geom, islands, seed)
    for k, L in enumerate(levs):
        mv, nv = L.mv, L.nv
        x, b = C.field(mv, nv, 10 * k), C.field(mv, nv, 10 * k + 1)
        A5 = L.A[:, :, :5]
        # smoothtwicewitha: the whole array, quirk cells included
        ref = x.copy()
        K().smoothtwicewitha(L.msk, A5, ref, b, 8. / 9., np.zeros((3, nv)))
        g = cuda(x)
        gk.smoothtwicewitha(cuda(L.msk), A5, g, cuda(b), 8. / 9.)
        check(host(g), ref, variant)
        # residual (outer ring untouched)
        r0 = C.field(mv, nv, 99)
        ref = r0.copy()
        K().computeresidualwitha(L.msk, A5, x, b, ref)
        g = cuda(r0)
        gk.computeresidualwitha(cuda(L.msk), A5, cuda(x), cuda(b), g)
        check(host(g), ref, variant)
        # fillhalo
        ref = x.copy()
        K().fillhalo(ref, 3)
        g = cuda(x)
        gk.fillhalo(g, 3)
        assert np.array_equal(host(g), ref)
        if k + 1 < len(levs):
            Lc = levs[k + 1]
            # restrict fine -> coarse
            c0 = C.field(Lc.mv, Lc.nv, 5)
            ref = c0.copy()
            K().restrict(Lc.msk, x, 3, ref)
            g = cuda(c0)
            gk.restrict(cuda(Lc.msk), cuda(x), 3, g)
            check(host(g), ref, variant)
            # interpolate coarse -> fine
            xc = C.field(Lc.mv, Lc.nv, 6)
            ref = r0.copy()
            K().interpolate(L.msk, Lc.msk, xc, 3, ref)
            g = cuda(r0)
            gk.interpolate(cuda(L.msk), cuda(Lc.msk), cuda(xc), 3, g)
            check(host(g), ref, variant)
            # coarsenmatrix (written cells only; f2py's buffer is zero elsewhere)
            ref = K().coarsenmatrix(L.A, L.msk, Lc.msk, 3)
            got = gk.coarsenmatrix(L.A, L.msk, Lc.msk, 3)
            check(np.asarray(got), ref, variant)


@pytest.mark.parametrize("m,n,geom,islands,seed", [(102, 22, "closed", 0, 4),
                                                   (70, 38, "xchannel", 2, 5),
                                                   (134, 70, "perio", 0, 6)])
def test_smoothtridiag(gk, variant, m, n, geom, islands, seed):
    """The vertical line relaxation on the levels of a flat-cell hierarchy
    (dy = dx/6), whole array compared (no halo fill inside the routine)."""
    dx = 1. / (n - 6)
    levs = _hierarchy(m, n, geom, islands, seed, dx=dx, dy=dx / 6)
    for k, L in enumerate(levs):
        if L.m + 6 < 8:
            continue
        mv, nv = L.mv, L.nv
        x, b = C.field(mv, nv, 20 * k), C.field(mv, nv, 20 * k + 1)
        A5 = np.ascontiguousarray(L.A[:, :, :5])
        ref = x.copy()
        for _ in range(3):
            K().smoothtridiag(L.msk, A5, ref, b)
        g = cuda(x)
        for _ in range(3):
            gk.smoothtridiag(cuda(L.msk), A5, g, cuda(b))
        check(host(g), ref, variant)
