"""The oracle's restated kernels against the mathematics they discretise (no
GPU).  The reference's Fortran cannot be compiled here, so besides the
line-by-line review and the fixtures (which pin everything above the kernels
to the reference's own Python), these checks would catch a mistranscribed
coefficient or index: each kernel converges to the continuous operator at
its design order on smooth periodic fields.

* upwind advection, orders 1/3/5, both flux splittings, x and y, either
  sign of the velocity (core/fortran_advection.f90:2-165);
* centred advection, orders 2/4/6 (core/fortran_advection.f90:169-284);
* diffusion and the Boussinesq torque, second order
  (core/fortran_operators.f90:125-156, 330-381);
* psi -> (u, v) on the staggered grid: u = -dpsi/dy on the right face,
  v = dpsi/dx on the top face, psi at the upper-right corner, second order
  (core/fortran_operators.f90:2-39);
* the flux form moves a constant field by nothing under a velocity that
  comes from a streamfunction: to rounding on periodic domains, to the
  REAL*4 reconstruction weights' sums (1e-8) next to walls;
* cell <-> corner averages and the multigrid's interpolation and
  restriction, second order with their staggering;
* the multigrid solve (core/gmg/hierarchy.py:169-188 over the 9-point
  operator of core/gmg/level.py:261-302) converges to the continuous
  solution at second order and to 1e-12 in a few F-cycles.
"""
import numpy as np
import pytest

from tests import _cases as C

NH = 3
SIDES = (16, 32, 64, 128)


def K():
    from oracle import oracle
    return oracle


def _grid(n, offset):
    """Coordinates (X, Y) of an (n+6)^2 array with the halo, points at
    offset * h from the lower-left corner of each cell (0.5: centres)."""
    h = 1. / n
    c = (np.arange(n + 2 * NH) - NH + offset) * h
    X, Y = np.meshgrid(c, c)
    return h, X, Y


def _orders(errs):
    return [np.log2(errs[k] / errs[k + 1]) for k in range(len(errs) - 1)]


def _inner(a):
    return a[NH:-NH, NH:-NH]


def _advection_errors(kernel, order, method, axis, U):
    errs = []
    for n in SIDES:
        h, X, Y = _grid(n, 0.5)
        s = X if axis == 0 else Y
        q = np.sin(2 * np.pi * s) + 0.5 * np.cos(4 * np.pi * s + 0.3)
        dq = 2 * np.pi * np.cos(2 * np.pi * s) - 2 * np.pi * np.sin(4 * np.pi * s + 0.3)
        u = np.full_like(q, U if axis == 0 else 0.)
        v = np.full_like(q, U if axis == 1 else 0.)
        y = np.zeros_like(q)
        msk = C.mask(n + 2 * NH, n + 2 * NH, "perio", 0, 1)
        getattr(K(), kernel)(msk, q, y, u, v, np.array([h, h, 0.05, abs(U), 0.05]), NH,
                             method, order)
        errs.append(np.abs(_inner(y + U * dq)).max())   # dq/dt = -U dq/ds
    return errs


@pytest.mark.parametrize("order", [1, 3, 5])
@pytest.mark.parametrize("method,axis,U", [(1, 0, 0.7), (1, 1, -0.4), (0, 0, -0.4), (0, 1, 0.7)])
def test_upwind_advection_order(order, method, axis, U):
    p = _orders(_advection_errors("adv_upwind", order, method, axis, U))
    assert all(abs(r - order) < 0.2 for r in p), p


@pytest.mark.parametrize("order", [2, 4, 6])
def test_centered_advection_order(order):
    p = _orders(_advection_errors("adv_centered", order, 1, 0, 0.7))
    assert all(abs(r - order) < 0.2 for r in p), p


@pytest.mark.parametrize("kind", ["diffusion", "torque"])
def test_diffusion_and_torque_second_order(kind):
    errs = []
    for n in SIDES:
        h, X, Y = _grid(n, 0.5)
        q = np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
        y = np.zeros_like(q)
        msk = C.mask(n + 2 * NH, n + 2 * NH, "perio", 0, 1)
        if kind == "diffusion":           # + Kdiff lap(q)
            K().add_diffusion(msk, q, h, NH, 0.3, y)
            want = -0.3 * 8 * np.pi ** 2 * q
        else:                             # + gravity db/dx
            K().add_torque(msk, q, h, NH, 2.0, y)
            want = 2.0 * 2 * np.pi * np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Y)
        errs.append(np.abs(_inner(y - want)).max())
    assert all(abs(r - 2) < 0.1 for r in _orders(errs)), errs


def test_orthogradient_staggering_second_order():
    def psi_f(X, Y):
        return np.sin(2 * np.pi * X) * np.sin(2 * np.pi * Y) + 0.2 * np.cos(2 * np.pi * (X - Y))

    def dpsi(X, Y):
        a, b = 2 * np.pi * X, 2 * np.pi * Y
        return (2 * np.pi * (np.cos(a) * np.sin(b) - 0.2 * np.sin(a - b)),
                2 * np.pi * (np.sin(a) * np.cos(b) + 0.2 * np.sin(a - b)))

    errs = []
    for n in SIDES:
        h, Xc, Yc = _grid(n, 1.0)             # psi at the upper-right corners
        _, Xe, Ye = _grid(n, 0.5)
        psi = psi_f(Xc, Yc)
        u, v = np.zeros_like(psi), np.zeros_like(psi)
        msk = C.mask(n + 2 * NH, n + 2 * NH, "perio", 0, 1)
        K().computeorthogradient(msk, psi, h, h, NH, u, v)
        want_u = -dpsi(Xc, Ye)[1]             # right face: x of the corner, y of the centre
        want_v = dpsi(Xe, Yc)[0]              # top face
        errs.append(max(np.abs(_inner(u - want_u)).max(), np.abs(_inner(v - want_v)).max()))
    assert all(abs(r - 2) < 0.1 for r in _orders(errs)), errs


@pytest.mark.parametrize("geom,islands,bound", [("perio", 0, 1e-14), ("closed", 2, 1e-7),
                                                ("xchannel", 1, 1e-7)])
@pytest.mark.parametrize("order", [1, 3, 5])
def test_streamfunction_velocity_moves_a_constant_by_nothing(geom, islands, bound, order):
    m, n = 38, 54
    msk = C.mask(m, n, geom, islands, 3)
    psi = C.field(m, n, 7) * C.corner_mask(msk)
    K().fillhalo(psi, NH)
    dx = 1. / 48
    u, v = np.zeros((m, n)), np.zeros((m, n))
    K().computeorthogradient(msk, psi, dx, dx, NH, u, v)
    K().fillhalo(u, NH)
    K().fillhalo(v, NH)
    q = 2.0 * msk
    y = np.zeros((m, n))
    K().adv_upwind(msk, q, y, u, v, np.array([dx, dx, 0.05, np.abs(u).max(), 0.05]), NH, 1,
                   order)
    scale = 2.0 * np.abs(u).max() / dx
    assert np.abs(_inner(y * msk)).max() <= bound * scale


def test_poisson_solve_second_order():
    from oracle import stepper
    errs = []
    for n in SIDES:
        h, X, Y = _grid(n, 0.)
        msk = C.corner_mask(C.mask(n + 2 * NH, n + 2 * NH, "perio", 0, 1))
        G = stepper.Gmg({'nh': NH, 'n': n, 'm': n, 'omega': 8. / 9., 'dx': h, 'dy': h},
                        msk * 1.)
        a, c = 2 * np.pi * X, 2 * np.pi * (X + 2 * Y)
        psi = np.sin(a) * np.sin(2 * np.pi * Y) + 0.3 * np.cos(c)
        b = -8 * np.pi ** 2 * np.sin(a) * np.sin(2 * np.pi * Y) - 6 * np.pi ** 2 * np.cos(c)
        x = np.zeros_like(b)
        nite, res = G.solve(x, b, {'maxite': 20, 'tol': 1e-12})
        assert nite <= 8 and res <= 1e-12, (n, nite, res)
        e = _inner(x) - _inner(x).mean() - (_inner(psi) - _inner(psi).mean())
        errs.append(np.abs(e).max())
    assert all(abs(r - 2) < 0.1 for r in _orders(errs)), errs


def _smooth(X, Y):
    return np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y) + 0.3 * np.sin(2 * np.pi * (X + Y))


@pytest.mark.parametrize("kind", ["celltocorner", "cornertocell"])
def test_cell_corner_averages_second_order(kind):
    """celltocorner / cornertocell (core/fortran_operators.f90:44-64,
    102-122): the corner (j, i) is the upper-right corner of cell (j, i)."""
    errs = []
    for n in SIDES:
        _, Xc, Yc = _grid(n, 0.5)
        _, Xk, Yk = _grid(n, 1.0)
        out = np.zeros(Xc.shape)
        if kind == "celltocorner":
            K().celltocorner(_smooth(Xc, Yc), out)
            want = _smooth(Xk, Yk)
        else:
            K().cornertocell(_smooth(Xk, Yk), out)
            want = _smooth(Xc, Yc)
        errs.append(np.abs(_inner(out - want)).max())
    assert all(abs(r - 2) < 0.1 for r in _orders(errs)), errs


@pytest.mark.parametrize("kind", ["interpolate", "restrict"])
def test_transfer_operators_second_order(kind):
    """interpolate / restrict (core/gmg/fortran_multigrid.f90:415-546)
    between the finest level and level 1 of the oracle's hierarchy: a coarse
    point sits midway between the two fine points it covers in each
    direction (fine point i at (i - 3) h, coarse point I at (I - 3) 2h + h)."""
    from oracle import stepper
    errs = []
    for n in (32, 64, 128):
        h = 1. / n
        msk = C.corner_mask(C.mask(n + 2 * NH, n + 2 * NH, "perio", 0, 1))
        G = stepper.Gmg({'nh': NH, 'n': n, 'm': n, 'omega': 8. / 9., 'dx': h, 'dy': h},
                        msk * 1.)
        fine, coarse = G.grid[0], G.grid[1]
        xf = (np.arange(fine.nv) - NH) * h
        xc = (np.arange(coarse.nv) - NH) * 2 * h + h
        Xf, Yf = np.meshgrid(xf, xf)
        Xc, Yc = np.meshgrid(xc, xc)
        if kind == "interpolate":
            out = np.zeros((fine.mv, fine.nv))
            K().interpolate(fine.msk, coarse.msk, _smooth(Xc, Yc), NH, out)
            want = _smooth(Xf, Yf)
        else:
            out = np.zeros((coarse.mv, coarse.nv))
            K().restrict(coarse.msk, _smooth(Xf, Yf), NH, out)
            want = _smooth(Xc, Yc)
        errs.append(np.abs(_inner(out - want)).max())
    assert all(abs(r - 2) < 0.1 for r in _orders(errs)), errs


@pytest.mark.parametrize("hydroepsilon", [1.0, 0.1])
def test_smoothers_keep_the_discrete_solution(hydroepsilon):
    """One smoothing call leaves x unchanged where A x = b: damped Jacobi
    (smoothtwicewithA, core/gmg/fortran_multigrid.f90:2-127) and, for
    hydroepsilon dy/dx <= 0.2, the line relaxation (smoothtridiag,
    :215-288) on a closed domain; the Jacobi form damps the checkerboard
    mode by more than 10."""
    from oracle import stepper
    n = 64
    h = 1. / n
    msk = C.corner_mask(C.mask(n + 2 * NH, n + 2 * NH, "closed", 0, 3))
    G = stepper.Gmg({'nh': NH, 'n': n, 'm': n, 'omega': 8. / 9., 'dx': h, 'dy': h,
                     'hydroepsilon': hydroepsilon}, msk * 1.)
    g = G.grid[0]
    assert g.relaxation == ("tridiagonal" if hydroepsilon < 0.2 else "default")
    x = C.field(n + 2 * NH, n + 2 * NH, 4) * g.msk
    K().fillhalo(x, NH)
    r = np.zeros_like(x)
    K().computeresidualwitha(g.msk, g.A, x, np.zeros_like(x), r)   # r = -A x
    b = -r
    x1 = x.copy()
    g.smooth(x1, b, 1)
    assert np.abs(x1 - x)[g.msk != 0].max() <= 1e-13 * np.abs(x).max()
    if hydroepsilon == 1.0:
        J, I = np.indices(x.shape)
        e = (-1.) ** (J + I) * g.msk
        g.smooth(e, np.zeros_like(e), 1)
        assert np.abs(_inner(e)).max() < 0.1


def test_line_relaxation_across_an_island_is_not_finite():
    """The reference's line relaxation divides by the diagonal of every point
    of a column whose first interior row is fluid (smoothtridiag and tridiag,
    core/gmg/fortran_multigrid.f90:240-317), so a column that crosses an
    island (zero diagonal) gets non-finite values: it is meant for columns
    fluid from wall to wall.  The restatement keeps that behaviour."""
    from oracle import stepper
    n = 64
    h = 1. / n
    msk = C.corner_mask(C.mask(n + 2 * NH, n + 2 * NH, "closed", 2, 3))
    G = stepper.Gmg({'nh': NH, 'n': n, 'm': n, 'omega': 8. / 9., 'dx': h, 'dy': h,
                     'hydroepsilon': 0.1}, msk * 1.)
    g = G.grid[0]
    x = C.field(n + 2 * NH, n + 2 * NH, 4) * g.msk
    with np.errstate(all="ignore"):
        K().smoothtridiag(g.msk, g.A, x, np.zeros_like(x))
    assert not np.all(np.isfinite(x))
