"""Restatement of Fluid2d's Python sequencing over the C oracle kernels.

TEST INFRASTRUCTURE ONLY: the step-level reference the parity tests compare
fluid2d_gb300 against.
Only tests/, __graft_entry__.smoke() and the CPU baseline / reference arm of
bench.py may import it.

It restates, for one MPI rank, the numpy code of

* core/grid.py:12-140               grid, masks, coordinates, areas
* core/gmg/level.py:24-496          level hierarchy, masks and operators,
                                    smooth/residual/norm, fine<->coarse
* core/gmg/hierarchy.py:21-218      Vcycle, Fcycle, solve, twoVcycle
* core/operators.py:12-236,303-314,421-498
                                    corner mask, rhs_adv, rhs_torque,
                                    rhs_diffusion, invert_vorticity
* core/timescheme.py:6-201          the time schemes
* core/euler.py, core/boussinesq.py, core/quasigeostrophic.py
                                    step / dynamics / diagnostics
* core/fluid2d.py:235-314,376-397   the time loop and set_dt

with the same numpy expressions in the same order, so that it reproduces the
reference's own Python bit for bit when both run over the same kernels
(checked by tests/golden/make_golden.py, which imports the reference).

One deliberate difference: when a grid dimension becomes odd before the
coarsest level is reached, coarsening stops there (the reference would halve
the odd dimension, giving a coarse grid that no longer covers the fine one).
Power-of-two grids, which are all the reference supports, are unaffected.
"""
import numpy as np

try:  # imported as part of the ``oracle`` package
    from . import oracle as K
except ImportError:  # imported with oracle/ itself on sys.path
    import oracle as K


def use_kernels(kernels):
    """Run the sequencing over another kernel set with the oracle's names
    (the tests pass the GPU drop-in modules of fluid2d_gb300.f2py_compat,
    mapped by ``oracle.refshim.F2PY_NAMES``); returns the previous set."""
    global K
    old, K = K, kernels
    return old


class Param(object):
    """The defaults of core/defaults.json that the hot path reads."""

    def __init__(self, **kw):
        self.modelname = 'euler'
        self.nx = 128
        self.ny = 128
        self.Lx = 1.
        self.Ly = 1.
        self.nh = 3
        self.geometry = 'closed'
        self.order = 5
        self.aparab = 0.05
        self.flux_splitting_method = 'parabolic'
        self.timestepping = 'RK3_SSP'
        self.hydroepsilon = 1.
        self.relaxation = 'default'
        self.diffusion = False
        self.Kdiff = 0.
        self.gravity = 1.
        self.Rd = 1.
        self.beta = 0.
        self.noslip = False
        self.adaptable_dt = False
        self.dt = 0.1
        self.cfl = 0.5
        self.dtmax = 5.
        self.npx = 1
        self.npy = 1
        for k, v in kw.items():
            setattr(self, k, v)


# ------------------------------------------------------------------ grid
class Grid(object):
    """core/grid.py:12-140 for one rank (ishift = jshift = 0)."""

    def __init__(self, param):
        self.nx, self.ny = int(param.nx), int(param.ny)
        self.Lx, self.Ly = param.Lx, param.Ly
        self.nh = nh = param.nh
        self.geometry = param.geometry
        self.nxl = self.nx + 2 * nh
        self.nyl = self.ny + 2 * nh
        self.dx = self.Lx / self.nx
        self.dy = self.Ly / self.ny
        self.x1d = (np.arange(self.nxl) + 0.5 - nh + 0) * self.dx
        self.y1d = (np.arange(self.nyl) + 0.5 - nh + 0) * self.dy
        self.xr, self.yr = np.meshgrid(self.x1d, self.y1d)
        self.set_msk()

    def set_msk(self):
        nh = self.nh
        self.msk = np.ones((self.nyl, self.nxl), dtype=np.int8)
        if self.geometry in ['xperio', 'xchannel', 'closed', 'disc']:
            self.msk[-nh:, :] = 0
            self.msk[:nh, :] = 0
        if self.geometry in ['yperio', 'ychannel', 'closed', 'disc']:
            self.msk[:, -nh:] = 0
            self.msk[:, :nh] = 0
        if self.geometry == 'disc':
            r = np.sqrt((self.xr / self.Lx - 0.5)**2 + (self.yr / self.Ly - 0.5)**2)
            self.msk[r >= 0.5] = 0
        # the no-slip walls are those of the geometry, before the user edits
        # the mask (core/grid.py:101)
        self.msknoslip = self.msk.copy()
        self.finalize_msk()

    def finalize_msk(self):
        msk = self.msk
        self.area = self.domain_integration(msk)
        x0 = self.domain_integration(self.xr * msk) / self.area
        y0 = self.domain_integration(self.yr * msk) / self.area
        self.xr0 = (self.xr - x0) * msk
        self.yr0 = (self.yr - y0) * msk

    def domain_integration(self, z2d):
        nh = self.nh
        return np.sum(z2d[nh:-nh, nh:-nh]) * 1.


# ------------------------------------------------------------------ gmg
def gridinfo(n, m, dx, dy, n0=4):
    """core/gmg/level.py:24-117 for one rank, plus the even-coarsening stop."""
    info = []
    lev = 0
    while True:
        if lev > 0:
            n = n // 2
            m = m // 2
            dx = dx * 2
            dy = dy * 2
        last = (n <= n0) or (m <= n0) or (n % 2 == 1) or (m % 2 == 1)
        info.append({'n': n, 'm': m, 'dx': dx, 'dy': dy, 'lev': lev})
        lev += 1
        if last:
            break
        if lev > 20:
            raise RuntimeError('too many levels')
    return info


class Level(object):
    """core/gmg/level.py:120-442 (one rank, halo method 0)."""

    def __init__(self, info, nh, omega, hydroepsilon, relaxation):
        self.n, self.m = info['n'], info['m']
        self.dx, self.dy = info['dx'], info['dy']
        self.lev = info['lev']
        self.nh = nh
        self.nv = self.n + 2 * nh
        self.mv = self.m + 2 * nh
        self.omega = omega
        self.hydroepsilon = hydroepsilon
        self.relaxation = relaxation
        if self.hydroepsilon * self.dy / self.dx <= .2:
            self.relaxation = 'tridiagonal'
        self.msk = np.ones((self.mv, self.nv), dtype=np.int8)

    def fill(self, x):
        K.fillhalo(x, self.nh)

    def set_finest(self, mskf):
        self.msk = mskf
        self.compute_A_atfinest()
        self.yo = np.zeros((3, self.nv))

    def set_coarser(self, prev):
        mskf = prev.msk * 1.0
        coef = np.ones((self.mv, self.nv))
        K.restrict(self.msk, mskf, self.nh, coef)
        self.fill(coef)
        self.msk[coef <= 0.5] = 0
        A = K.coarsenmatrix(prev.A, prev.msk, self.msk, prev.nh)
        for k in range(9):
            # each plane's halo is filled through a strided view of A, as
            # core/gmg/level.py:323-327 passes it
            c = A[:, :, k].squeeze()
            self.fill(c)
            A[:, :, k] = c
        self.A = A
        self.yo = np.zeros((3, self.nv))

    def compute_A_atfinest(self):
        bx = self.dy / self.dx * self.hydroepsilon
        by = self.dx / self.dy
        a = -2 * (bx + by)
        c = 0.
        stencil = np.array([[c, by, c], [bx, a, bx], [c, by, c]]).astype(float)
        if (self.dx == self.dy) and (self.hydroepsilon == 1):
            a, b, c = -6. / 2, 1. / 2, 0.5 / 2
            stencil = np.array([[c, b, c], [b, a, b], [c, b, c]]).astype(float)
        A = np.zeros((self.mv, self.nv, 9))
        I, J = np.meshgrid(np.arange(self.nv - 2) + 1, np.arange(self.mv - 2) + 1)
        coef = 1. / (self.dx * self.dy)
        for k in range(9):
            Acoef = np.zeros((self.mv, self.nv))
            i, j = (k % 3) - 1, (k // 3) - 1
            Acoef[J, I] = stencil[j + 1, i + 1] * coef * self.msk[J + j, I + i] * self.msk[J, I]
            self.fill(Acoef)
            A[:, :, k] = Acoef
        self.A = A

    def ninetofive(self):
        self.A = self.A[:, :, :5]

    def smooth(self, x, b, nite):
        if self.relaxation == 'tridiagonal':
            nite *= 3
        for k in range(nite):
            if self.relaxation == 'tridiagonal':
                K.smoothtridiag(self.msk, self.A, x, b)
            else:
                K.smoothtwicewitha(self.msk, self.A, x, b, self.omega, self.yo)
            self.fill(x)

    def residual(self, x, b, r):
        K.computeresidualwitha(self.msk, self.A, x, b, r)
        self.fill(r)

    def norm(self, x):
        local_sum = K.computenorm(self.msk, x, self.nh)
        return np.sqrt(local_sum / 1.0)


def coarsetofine(coarse, fine, x, y):
    K.interpolate(fine.msk, coarse.msk, x, fine.nh, y)
    if coarse.nh <= 2:
        fine.fill(y)


def finetocoarse(fine, coarse, x, y):
    K.restrict(coarse.msk, x, coarse.nh, y)
    coarse.fill(y)


class Gmg(object):
    """core/gmg/hierarchy.py:21-218 for one rank."""

    def __init__(self, pp, mskp):
        info = gridinfo(pp['n'], pp['m'], pp['dx'], pp['dy'], pp.get('n0', 4))
        self.nlevs = len(info)
        self.npre = 1
        self.npost = 1
        self.nvcyc = 1
        self.ndeepest = 16
        # the QG hierarchy ignores hydroepsilon (core/gmg/level.py:94-103,138-141)
        he = 1. if pp.get('qgoperator', False) else pp.get('hydroepsilon', 1.)
        self.grid = [Level(inf, pp['nh'], pp['omega'], he,
                           pp.get('relaxation', 'default')) for inf in info]
        msk = mskp.astype(np.int8)
        self.x, self.b, self.r = [], [], []
        for lev in range(self.nlevs):
            g = self.grid[lev]
            if lev == 0:
                g.set_finest(msk)
            else:
                g.set_coarser(self.grid[lev - 1])
            self.x.append(np.zeros((g.mv, g.nv)))
            self.b.append(np.zeros((g.mv, g.nv)))
            self.r.append(np.zeros((g.mv, g.nv)))
        for g in self.grid:
            g.ninetofive()
        if pp.get('qgoperator', False):
            for g in self.grid:
                d = g.A[:, :, 4]
                g.A[d != 0., 4] -= 1. / (pp['Rd']**2)

    def Vcycle(self, lev1):
        deepest = self.nlevs - 1
        for lev in range(lev1, deepest):
            if lev > lev1:
                self.x[lev][:, :] = 0.
            self.grid[lev].smooth(self.x[lev], self.b[lev], self.npre)
            self.grid[lev].residual(self.x[lev], self.b[lev], self.r[lev])
            finetocoarse(self.grid[lev], self.grid[lev + 1], self.r[lev], self.b[lev + 1])
        lev = deepest
        self.x[lev][:, :] = 0.
        self.grid[lev].smooth(self.x[lev], self.b[lev], self.ndeepest)
        for lev in range(deepest - 1, lev1 - 1, -1):
            coarsetofine(self.grid[lev + 1], self.grid[lev], self.x[lev + 1], self.r[lev])
            self.x[lev] += self.r[lev]
            self.grid[lev].smooth(self.x[lev], self.b[lev], self.npost)

    def Fcycle(self, lev1):
        deepest = self.nlevs - 1
        for lev in range(lev1, deepest):
            finetocoarse(self.grid[lev], self.grid[lev + 1], self.b[lev], self.b[lev + 1])
        lev = deepest
        self.x[lev][:, :] = 0.
        self.grid[lev].smooth(self.x[lev], self.b[lev], self.ndeepest)
        for lev in range(deepest - 1, lev1 - 1, -1):
            coarsetofine(self.grid[lev + 1], self.grid[lev], self.x[lev + 1], self.x[lev])
            for k in range(self.nvcyc):
                self.Vcycle(lev)

    def solve(self, x, b, param):
        g = self.grid[0]
        g.residual(x, b, self.b[0])
        normeb = g.norm(b)
        if normeb > 0:
            res0 = (g.norm(self.b[0]) / normeb)
        else:
            return 0, 0.
        res = res0
        nite = 0
        nite_diverge = 0
        while (nite < param['maxite']) and (res0 > param['tol']):
            self.Fcycle(0)
            x += self.x[0]
            g.residual(x, b, self.b[0])
            res = (g.norm(self.b[0]) / normeb)
            conv = res0 / res
            res0 = res
            nite += 1
            if conv < 1:
                nite_diverge += 1
            if nite_diverge > 4:
                raise RuntimeError('solver is not converging')
        return nite, res

    def twoVcycle(self, x, b, param=None):
        g = self.grid[0]
        self.x[0][:, :] = x
        self.b[0][:, :] = b
        for k in range(2):
            g.residual(self.x[0], self.b[0], self.r[0])
            self.Vcycle(0)
        x[:, :] = self.x[0]
        return 1, 0.


# ------------------------------------------------------------------ operators
class Operators(object):
    """core/operators.py:12-155, 214-236, 292-314, 421-498 (no islands)."""

    def __init__(self, param, grid, varname_list, tracer_list, whosetspsi,
                 qgoperator=False):
        self.varname_list = varname_list
        self.tracer_list = tracer_list
        self.whosetspsi = whosetspsi
        self.nh = param.nh
        self.order = param.order
        self.gravity = param.gravity
        self.geometry = param.geometry
        self.Kdiff = param.Kdiff
        self.msk = grid.msk
        self.nxl, self.nyl = grid.nxl, grid.nyl
        self.dx, self.dy = grid.dx, grid.dy
        self.grid = grid
        self.area = grid.area
        self.work = np.zeros((self.nyl, self.nxl))
        pp = {'nh': param.nh, 'n': param.nx, 'm': param.ny, 'omega': 8. / 9.,
              'dx': grid.dx, 'dy': grid.dy, 'n0': 4,
              'hydroepsilon': param.hydroepsilon, 'relaxation': param.relaxation}
        mskr = self.msk * 1.
        K.celltocorner(mskr, self.work)
        self.work[self.work < 1.] = 0.
        self.mskp = self.msk * 0
        self.mskp[self.work == 1.] = 1
        if qgoperator:
            pp['qgoperator'] = True
            pp['Rd'] = param.Rd
        self.gmg = Gmg(pp, self.work)
        self.fill_halo = self.gmg.grid[0].fill
        self.cst = np.zeros(5,)
        if self.order % 2 == 0:
            self.fortran_adv = K.adv_centered
            self.cst[0] = grid.dx
            self.cst[1] = grid.dy
            self.cst[2] = 0.05
            self.cst[3] = 0
            self.cst[4] = 0
        else:
            self.fortran_adv = K.adv_upwind
            self.cst[0] = grid.dx
            self.cst[1] = grid.dy
            self.cst[2] = 0.05
            self.cst[3] = 0
            self.cst[4] = param.aparab
        lst = ['minmax', 'parabolic']
        self.fs_method = lst.index(param.flux_splitting_method) \
            if param.flux_splitting_method in lst else 1
        self.last_solve = (0, 0.)
        self.msknoslip = grid.msknoslip
        self.set_boundary_msk()
        # the thermal-wind coefficients every model computes at set-up
        # (core/operators.py:132-145); unused by these models, kept so that the
        # kernel calls are the reference's, call for call
        for a, b in (((slice(1, -1), slice(2, None)), (slice(1, -1), slice(0, -2))),
                     ((slice(2, None), slice(1, -1)), (slice(0, -2), slice(1, -1)))):
            coef = 0. * np.zeros_like(self.msk)
            coef[1:-1, 1:-1] = self.msk[a] + self.msk[b]
            coef[coef < 2] = 0.
            coef[coef == 2] = 0.5
            self.fill_halo(coef)

    def set_boundary_msk(self):
        """core/operators.py:157-184: the cells along the solid boundary."""
        msk = self.msknoslip
        z = (np.roll(msk, -1, axis=1) + np.roll(msk, -1, axis=0)
             + np.roll(msk, +1, axis=1) + np.roll(msk, +1, axis=0) - 4 * msk)
        z = z * msk
        self.mskbc = self.msk * 0
        self.mskbc[z < 0] = 1
        self.mskbc *= self.msknoslip
        self.fill_halo(self.mskbc)
        self.bcarea = self.grid.domain_integration(self.mskbc)

    def rhs_noslip(self, x, source):
        """core/operators.py:245-290 (without enforce_momentum): the vorticity
        source along the walls that cancels the tangential velocity."""
        ip = self.varname_list.index('psi')
        iw = self.varname_list.index(self.whosetspsi)
        K.cornertocell(x[ip], self.work)
        K.computenoslipsourceterm(self.msknoslip, x[ip], self.work, self.dx, self.dy,
                                  self.nh)
        source[:, :] = self.work
        meansource = self.grid.domain_integration(source) / self.bcarea
        source -= meansource * self.mskbc
        self.fill_halo(source)
        x[iw] -= source

    def rhs_adv(self, x, t, dxdt):
        iu = self.varname_list.index('u')
        iv = self.varname_list.index('v')
        u = x[iu]
        v = x[iv]
        for trac in self.tracer_list:
            ik = self.varname_list.index(trac)
            y = dxdt[ik]
            self.fortran_adv(self.msk, x[ik], y, u, v, self.cst, self.nh,
                             self.fs_method, self.order)
            self.fill_halo(y)
            dxdt[ik][:, :] = y

    def rhs_diffusion(self, x, t, dxdt, coef=1.):
        for trac in self.tracer_list:
            ik = self.varname_list.index(trac)
            y = dxdt[ik]
            K.add_diffusion(self.msk, x[ik], self.dx, self.nh, coef * self.Kdiff, y)
            self.fill_halo(y)
            dxdt[ik] = y

    def rhs_torque(self, x, t, dxdt):
        ib = self.varname_list.index('buoyancy')
        iw = self.varname_list.index('vorticity')
        y = dxdt[iw]
        b = x[ib]
        y *= self.msk
        K.add_torque(self.msk, b, self.dx, self.nh, self.gravity, y)
        self.fill_halo(y)
        dxdt[iw][:, :] = y

    def invert_vorticity(self, x, flag='full', island=False):
        iu = self.varname_list.index('u')
        iv = self.varname_list.index('v')
        ip = self.varname_list.index('psi')
        iw = self.varname_list.index(self.whosetspsi)
        u = x[iu]
        v = x[iv]
        psi = x[ip]
        K.celltocorner(x[iw], self.work)
        if island:  # core/operators.py:442-444
            self.work[:, :] -= self.rhsp
        if flag == 'fast':
            self.gmg.twoVcycle(psi, self.work, {'maxite': 1, 'tol': 1e-6})
        else:
            self.last_solve = self.gmg.solve(psi, self.work,
                                             {'maxite': 4, 'tol': 1e-11})
            if self.geometry == 'perio':
                psim = self.grid.domain_integration(psi) / self.area
                psi -= psim
        psi = psi * self.mskp
        if island:  # core/operators.py:482-486
            psi += self.psi
        K.computeorthogradient(self.msk, psi, self.dx, self.dy, self.nh, u, v)
        x[iu] = u
        x[iv] = v
        x[ip] = psi


# ------------------------------------------------------------------ time
class Timescheme(object):
    """core/timescheme.py:6-201"""

    def __init__(self, timestepping, x):
        self.timestepping = timestepping
        coefondt = {'EF': 1., 'LF': 1., 'Heun': 2., 'AB2': 1., 'AB3': 1.,
                    'LFAM3': 1., 'RK3_SSP': 1.5, 'RK3': 1., 'RK4_LS': 1.}
        self.dtcoef = coefondt[timestepping]
        self.asselin_cst = 0.1
        self.ab2_epsilon = 0.1
        self.x = np.zeros_like(x)
        self.dx0 = np.zeros_like(x)
        self.dx1 = np.zeros_like(x)
        if timestepping in ['RK3_SSP', 'AB3', 'RK3']:
            self.dx2 = np.zeros_like(x)
        if timestepping in ['LF', 'LFAM3']:
            self.xb = np.zeros_like(x)
        self.first = True
        self.second = True
        self.kstage = 0

    def set(self, rhs):
        self.rhs = rhs
        self.forward = getattr(self, {'EF': 'EulerForward', 'LF': 'LeapFrog'}.get(
            self.timestepping, self.timestepping))
        self.kforcing = {'RK4_LS': 3, 'RK3_SSP': 2, 'Heun': 1, 'LFAM3': 1}.get(
            self.timestepping, 0)

    def EulerForward(self, x, t, dt):
        self.rhs(x, t, self.dx0)
        x += dt * self.dx0

    def AB2(self, x, t, dt):
        self.rhs(x, t, self.dx0)
        if self.first:
            x += dt * self.dx0
            self.first = False
        else:
            x += ((1.5 + self.ab2_epsilon) * dt) * self.dx0 \
                - ((0.5 + self.ab2_epsilon) * dt) * self.dx1
        self.dx1[:] = self.dx0

    def AB3(self, x, t, dt):
        self.rhs(x, t, self.dx0)
        if self.first:
            x += dt * self.dx0
            self.first = False
        elif self.second:
            x += (1.5 * dt) * self.dx0 - (0.5 * dt) * self.dx1
            self.second = False
        else:
            x += (23 * dt / 12.) * self.dx0 \
                - (16 * dt / 12.) * self.dx1 + (5 * dt / 12.) * self.dx2
        self.dx2[:] = self.dx1
        self.dx1[:] = self.dx0

    def LeapFrog(self, x, t, dt):
        self.x[:] = x
        self.rhs(x, t, self.dx0)
        if self.first:
            x += dt * self.dx0
            self.first = False
        else:
            x[:] = self.xb + (2 * dt) * self.dx0
            self.x += self.asselin_cst * (x + self.xb - 2 * self.x)
        self.xb[:] = self.x

    def LFAM3(self, x, t, dt):
        self.x[:] = x
        self.kstage = 0
        self.rhs(x, t, self.dx0)
        if self.first:
            x += dt * self.dx0
            self.first = False
        else:
            x[:] = self.xb + (2 * dt) * self.dx0
            x[:] = (1. / 12.) * (5. * x + 8. * self.x - self.xb)
            self.kstage = 1
            self.rhs(x, t + dt * .5, self.dx0)
            x[:] = self.x + dt * self.dx0
        self.xb[:] = self.x

    def Heun(self, x, t, dt):
        self.kstage = 0
        self.rhs(x, t, self.dx0)
        self.x = x + dt * self.dx0
        self.kstage = 1
        self.rhs(self.x, t + dt, self.dx1)
        x += (0.5 * dt) * (self.dx0 + self.dx1)

    def RK3(self, x, t, dt):
        self.kstage = 0
        self.rhs(x, t, self.dx0)
        self.x = x + (dt / 3.) * self.dx0
        self.kstage = 1
        self.rhs(self.x, t + dt / 3., self.dx1)
        self.x = x + (0.5 * dt) * self.dx1
        self.kstage = 2
        self.rhs(self.x, t + 0.5 * dt, self.dx2)
        x += dt * self.dx2

    def RK3_SSP(self, x, t, dt):
        self.kstage = 0
        self.rhs(x, t, self.dx0)
        self.x = x + dt * self.dx0
        self.kstage = 1
        self.rhs(self.x, t + dt, self.dx1)
        self.x = x + (0.25 * dt) * (self.dx0 + self.dx1)
        self.kstage = 2
        self.rhs(self.x, t + 0.5 * dt, self.dx2)
        x += (dt / 6.) * (self.dx0 + self.dx1 + 4 * self.dx2)

    def RK4_LS(self, x, t, dt):
        self.kstage = 0
        self.rhs(x, t, self.dx0)
        self.x = x + (0.25 * dt) * self.dx0
        self.kstage = 1
        self.rhs(self.x, t + dt * 0.25, self.dx0)
        self.x = x + (dt / 3.) * self.dx0
        self.kstage = 2
        self.rhs(self.x, t + dt / 3., self.dx0)
        self.x = x + (dt / 2.) * self.dx0
        self.kstage = 3
        self.rhs(self.x, t + 0.5 * dt, self.dx0)
        x += dt * self.dx0


# ------------------------------------------------------------------ models
class _Model(object):
    varname_list = []
    tracer_list = []
    whosetspsi = 'vorticity'
    qgoperator = False

    def __init__(self, param, grid=None):
        self.param = param
        self.grid = grid if grid is not None else Grid(param)
        g = self.grid
        self.msk, self.nh, self.area = g.msk, g.nh, g.area
        self.xr, self.yr = g.xr, g.yr
        self.state = np.zeros((len(self.varname_list), g.nyl, g.nxl))
        self.ope = Operators(param, g, self.varname_list, self.tracer_list,
                             self.whosetspsi, qgoperator=self.qgoperator)
        self.tscheme = Timescheme(param.timestepping, self.state)
        self.tscheme.set(self.dynamics)
        self.diags = {}
        # islands with a prescribed streamfunction (core/fluid2d.py:110-113):
        # set_islands gives the Island's rhsp and psi (core/island.py:21-47)
        self.isisland = False

    def set_islands(self, rhsp, psi):
        self.ope.rhsp = np.array(rhsp, dtype=float)
        self.ope.psi = np.array(psi, dtype=float)
        self.isisland = True

    def get(self, name):
        return self.state[self.varname_list.index(name)]


class Euler(_Model):
    """core/euler.py:12-223 (no forcing, sponge, dye, islands)."""
    varname_list = ['vorticity', 'psi', 'u', 'v', 'source']
    tracer_list = ['vorticity']

    def step(self, t, dt):
        self.tscheme.forward(self.state, t, dt)
        if self.param.noslip:  # core/euler.py:109-113, 171-179
            source = self.get('source')
            self.ope.rhs_noslip(self.state, source)
            self.ope.invert_vorticity(self.state, flag='fast', island=self.isisland)
            source /= dt
        self.set_psi_from_vorticity()

    def dynamics(self, x, t, dxdt):
        self.ope.rhs_adv(x, t, dxdt)
        if self.tscheme.kstage == self.tscheme.kforcing:
            if self.param.diffusion:
                self.ope.rhs_diffusion(x, t, dxdt)
                self.ope.invert_vorticity(dxdt, flag='fast')
        else:
            self.ope.invert_vorticity(dxdt, flag='fast')

    def set_psi_from_vorticity(self):
        self.ope.invert_vorticity(self.state, island=self.isisland)

    def diagnostics(self, t=0.):
        u, v = self.get('u'), self.get('v')
        trac, psi, source = self.get('vorticity'), self.get('psi'), self.get('source')
        ke, maxu = K.computekemaxu(self.msk, u, v, self.nh)
        z, z2 = K.computesumandnorm(self.msk, trac, self.nh)
        px = K.computedotprod(self.msk, trac, self.xr, self.nh)
        py = K.computedotprod(self.msk, trac, self.yr, self.nh)
        angmom = K.computesum(self.msk, psi, self.nh)
        sce = K.computedotprod(self.msk, trac, source, self.nh)
        cst = np.array([maxu, ke, z, z2, px, py, angmom, sce], dtype=float)
        self.diags['maxspeed'] = cst[0]
        self.diags['ke'] = cst[1] / self.area
        self.diags['vorticity'] = cst[2] / self.area
        self.diags['enstrophy'] = 0.5 * cst[3] / self.area
        self.diags['px'] = cst[4] / self.area
        self.diags['py'] = cst[5] / self.area
        self.diags['angmom'] = cst[6] / self.area
        self.diags['source'] = cst[7] / self.area
        return self.diags


class Boussinesq(_Model):
    """core/boussinesq.py:10-153 (no forcing, islands)."""
    varname_list = ['vorticity', 'psi', 'u', 'v', 'buoyancy', 'banom']
    tracer_list = ['vorticity', 'buoyancy']

    def __init__(self, param, grid=None):
        _Model.__init__(self, param, grid)
        self.bref = self.get('buoyancy').copy()
        self.source = np.zeros(self.state.shape[1:])

    def step(self, t, dt):
        self.tscheme.forward(self.state, t, dt)
        if self.param.noslip:  # core/boussinesq.py:93-94, 116-118
            self.ope.rhs_noslip(self.state, self.source)
            self.ope.invert_vorticity(self.state, flag='fast', island=self.isisland)
        banom = self.get('banom')
        banom[:, :] = self.get('buoyancy') - self.bref

    def dynamics(self, x, t, dxdt):
        self.ope.rhs_adv(x, t, dxdt)
        self.ope.rhs_torque(x, t, dxdt)
        if self.tscheme.kstage == self.tscheme.kforcing:
            coef = self.tscheme.dtcoef
            if self.param.diffusion:
                self.ope.rhs_diffusion(x, t, dxdt, coef=coef)
        self.ope.invert_vorticity(dxdt, flag='fast')

    def set_psi_from_vorticity(self):
        self.ope.invert_vorticity(self.state, island=self.isisland)

    def diagnostics(self, t=0.):
        nh = self.nh
        u, v = self.get('u'), self.get('v')
        vort, buoy = self.get('vorticity'), self.get('buoyancy')
        ke, maxu = K.computekemaxu(self.msk, u, v, nh)
        z, z2 = K.computesumandnorm(self.msk, vort, nh)
        b, b2 = K.computesumandnorm(self.msk, buoy, nh)
        pe = - self.param.gravity * K.computesum(self.msk, buoy * self.yr, nh)
        cst = np.array([maxu, ke, z, z2, pe, b, b2], dtype=float)
        self.diags['maxspeed'] = cst[0]
        self.diags['ke'] = cst[1] / self.area
        self.diags['pe'] = cst[4] / self.area
        self.diags['energy'] = (cst[1] + cst[4]) / self.area
        self.diags['vorticity'] = cst[2] / self.area
        self.diags['enstrophy'] = 0.5 * cst[3] / self.area
        self.diags['buoyancy'] = cst[5] / self.area
        self.diags['brms'] = np.sqrt(cst[6] / self.area - (cst[5] / self.area)**2)
        return self.diags


class QG(_Model):
    """core/quasigeostrophic.py:11-218 (no forcing, noslip, bottom torque,
    ageostrophic diagnosis)."""
    varname_list = ['pv', 'psi', 'u', 'v', 'pvanom', 'vorticity']
    tracer_list = ['pv']
    whosetspsi = 'pvanom'
    qgoperator = True

    def __init__(self, param, grid=None):
        _Model.__init__(self, param, grid)
        g = self.grid
        self.pvback = param.beta * (g.yr - g.Ly * .5) * g.msk
        self.ipva = self.varname_list.index('pvanom')
        self.ipv = self.varname_list.index('pv')
        self.ivor = self.varname_list.index('vorticity')
        self.ipsi = self.varname_list.index('psi')
        self.Rd = param.Rd
        self.source = np.zeros(self.state.shape[1:])

    def step(self, t, dt):
        self.tscheme.forward(self.state, t, dt)
        if self.param.noslip:  # core/quasigeostrophic.py:112-114, 171-175
            self.ope.rhs_noslip(self.state, self.source)
            self.ope.invert_vorticity(self.state, flag='fast', island=self.isisland)
        self.set_psi_from_pv()
        self.state[self.ipva] = self.state[self.ipv] - self.pvback
        self.state[self.ivor] = (self.state[self.ipva]
                                 - (self.Rd**-2) * self.state[self.ipsi])

    def dynamics(self, x, t, dxdt):
        dxdt[:] = 0.
        self.ope.rhs_adv(x, t, dxdt)
        if self.tscheme.kstage == self.tscheme.kforcing:
            if self.param.diffusion:
                self.ope.rhs_diffusion(x, t, dxdt)
        else:
            dxdt[self.ipva] = dxdt[self.ipv]
            self.ope.invert_vorticity(dxdt, flag='fast', island=self.isisland)

    def set_psi_from_pv(self):
        state = self.state
        state[self.ipva] = state[self.ipv] - self.pvback
        self.ope.invert_vorticity(self.state, flag='full', island=self.isisland)

    def diagnostics(self, t=0.):
        u, v = self.get('u'), self.get('v')
        trac, psi = self.get('pv'), self.get('psi')
        K.cornertocell(psi, self.ope.work)
        psim, psi2 = K.computesumandnorm(self.msk, self.ope.work, self.nh)
        ape = 0.5 * psi2 / self.Rd**2
        ke, maxu = K.computekemaxu(self.msk, u, v, self.nh)
        z, z2 = K.computesumandnorm(self.msk, trac, self.nh)
        cst = np.array([maxu, ke, z, z2, ape], dtype=float)
        self.diags['maxspeed'] = cst[0]
        self.diags['ke'] = cst[1] / self.area
        self.diags['pv'] = cst[2] / self.area
        self.diags['pv2'] = 0.5 * cst[3] / self.area
        self.diags['ape'] = cst[4] / self.area
        self.diags['energy'] = (cst[1] + cst[4]) / self.area
        return self.diags


MODELS = {'euler': Euler, 'boussinesq': Boussinesq, 'quasigeostrophic': QG}


def set_dt(model, param, dt0):
    """core/fluid2d.py:376-397; returns dt and sets cst[3] = maxspeed."""
    maxspeed = model.diags['maxspeed']
    if param.adaptable_dt and maxspeed != 0:
        dt = param.cfl * min(model.grid.dx, model.grid.dy) / maxspeed
        if dt > param.dtmax:
            dt = param.dtmax
    else:
        dt = dt0
    model.ope.cst[3] = maxspeed
    return dt


def run(model, param, nsteps, dt0, t=0., callback=None):
    """The core of Fluid2d.loop (core/fluid2d.py:235-314) without I/O."""
    if not model.diags:
        model.diagnostics(t)
    for kt in range(nsteps):
        dt = set_dt(model, param, dt0)
        model.step(t, dt)
        t += dt
        model.diagnostics(t)
        if callback is not None:
            callback(kt + 1, t, model)
    return t


class Fluxes(object):
    """core/fluxes.py:6-213: the reversible and irreversible parts of the
    advective fluxes, from one step forward and one step back in time of an
    extended state (the model state, the cell-centred velocities uc, vc and
    the edge fluxes of every tracer, all advanced by the model's time scheme).
    It shares the model's Operators (multigrid, work array, cst[3])."""

    def __init__(self, model):
        p = model.param
        self.model, self.ope = model, model.ope
        self.varname_list = list(model.varname_list) + ['uc', 'vc']
        self.tracer_list = list(model.tracer_list) + ['uc', 'vc']
        self.nvarstate = len(self.varname_list)
        self.flx_list = ['flx_%s_%s' % (v, d) for v in self.tracer_list for d in 'xy']
        self.fullflx_list = ['%s_%s_%s' % (r, d, v) for r in ('rev', 'irr')
                             for v in self.tracer_list for d in 'xy']
        nyl, nxl = model.state.shape[1:]
        size = (self.nvarstate + len(self.flx_list), nyl, nxl)
        self.x = np.zeros(size)
        self.xe = np.zeros((self.nvarstate, nyl, nxl))
        self.xwork = np.zeros(size)
        self.flx = np.zeros((len(self.fullflx_list), nyl, nxl))
        self.fortran_adv = K.adv_centered_flux if p.order % 2 == 0 else K.adv_upwind_flux
        self.cst = np.array([model.grid.dx, model.grid.dy, 0.05, 0., p.aparab])
        self.order = p.order
        self.fs_method = self.ope.fs_method
        self.nh = model.nh
        self.msk = model.msk
        self.boussinesq = isinstance(model, Boussinesq)
        self.tscheme = Timescheme(p.timestepping, self.x)
        self.tscheme.set(self.advection)

    def diag_fluxes(self, x, t, dt):
        vl = self.varname_list
        iu, iv, ip, iw = vl.index('u'), vl.index('v'), vl.index('psi'), vl.index('vorticity')
        ns = self.nvarstate
        self.xe[:ns - 2, :, :] = x
        y = 0.5 * (x[iu] + np.roll(x[iu], 1, axis=1))
        self.ope.fill_halo(y)
        self.xe[ns - 2, :, :] = y
        y = 0.5 * (x[iv] + np.roll(x[iv], 1, axis=0))
        self.ope.fill_halo(y)
        self.xe[ns - 1, :, :] = y
        self.x[:ns, :, :] = self.xe
        self.x[ns:, :, :] = 0.
        self.tscheme.forward(self.x, t, dt)
        self.xwork[:, :, :] = self.x
        self.x[:ns, :, :] = self.xe
        for k in (iu, iv, ip, iw, ns - 2, ns - 1):
            self.x[k] *= -1
        self.x[ns:, :, :] = 0.
        self.tscheme.forward(self.x, t + dt, -dt)
        cff = 0.5 / dt
        nflx = len(self.flx_list)
        for k in range(nflx):
            l = ns + k
            j = nflx + k
            sign = -1 if (k < 2 or k >= nflx - 4) else 1
            self.flx[k, :, :] = cff * (self.xwork[l] + sign * self.x[l])
            self.flx[j, :, :] = cff * (self.xwork[l] - sign * self.x[l])

    def advection(self, x, t, dxdt):
        self.rhs_adv(x, t, dxdt)
        if self.boussinesq:
            self.ope.rhs_torque(x, t, dxdt)
        self.ope.invert_vorticity(dxdt, flag='fast')

    def rhs_adv(self, x, t, dxdt):
        vl = self.varname_list
        u, v = x[vl.index('u')], x[vl.index('v')]
        self.cst[3] = self.ope.cst[3]
        for itrac, trac in enumerate(self.tracer_list):
            ik = vl.index(trac)
            y = dxdt[ik]
            ix = self.nvarstate + itrac * 2
            iy = ix + 1
            xf, yf = dxdt[ix], dxdt[iy]
            self.fortran_adv(self.msk, x[ik], y, u, v, xf, yf, self.cst, self.nh,
                             self.fs_method, self.order)
            self.ope.fill_halo(y)
            self.ope.fill_halo(xf)
            self.ope.fill_halo(yf)
            dxdt[ik, :, :] = y
            dxdt[ix, :, :] = xf
            dxdt[iy, :, :] = yf


class History(object):
    """What Output.do (core/output.py:62-94) writes, kept in memory: history
    records (t, kt and the interior of each saved plane in float32, as the
    netCDF 'f' variables of core/output.py:227-243 store them) and diagnostic
    rows (t, kt and every model diagnostic, incl. dkedt and dvdt)."""

    def __init__(self, var_to_save, freq_his, freq_diag, tnexthis=0., tnextdiag=0.,
                 fluxes=None):
        self.var_to_save = list(var_to_save)
        self.freq_his, self.freq_diag = freq_his, freq_diag
        self.tnexthis, self.tnextdiag = tnexthis, tnextdiag
        self.fluxes = fluxes
        self.his = []
        self.diag = []
        self.flx = []

    def do(self, model, t, kt):
        nh = model.nh
        if t >= self.tnextdiag:
            self.tnextdiag += self.freq_diag
            self.diag.append((t, kt, dict(model.diags)))
        if t >= self.tnexthis:
            self.tnexthis += self.freq_his
            self.his.append((t, kt, {v: model.get(v)[nh:-nh, nh:-nh].astype(np.float32)
                                     for v in self.var_to_save}))
            if self.fluxes is not None:  # the 'flx' file (core/output.py:92-93)
                F = self.fluxes
                self.flx.append((t, kt, {v: F.flx[k][nh:-nh, nh:-nh].astype(np.float32)
                                         for k, v in enumerate(F.fullflx_list)}))


def loop(model, param, tend, dt0, out, t=0., kt=0, exacthistime=True,
         rescaledtime='none', max_steps=None):
    """Fluid2d.loop (core/fluid2d.py:190-314): diagnostics and output at the
    start, then set_dt, the exact-history-time adjustment, step, clock,
    diagnostics, dkedt/dvdt, output and the blow-up stop.  Returns (t, kt,
    list of the dt used, stop reason)."""
    ensname = 'pv2' if isinstance(model, QG) else 'enstrophy'
    model.diagnostics(t)
    model.diags['dkedt'] = 0.
    model.diags['dvdt'] = 0.
    if out.fluxes is not None:  # core/fluid2d.py:203-210
        out.fluxes.diag_fluxes(model.state, t, set_dt(model, param, dt0))
    out.do(model, t, kt)
    reduce = 0
    dts = []
    reason = 'tend'
    while t < tend:
        if max_steps is not None and len(dts) >= max_steps:
            reason = 'max_steps'
            break
        dt = set_dt(model, param, dt0)
        if exacthistime and param.adaptable_dt:
            if (t + 8 * dt > out.tnexthis) and (reduce == 0):
                reduce = 8
            if reduce > 0:
                dt = (out.tnexthis - t) / (reduce * 0.95)
                reduce -= 1
            if t + dt > out.tnexthis:
                reduce = 0
                dt = out.tnexthis - t
        model.step(t, dt)
        dts.append(dt)
        if rescaledtime == 'enstrophy':
            t += dt * np.sqrt(model.diags['enstrophy'])
        else:
            t += dt
        kt += 1
        ke_old = model.diags['ke']
        ens_old = model.diags[ensname]
        model.diagnostics(t)
        model.diags['dkedt'] = (model.diags['ke'] - ke_old) / dt
        model.diags['dvdt'] = (model.diags[ensname] - ens_old) / dt
        if out.fluxes is not None and t >= out.tnexthis:  # core/fluid2d.py:291-293
            out.fluxes.diag_fluxes(model.state, t, dt)
        out.do(model, t, kt)
        if model.diags['maxspeed'] > 1e3:
            reason = 'blowup'
            break
    return t, kt, dts, reason


def fixture_param(z):
    """The Param of a tests/golden step fixture (its recorded overrides)."""
    import ast
    prm = ast.literal_eval(str(z["params"][0]))
    kw = {k: v for k, v in prm.items() if k not in ("model", "nx", "ny", "Lx", "Ly",
                                                    "geometry", "gravity")}
    return Param(modelname=prm["model"], nx=prm["nx"], ny=prm["ny"], Lx=prm["Lx"],
                 Ly=prm["Ly"], geometry=prm["geometry"], gravity=prm["gravity"], **kw)


def from_fixture(z, **kw):
    """A model on the initial state of a tests/golden step fixture, as the
    fixture's run had it after its set-up: mask, no-slip walls, islands'
    arrays, the state, the diagnostics (no initial inversion: the state
    already holds its result).  ``kw`` overrides Param attributes (another
    time scheme, ...).  Returns (param, model)."""
    p = fixture_param(z)
    for k, v in kw.items():
        setattr(p, k, v)
    g = Grid(p)
    g.msk = np.array(z["msk"])
    if "msknoslip" in z:
        g.msknoslip = np.array(z["msknoslip"])
    g.finalize_msk()
    M = MODELS[p.modelname](p, grid=g)
    if "rhsp" in z:
        M.set_islands(z["rhsp"], z["psi_island"])
    M.state[...] = z["states"][0]
    M.diagnostics()
    return p, M


def from_workload(wl, **kw):
    """An oracle model for a fluid2d_gb300.workloads dict: mask, fields,
    initial inversion (set_psi_from_vorticity / set_psi_from_pv) and
    diagnostics, as a Fluid2d experiment script sets them up."""
    p = Param(modelname=wl["model"], nx=wl["nx"], ny=wl["ny"], Lx=wl["Lx"], Ly=wl["Ly"],
              geometry=wl["geometry"], gravity=wl.get("gravity", 1.), **kw)
    g = Grid(p)
    g.msk = wl["msk"].copy()
    if "msknoslip" in wl:  # an experiment's own no-slip walls
        g.msknoslip = wl["msknoslip"].copy()
    g.finalize_msk()
    M = MODELS[wl["model"]](p, grid=g)
    if "island_arrays" in wl:  # rhsp, psi of core/island.py
        M.set_islands(*wl["island_arrays"])
    for name, f in wl["fields"].items():
        M.get(name)[:] = f
    if wl["model"] == "quasigeostrophic":
        M.get("pv")[:] += M.pvback
        M.set_psi_from_pv()
    else:
        M.set_psi_from_vorticity()
    M.diagnostics()
    return p, M
