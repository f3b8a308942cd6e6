"""History, diagnostic and restart files of a run, in the reference's layout.

The reference writes NETCDF4 files through the netCDF4 package
(core/output.py:100-246, core/restart.py:120-177).  That package is not
available here, so these writers produce netCDF classic (64-bit offset)
files with scipy.io.netcdf_file: the same dimensions, variable names, types
and global attributes, readable by netCDF4.Dataset, xarray and ncdump.

* ``Output``  -- ``<expdir>/<expname>_his.nc``: dimensions t (unlimited), x, y;
  variables x, y (cell centres, 'f'), msk ('i'), t ('f'), kt ('i') and one
  ('t', 'y', 'x') 'f' variable per saved plane, interior only
  (core/output.py:164-246).  ``<expdir>/<expname>_diag.nc``: t, kt and one
  'f' variable per diagnostic (core/output.py:100-152).
* ``Restart`` -- ``<expdir>/<expname>_<job>_restart_<rank>.nc``: the clock as
  global attributes (tend, t, dt, kt, tnextdiag, tnexthis) and every state
  variable in float64 with its halo, dimensions x = nx+6, y = ny+6
  (core/restart.py:120-177).

The device loop (``engine.Model.loop``) hands records to ``Output`` as the
rings drain; the writers never touch the GPU.
"""
import os

import numpy as np
from scipy.io import netcdf_file

NH = 3


def _attrs_of(param):
    """Global attributes as core/output.py:185-201 stores them: lists and
    dicts skipped, booleans as 0/1, None skipped (netCDF has no null)."""
    items = param.items() if isinstance(param, dict) else vars(param).items()
    out = {}
    for k, v in items:
        if k.startswith("_") or isinstance(v, (list, tuple, dict)) or v is None:
            continue
        if isinstance(v, (bool, np.bool_)):
            v = int(v)
        if isinstance(v, (int, float, str, np.integer, np.floating)):
            out[k] = _typed(v)
    return out


def _typed(v):
    """A netCDF attribute value with an explicit type: scipy would store a
    bare Python float as 32-bit; netCDF4 stores it as a double."""
    if isinstance(v, (bool, np.bool_)):
        return np.int32(int(v))
    if isinstance(v, (int, np.integer)):
        return np.int32(v)
    if isinstance(v, (float, np.floating)):
        return np.float64(v)
    return v


def cell_centres(n, L, nh=NH):
    """core/grid.py:35-41: x1d = (arange(n + 2 nh) + 0.5 - nh) dx, interior part."""
    d = L / n
    return ((np.arange(n + 2 * nh) + 0.5 - nh) * d)[nh:-nh]


class NcfileIO(object):
    """A history-type file: a sequence of 2D snapshots (core/output.py:164-246)."""

    def __init__(self, ncfile, var_to_save, msk, x, y, attrs=None):
        self.ncfile = ncfile
        self.var_to_save = list(var_to_save)
        self.msk = np.asarray(msk)
        self.x, self.y = np.asarray(x), np.asarray(y)
        self.attrs = attrs or {}
        self.khis = 0

    def create(self):
        ny, nx = self.msk.shape[0] - 2 * NH, self.msk.shape[1] - 2 * NH
        with netcdf_file(self.ncfile, "w", version=2) as nc:
            for k, v in self.attrs.items():
                setattr(nc, k, v)
            nc.createDimension("t", None)
            nc.createDimension("x", nx)
            nc.createDimension("y", ny)
            d = nc.createVariable("x", "f", ("x",))
            d.long_name = "coordinate in the x-direction (at cell center)"
            d = nc.createVariable("y", "f", ("y",))
            d.long_name = "coordinate in the y-direction (at cell center)"
            d = nc.createVariable("msk", "i", ("y", "x"))
            d.long_name = "mask at cell center"
            d = nc.createVariable("t", "f", ("t",))
            d.long_name = "model time"
            d = nc.createVariable("kt", "i", ("t",))
            d.long_name = "model iteration"
            for v in self.var_to_save:
                d = nc.createVariable(v, "f", ("t", "y", "x"))
                d.long_name = v
            nc.variables["msk"][:, :] = self.msk[NH:-NH, NH:-NH]
            nc.variables["x"][:] = self.x
            nc.variables["y"][:] = self.y
        self.khis = 0

    def write(self, fields, t, kt):
        """fields: {name: interior (ny, nx) array}, or full (ny+6, nx+6) planes."""
        ny, nx = self.msk.shape[0] - 2 * NH, self.msk.shape[1] - 2 * NH
        with netcdf_file(self.ncfile, "a", mmap=False) as nc:
            nc.variables["t"][self.khis] = t
            nc.variables["kt"][self.khis] = kt
            for v in self.var_to_save:
                a = np.asarray(fields[v])
                if a.shape != (ny, nx):
                    a = a[NH:-NH, NH:-NH]
                nc.variables[v][self.khis, :, :] = a
        self.khis += 1


class Output(object):
    """The history and diagnostic files of one run (core/output.py:8-152)."""

    def __init__(self, expdir, expname, var_to_save, msk, Lx, Ly, param=None,
                 list_diag="all", flxlist=None):
        self.expdir, self.expname = expdir, expname
        os.makedirs(expdir, exist_ok=True)
        self.hisfile = "%s/%s_his.nc" % (expdir, expname)
        self.diagfile = "%s/%s_diag.nc" % (expdir, expname)
        msk = np.asarray(msk)
        ny, nx = msk.shape[0] - 2 * NH, msk.shape[1] - 2 * NH
        attrs = _attrs_of(param or {})
        x, y = cell_centres(nx, Lx), cell_centres(ny, Ly)
        self.nchis = NcfileIO(self.hisfile, var_to_save, msk, x, y, attrs)
        # the flux records (core/output.py:41-47, 75-77): same layout, one
        # variable per rev/irr flux
        self.flxfile = "%s/%s_flx.nc" % (expdir, expname) if flxlist else None
        self.ncflx = NcfileIO(self.flxfile, flxlist, msk, x, y, attrs) if flxlist else None
        self.list_diag = list_diag
        self._his_created = False
        self._flx_created = False
        self.kdiag = 0

    @classmethod
    def for_model(cls, model, expdir, expname, var_to_save=None, param=None, fluxes=False):
        """An Output for an engine.Model (mask and domain from the model);
        fluxes: also the flux file (the model's flux diagnostic names)."""
        d = model.desc
        flxlist = None
        if fluxes:
            if not hasattr(model, "fullflx_list"):
                model.flux_setup()
            flxlist = model.fullflx_list
        return cls(expdir, expname, var_to_save or getattr(model, "var_to_save", ["vorticity"]),
                   model.msk, d.Lx, d.Ly, param=param, flxlist=flxlist)

    def write_his(self, t, kt, fields):
        if not self._his_created:
            self.nchis.create()
            self._his_created = True
        self.nchis.write(fields, t, kt)

    def write_flx(self, t, kt, fields):
        if self.ncflx is None:
            raise ValueError("this Output has no flux file (flxlist not given)")
        if not self._flx_created:
            self.ncflx.create()
            self._flx_created = True
        self.ncflx.write(fields, t, kt)

    def create_diag(self, names):
        with netcdf_file(self.diagfile, "w", version=2) as nc:
            nc.createDimension("t", None)
            d = nc.createVariable("t", "f", ("t",))
            d.long_name = "model time"
            d = nc.createVariable("kt", "i", ("t",))
            d.long_name = "model iteration"
            for v in names:
                d = nc.createVariable(v, "f", ("t",))
                d.long_name = v
        self.kdiag = 0

    def write_diag(self, t, kt, diags):
        if self.list_diag == "all":
            self.list_diag = list(diags)
        if self.kdiag == 0 and not os.path.exists(self.diagfile):
            self.create_diag(self.list_diag)
        with netcdf_file(self.diagfile, "a", mmap=False) as nc:
            nc.variables["t"][self.kdiag] = t
            nc.variables["kt"][self.kdiag] = kt
            for v in self.list_diag:
                nc.variables[v][self.kdiag] = diags[v]
        self.kdiag += 1


class Restart(object):
    """Restart files (core/restart.py:38-177): the state in float64 with its
    halo and the clock as global attributes."""

    def __init__(self, expdir, expname, myrank=0):
        self.expdir, self.expname, self.myrank = expdir, expname, myrank
        self.template = expdir + "/%s_%02i_restart_%03i.nc"

    def path(self, job):
        return self.template % (self.expname, job, self.myrank)

    def last(self):
        """Index of the last restart present (core/restart.py:66-80), or None."""
        import glob
        files = glob.glob(self.expdir + "/%s_*_restart_000.nc" % self.expname)
        if not files:
            return None
        k = 0
        for f in files:
            # the job index sits just before '_restart_' in the file name (the
            # reference searches the whole path, which breaks when a directory
            # name contains 'restart')
            b = os.path.basename(f)
            pos = b.rfind("_restart_")
            k = max(k, int(b[pos - 2:pos]))
        return k

    @staticmethod
    def write(path, tend, t, dt, kt, tnextdiag, tnexthis, state, varname_list):
        state = np.asarray(state)
        with netcdf_file(path, "w", version=2) as nc:
            nc.tend = np.float64(tend)
            nc.t = np.float64(t)
            nc.dt = np.float64(dt)
            nc.kt = np.int32(kt)
            nc.tnextdiag = np.float64(tnextdiag)
            nc.tnexthis = np.float64(tnexthis)
            nc.createDimension("x", state.shape[-1])
            nc.createDimension("y", state.shape[-2])
            for k, v in enumerate(varname_list):
                nc.createVariable(v, "d", ("y", "x"))
                nc.variables[v][:, :] = state[k]

    @staticmethod
    def read(path, varname_list):
        """Returns (clock dict, state array (nvar, ny+6, nx+6))."""
        with netcdf_file(path, "r", mmap=False) as nc:
            a = nc._attributes
            clock = {k: (int(a[k]) if k == "kt" else float(a[k]))
                     for k in ("tend", "t", "dt", "kt", "tnextdiag", "tnexthis")}
            state = np.array([nc.variables[v][:, :].copy() for v in varname_list])
        return clock, state
