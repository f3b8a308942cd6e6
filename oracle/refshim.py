"""Import the reference's own Python layers over the C oracle kernels.

TEST INFRASTRUCTURE ONLY (used by tests/golden/make_golden.py and by CPU
tests that skip themselves when the reference sources are absent).

The reference's Python (core/operators.py, core/gmg/*.py, core/timescheme.py,
core/euler.py, ...) imports five f2py extension modules that cannot be built
here (no Fortran compiler), plus mpi4py and netCDF4.  ``install(core_dir)``
puts stand-ins for all of them into ``sys.modules``:

* ``fortran_advection``, ``fortran_operators``, ``fortran_diag``,
  ``fortran_fluxes`` and ``gmg.fortran_multigrid`` -> the C oracle, with the
  f2py signatures the reference calls;
* ``mpi4py.MPI`` -> a single-rank communicator (reductions are identities,
  persistent requests are inert -- the reference only uses halo method 0
  when it runs on one rank);
* ``netCDF4`` -> an empty module (only imported, never used on the path);
* ``numpy.NaN`` -> ``numpy.nan`` (removed in numpy 2).

Nothing of the reference is copied; its files are imported from where they
lie, read-only.
"""
import os
import sys
import types

import numpy as np

try:
    from . import oracle as K
except ImportError:
    import oracle as K


class _Comm(object):
    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def allreduce(self, x, op=None):
        return x

    def allgather(self, x):
        return [x]

    def bcast(self, x, root=0):
        return x

    def Barrier(self):
        pass

    def Send_init(self, *a, **k):
        return None

    Recv_init = Ssend_init = Send_init

    def Split(self, *a, **k):
        return self


def _module(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    m.__all__ = list(attrs)
    return m


def install(core_dir):
    """Make ``core_dir`` (the reference's core/) importable over the oracle."""
    if not hasattr(np, 'NaN'):
        np.NaN = np.nan
    mpi = _module('mpi4py.MPI', COMM_WORLD=_Comm(), SUM='sum', MAX='max', MIN='min')
    sys.modules['mpi4py'] = _module('mpi4py', MPI=mpi)
    sys.modules['mpi4py.MPI'] = mpi
    sys.modules['netCDF4'] = _module('netCDF4', Dataset=None)
    sys.modules['fortran_advection'] = _module(
        'fortran_advection', adv_upwind=K.adv_upwind, adv_centered=K.adv_centered)
    sys.modules['fortran_fluxes'] = _module(
        'fortran_fluxes', adv_upwind=K.adv_upwind_flux, adv_centered=K.adv_centered_flux)
    sys.modules['fortran_operators'] = _module(
        'fortran_operators',
        computeorthogradient=K.computeorthogradient, celltocorner=K.celltocorner,
        cornertocell=K.cornertocell, add_diffusion=K.add_diffusion,
        add_torque=K.add_torque, computenoslipsourceterm=K.computenoslipsourceterm)
    sys.modules['fortran_diag'] = _module(
        'fortran_diag',
        computedotprod=K.computedotprod, computemax=K.computemax,
        computesum=K.computesum, computesumandnorm=K.computesumandnorm,
        computenormmaxu=K.computenormmaxu, computekemaxu=K.computekemaxu,
        computekemaxuv=K.computekemaxuv, computekewithpsi=K.computekewithpsi)
    sys.modules['gmg.fortran_multigrid'] = _module(
        'gmg.fortran_multigrid',
        smoothtwicewitha=K.smoothtwicewitha, smoothoncewitha=K.smoothoncewitha,
        smoothtridiag=K.smoothtridiag, computeresidualwitha=K.computeresidualwitha,
        fillhalo=K.fillhalo, interpolate=K.interpolate, restrict=K.restrict,
        coarsenmatrix=K.coarsenmatrix, computenorm=K.computenorm,
        computeinner=K.computeinner)
    core_dir = os.path.abspath(core_dir)
    if core_dir not in sys.path:
        sys.path.insert(0, core_dir)
    argv = sys.argv
    sys.argv = [argv[0] if argv else 'x']  # Param() parses sys.argv
    try:
        import gmg  # noqa: F401  (binds gmg.fortran_multigrid)
        import param as ref_param
    finally:
        sys.argv = argv
    return ref_param


def reference_param(core_dir, **overrides):
    """A reference ``Param`` object with the given attribute overrides."""
    ref_param = install(core_dir)
    argv = sys.argv
    sys.argv = [argv[0] if argv else 'x']
    try:
        p = ref_param.Param('default.json')
    finally:
        sys.argv = argv
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


# ------------------------------------------------------------ netCDF recorder
class _RecVar(object):
    """A netCDF variable kept in memory: numpy array, first axis growing when
    it is the unlimited dimension, values cast to the declared type on write
    ('f' float32, 'd' float64, 'i' int32) as netCDF4 does."""

    TYPES = {'f': np.float32, 'd': np.float64, 'i': np.int32}

    def __init__(self, typ, shape, unlimited):
        self.unlimited = unlimited
        self.a = np.zeros(((0,) if unlimited else ()) + tuple(shape), dtype=self.TYPES[typ])

    def __setitem__(self, idx, val):
        if self.unlimited:
            first = idx[0] if isinstance(idx, tuple) else idx
            if isinstance(first, (range, list, np.ndarray)):
                need = max(first) + 1 if len(first) else 0
            elif isinstance(first, slice):
                need = first.stop if first.stop is not None else self.a.shape[0]
            else:
                need = int(first) + 1
            if need > self.a.shape[0]:
                grown = np.zeros((need,) + self.a.shape[1:], dtype=self.a.dtype)
                grown[:self.a.shape[0]] = self.a
                self.a = grown
        if isinstance(idx, range):
            idx = np.asarray(idx)
        self.a[idx] = val

    def __getitem__(self, idx):
        return self.a[idx]


class RecordingDataset(object):
    """Stand-in for netCDF4.Dataset that keeps every file in ``FILES``
    (path -> {'attrs', 'dims', 'variables'}), so that the reference's own
    Output/NcfileIO/Restart code can run and its writes be compared."""

    FILES = {}

    def __init__(self, path, mode='r', format=None):
        if mode == 'w':
            RecordingDataset.FILES[path] = {'attrs': {}, 'dims': {}, 'variables': {}}
        self._f = RecordingDataset.FILES[path]
        self.variables = self._f['variables']

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def close(self):
        pass

    def setncattr(self, k, v):
        self._f['attrs'][k] = v

    def getncattr(self, k):
        return self._f['attrs'][k]

    def createDimension(self, name, size):
        self._f['dims'][name] = size

    def createVariable(self, name, typ, dims):
        if isinstance(dims, str):
            dims = (dims,)
        sizes = [self._f['dims'][d] for d in dims]
        unlimited = bool(dims) and sizes[0] is None
        shape = sizes[1:] if unlimited else sizes
        v = _RecVar(typ, shape, unlimited)
        self._f['variables'][name] = v
        return v


def install_recording_netcdf():
    """Route the reference's ``from netCDF4 import Dataset`` to the recorder."""
    sys.modules['netCDF4'] = _module('netCDF4', Dataset=RecordingDataset)
    return RecordingDataset
