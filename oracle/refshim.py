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


# the f2py modules the reference imports by bare name (install.sh:44-46) and,
# for each of their routines, the oracle function that stands in for it
F2PY_NAMES = {
    'fortran_advection': {'adv_upwind': 'adv_upwind', 'adv_centered': 'adv_centered'},
    'fortran_fluxes': {'adv_upwind': 'adv_upwind_flux', 'adv_centered': 'adv_centered_flux'},
    'fortran_operators': {n: n for n in (
        'computeorthogradient', 'celltocorner', 'cornertocell', 'add_diffusion', 'add_torque',
        'computenoslipsourceterm')},
    'fortran_diag': {n: n for n in (
        'computedotprod', 'computemax', 'computesum', 'computesumandnorm', 'computenormmaxu',
        'computekemaxu', 'computekemaxuv', 'computekewithpsi')},
    'gmg.fortran_multigrid': {n: n for n in (
        'smoothtwicewitha', 'smoothoncewitha', 'smoothtridiag', 'computeresidualwitha',
        'fillhalo', 'interpolate', 'restrict', 'coarsenmatrix', 'computenorm',
        'computeinner')},
}


def arg_kind(a):
    """How an argument is passed: dtype, rank and memory order of an array
    (C, F or S for strided), 'scalar' for a number, else the type name."""
    if isinstance(a, np.ndarray):
        order = 'C' if a.flags.c_contiguous else ('F' if a.flags.f_contiguous else 'S')
        return '%s:%dd:%s' % (a.dtype.str, a.ndim, order)
    if isinstance(a, (int, float, np.integer, np.floating)):
        return 'scalar'
    return type(a).__name__


class CallTrace(object):
    """Records every kernel call made through ``traced`` functions as
    (module.routine, argument kinds)."""

    def __init__(self):
        self.calls = []
        self.on = True

    def traced(self, qualname, fn):
        def call(*args):
            if self.on:
                self.calls.append((qualname, tuple(arg_kind(a) for a in args)))
            return fn(*args)
        call.__name__ = getattr(fn, '__name__', qualname)
        return call

    def forms(self):
        """the distinct calls as text: routine(kind, kind, ...)"""
        return sorted(set(call_form(c) for c in self.calls))

    def digest(self):
        """sha256 of the whole call sequence, one call per line"""
        import hashlib
        return hashlib.sha256('\n'.join(call_form(c) for c in self.calls).encode()).hexdigest()


def call_form(call):
    return '%s(%s)' % (call[0], ', '.join(call[1]))


TRACE = CallTrace()
TRACE.on = False


def kernel_set(modules, trace=None):
    """A namespace with the oracle's names over the routines of the given
    f2py-named modules ({module name: module}), optionally traced."""
    ns = types.SimpleNamespace()
    for mod, names in F2PY_NAMES.items():
        m = modules[mod]
        for routine, oname in names.items():
            if not hasattr(m, routine):
                continue
            fn = getattr(m, routine)
            if trace is not None:
                fn = trace.traced(mod + '.' + routine, fn)
            setattr(ns, oname, fn)
    return ns


def install(core_dir):
    """Make ``core_dir`` (the reference's core/) importable over the oracle.
    Kernel calls are recorded in ``TRACE`` while ``TRACE.on`` is set."""
    if not hasattr(np, 'NaN'):
        np.NaN = np.nan
    mpi = _module('mpi4py.MPI', COMM_WORLD=_Comm(), SUM='sum', MAX='max', MIN='min')
    sys.modules['mpi4py'] = _module('mpi4py', MPI=mpi)
    sys.modules['mpi4py.MPI'] = mpi
    sys.modules['netCDF4'] = _module('netCDF4', Dataset=None)
    for mod, names in F2PY_NAMES.items():
        sys.modules[mod] = _module(mod, **{
            routine: TRACE.traced(mod + '.' + routine, getattr(K, oname))
            for routine, oname in names.items()})
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
