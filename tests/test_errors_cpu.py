"""Error behaviour of the C ABI that is decided on the host, before any
device work (no GPU needed; nothing is launched): the reference's Fortran
stop on a halo other than 3 becomes F2D_ERR_NH with its message
(core/fortran_advection.f90:30-34), unusable shapes F2D_ERR_SHAPE, null
pointers and bad options F2D_ERR_ARG, and a model description the engine
cannot run is refused before anything is allocated."""
import ctypes

import numpy as np
import pytest

OK, ERR_NH, ERR_SHAPE, ERR_ARG = 0, 1, 2, 3


@pytest.fixture(scope="module")
def L():
    from fluid2d_gb300 import _lib
    _lib.build()
    lib = ctypes.CDLL(_lib.so_path("product"))
    lib.f2d_last_error.restype = ctypes.c_char_p
    return lib


def _adv(L, nh, m, n, null_msk=False):
    dummy = ctypes.c_void_p(16)     # never dereferenced: the checks come first
    msk = None if null_msk else dummy
    return L.f2d_adv_upwind(msk, dummy, dummy, dummy, dummy, dummy, ctypes.c_int(nh),
                            ctypes.c_int(1), ctypes.c_int(5), ctypes.c_int(m), ctypes.c_int(n),
                            None)


def test_advection_halo_must_be_three(L):
    assert _adv(L, 2, 38, 38) == ERR_NH
    assert b"NHALO = 3" in L.f2d_last_error()


def test_advection_shape_and_pointers(L):
    assert _adv(L, 3, 6, 38) == ERR_SHAPE
    assert _adv(L, 3, 38, 38, null_msk=True) == ERR_ARG


def _desc(**kw):
    from fluid2d_gb300 import _lib
    d = _lib.ModelDesc()
    d.model, d.nx, d.ny, d.Lx, d.Ly = 0, 32, 32, 1., 1.
    d.order, d.flux_method, d.aparab = 5, 1, 0.05
    d.gravity, d.Rd, d.hydroepsilon = 1., 1., 1.
    d.dt, d.cfl, d.dtmax = 0.1, 0.5, 5.
    for k, v in kw.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("kw,code,words", [
    (dict(nx=2), ERR_SHAPE, b"bad grid"),
    (dict(ny=40000), ERR_SHAPE, b"bad grid"),
    (dict(Lx=-1.), ERR_SHAPE, b"bad grid"),
    (dict(model=7), ERR_ARG, b"unknown kind"),
    (dict(order=9), ERR_ARG, b"bad order"),
    (dict(dt=0.), ERR_ARG, b"dt"),
    (dict(precision=4), ERR_ARG, b"precision"),
])
def test_model_descriptions_refused(L, kw, code, words):
    d = _desc(**kw)
    msk = np.ones((d.ny + 6, d.nx + 6), dtype=np.int8) if d.ny < 1000 else np.ones(1, np.int8)
    h = ctypes.c_void_p()
    rc = L.f2d_model_create(ctypes.byref(d), msk.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
    assert rc == code and words in L.f2d_last_error(), (rc, L.f2d_last_error())
    assert not h.value


def test_model_without_fluid_or_arguments(L):
    d = _desc()
    solid = np.zeros((38, 38), dtype=np.int8)
    h = ctypes.c_void_p()
    assert L.f2d_model_create(ctypes.byref(d), solid.ctypes.data_as(ctypes.c_void_p),
                              ctypes.byref(h)) == ERR_ARG
    assert b"no fluid cell" in L.f2d_last_error()
    assert L.f2d_model_create(None, None, ctypes.byref(h)) == ERR_ARG
    assert L.f2d_model_destroy(None) == OK
