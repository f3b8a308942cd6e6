"""Seeded synthetic initial states of the benchmark workloads.

The reference publishes no dataset: every workload is generated here, on the
host, in float64 with numpy's default_rng(seed), so that the oracle and the
GPU start from byte-identical states.

* ``dipole``      Euler, closed square, two Gaussians +-1 (sigma 0.05) at
                  (0.4, 0.5) and (0.6, 0.5) plus uniform noise of 1e-3
                  (the form of experiments/Vortex/vortex.py:125).
* ``turbulence``  Euler, doubly periodic, random-phase vorticity with
                  E(k) ~ k^3 exp(-(k/10)^2), zero mean, rms 1.
* ``shear``       Boussinesq shear layer, 'xchannel': u = tanh((y-1/2)/d)
                  set through its vorticity, b = tanh((y-1/2)/d) plus
                  1e-3 N(0,1) noise, d = 0.02.
* ``ensemble``    Euler, closed, islands rasterised into the mask, 3-12
                  Gaussian vortices.
"""
import numpy as np


def cell_coords(nx, ny, Lx, Ly, nh=3):
    """Cell-centre coordinates of core/grid.py:47-52 (one rank)."""
    dx, dy = Lx / nx, Ly / ny
    x1d = (np.arange(nx + 2 * nh) + 0.5 - nh + 0) * dx
    y1d = (np.arange(ny + 2 * nh) + 0.5 - nh + 0) * dy
    return np.meshgrid(x1d, y1d)


def base_mask(nx, ny, geometry, nh=3):
    """The geometry mask of core/grid.py:67-99 (one rank)."""
    msk = np.ones((ny + 2 * nh, nx + 2 * nh), dtype=np.int8)
    if geometry in ('xperio', 'xchannel', 'closed', 'disc'):
        msk[-nh:, :] = 0
        msk[:nh, :] = 0
    if geometry in ('yperio', 'ychannel', 'closed', 'disc'):
        msk[:, -nh:] = 0
        msk[:, :nh] = 0
    if geometry == 'disc':
        xr, yr = cell_coords(nx, ny, 1., 1., nh)
        r = np.sqrt((xr - 0.5) ** 2 + (yr - 0.5) ** 2)
        msk[r >= 0.5] = 0
    return msk


def dipole(nx=128, ny=128, seed=1, sigma=0.05, noise=1e-3):
    xr, yr = cell_coords(nx, ny, 1., 1.)
    msk = base_mask(nx, ny, 'closed')
    rng = np.random.default_rng(seed)
    w = (np.exp(-((xr - 0.4) ** 2 + (yr - 0.5) ** 2) / sigma ** 2)
         - np.exp(-((xr - 0.6) ** 2 + (yr - 0.5) ** 2) / sigma ** 2))
    w = w + rng.uniform(-noise, noise, size=w.shape)
    return {'model': 'euler', 'geometry': 'closed', 'nx': nx, 'ny': ny, 'Lx': 1., 'Ly': 1.,
            'msk': msk, 'fields': {'vorticity': w * msk}}


def turbulence(nx=1024, ny=1024, seed=2, k0=10.):
    """Random-phase field with E(k) ~ k^3 exp(-(k/k0)^2) in integer wavenumber
    units, zero mean, rms 1, periodic halo."""
    nh = 3
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx) * nx
    ky = np.fft.fftfreq(ny) * ny
    KX, KY = np.meshgrid(kx, ky)
    K = np.sqrt(KX ** 2 + KY ** 2)
    E = np.where(K > 0, K ** 3 * np.exp(-(K / k0) ** 2), 0.)
    amp = np.sqrt(np.where(K > 0, E / np.maximum(K, 1e-300), 0.))
    phase = np.exp(2j * np.pi * rng.random((ny, nx)))
    w = np.real(np.fft.ifft2(amp * phase))
    w -= w.mean()
    w /= np.sqrt((w ** 2).mean())
    full = np.zeros((ny + 2 * nh, nx + 2 * nh))
    full[nh:-nh, nh:-nh] = w
    # periodic halo
    full[:nh, :] = full[ny:ny + nh, :]
    full[-nh:, :] = full[nh:2 * nh, :]
    full[:, :nh] = full[:, nx:nx + nh]
    full[:, -nh:] = full[:, nh:2 * nh]
    msk = base_mask(nx, ny, 'perio')
    return {'model': 'euler', 'geometry': 'perio', 'nx': nx, 'ny': ny, 'Lx': 1., 'Ly': 1.,
            'msk': msk, 'fields': {'vorticity': full}}


def shear(nx=2048, ny=512, seed=3, delta=0.02, gravity=5.):
    Lx, Ly = 4., 1.
    xr, yr = cell_coords(nx, ny, Lx, Ly)
    msk = base_mask(nx, ny, 'xchannel')
    rng = np.random.default_rng(seed)
    s = (yr - 0.5) / delta
    w = -(1. / delta) / np.cosh(s) ** 2
    b = np.tanh(s) + 1e-3 * rng.standard_normal(w.shape)
    return {'model': 'boussinesq', 'geometry': 'xchannel', 'nx': nx, 'ny': ny, 'Lx': Lx,
            'Ly': Ly, 'gravity': gravity, 'msk': msk,
            'fields': {'vorticity': w * msk, 'buoyancy': b * msk}}


def ensemble_member(rng, nmin=64, nmax=768, step=64):
    """One instance of the batched ensemble: sizes log-uniform in
    [nmin, nmax] rounded to multiples of `step`, dx = dy (Lx = 1,
    Ly = ny/nx), 0-4 circular islands, 3-12 Gaussian vortices."""
    def side():
        v = np.exp(rng.uniform(np.log(nmin), np.log(nmax)))
        return int(max(nmin, min(nmax, step * round(v / step))))
    nx, ny = side(), side()
    Lx, Ly = 1., ny / nx
    xr, yr = cell_coords(nx, ny, Lx, Ly)
    msk = base_mask(nx, ny, 'closed')
    L = min(Lx, Ly)
    for _ in range(rng.integers(0, 5)):
        r = rng.uniform(0.03, 0.1) * L
        cx, cy = rng.uniform(r, Lx - r), rng.uniform(r, Ly - r)
        msk[(xr - cx) ** 2 + (yr - cy) ** 2 < r * r] = 0
    w = np.zeros_like(xr)
    fluid = np.argwhere(msk[3:-3, 3:-3] == 1)
    for _ in range(rng.integers(3, 13)):
        a = rng.standard_normal()
        sig = rng.uniform(0.02, 0.08)
        j, i = fluid[rng.integers(len(fluid))]
        cx, cy = xr[3, 3 + i], yr[3 + j, 3]
        w += a * np.exp(-((xr - cx) ** 2 + (yr - cy) ** 2) / sig ** 2)
    return {'model': 'euler', 'geometry': 'closed', 'nx': nx, 'ny': ny, 'Lx': Lx, 'Ly': Ly,
            'msk': msk, 'fields': {'vorticity': w * msk}}


def ensemble(count=96, seed=4, **kw):
    rng = np.random.default_rng(seed)
    return [ensemble_member(rng, **kw) for _ in range(count)]


def served_request(rng, euler_fraction=0.7, side_min=128, side_max=2048, step=128,
                   steps_min=50, steps_max=500):
    """One request of the served stream: 70 % Euler / 30 % Boussinesq, sides
    log-uniform in [side_min, side_max] rounded to multiples of `step`
    (dx = dy), island masks and initial fields from the request's own seed
    as in the ensemble (Euler, closed) and shear-layer (Boussinesq,
    'xchannel') workloads, a step count uniform in [steps_min, steps_max]."""
    seed = int(rng.integers(2 ** 31))
    r = np.random.default_rng(seed)

    def side():
        v = np.exp(r.uniform(np.log(side_min), np.log(side_max)))
        return int(max(side_min, min(side_max, step * round(v / step))))
    nx, ny = side(), side()
    steps = int(r.integers(steps_min, steps_max + 1))
    if r.random() < euler_fraction:
        wl = _euler_with_islands(r, nx, ny)
    else:
        wl = _shear_with_islands(r, nx, ny)
    wl["seed"] = seed
    return wl, steps


def _euler_with_islands(r, nx, ny):
    Lx, Ly = 1., ny / nx
    xr, yr = cell_coords(nx, ny, Lx, Ly)
    msk = base_mask(nx, ny, 'closed')
    L = min(Lx, Ly)
    for _ in range(r.integers(0, 5)):
        rad = r.uniform(0.03, 0.1) * L
        cx, cy = r.uniform(rad, Lx - rad), r.uniform(rad, Ly - rad)
        msk[(xr - cx) ** 2 + (yr - cy) ** 2 < rad * rad] = 0
    w = np.zeros_like(xr)
    fluid = np.argwhere(msk[3:-3, 3:-3] == 1)
    for _ in range(r.integers(3, 13)):
        a = r.standard_normal()
        sig = r.uniform(0.02, 0.08)
        j, i = fluid[r.integers(len(fluid))]
        cx, cy = xr[3, 3 + i], yr[3 + j, 3]
        w += a * np.exp(-((xr - cx) ** 2 + (yr - cy) ** 2) / sig ** 2)
    return {'model': 'euler', 'geometry': 'closed', 'nx': nx, 'ny': ny, 'Lx': Lx, 'Ly': Ly,
            'msk': msk, 'fields': {'vorticity': w * msk}}


def _shear_with_islands(r, nx, ny, delta=0.02, gravity=5.):
    """Boussinesq shear layer (Ri = 0.1) in a periodic channel with islands
    kept away from the periodic ends (the halo of the mask is not filled)."""
    Ly = 1.
    Lx = nx / ny * Ly
    xr, yr = cell_coords(nx, ny, Lx, Ly)
    msk = base_mask(nx, ny, 'xchannel')
    dx = Lx / nx
    for _ in range(r.integers(0, 5)):
        rad = r.uniform(0.03, 0.1) * min(Lx, Ly)
        cx = r.uniform(rad + 4 * dx, Lx - rad - 4 * dx)
        cy = r.uniform(rad, Ly - rad)
        msk[(xr - cx) ** 2 + (yr - cy) ** 2 < rad * rad] = 0
    s = (yr - 0.5) / delta
    w = -(1. / delta) / np.cosh(s) ** 2
    b = np.tanh(s) + 1e-3 * r.standard_normal(w.shape)
    return {'model': 'boussinesq', 'geometry': 'xchannel', 'nx': nx, 'ny': ny, 'Lx': Lx,
            'Ly': Ly, 'gravity': gravity, 'msk': msk,
            'fields': {'vorticity': w * msk, 'buoyancy': b * msk}}


def served_stream(count=2000, rate=40., seed=5, **kw):
    """(arrival time, workload, steps) of `count` requests with Poisson
    arrivals at `rate` per second."""
    rng = np.random.default_rng(seed)
    t = 0.
    out = []
    for _ in range(count):
        t += rng.exponential(1. / rate)
        wl, steps = served_request(rng, **kw)
        out.append((t, wl, steps))
    return out
