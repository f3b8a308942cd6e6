"""Seeded inputs shared by the parity tests (masks with islands, fields)."""
import numpy as np


def mask(m, n, geometry="closed", islands=0, seed=0, nh=3):
    """int8 (m, n) mask with the geometry's walls in the halo and circular
    islands (msk = 0) rasterised at cell centres."""
    rng = np.random.default_rng(seed)
    msk = np.ones((m, n), dtype=np.int8)
    jj, ii = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    inner = (jj >= nh) & (jj < m - nh) & (ii >= nh) & (ii < n - nh)
    for _ in range(islands):
        cj, ci = rng.uniform(nh, m - nh), rng.uniform(nh, n - nh)
        r = rng.uniform(1.0, max(1.5, 0.15 * min(m, n)))
        msk[inner & ((jj + 0.5 - cj) ** 2 + (ii + 0.5 - ci) ** 2 < r * r)] = 0
    # periodic directions see the islands through the halo
    msk[:nh, :] = msk[m - 2 * nh:m - nh, :]
    msk[m - nh:, :] = msk[nh:2 * nh, :]
    msk[:, :nh] = msk[:, n - 2 * nh:n - nh]
    msk[:, n - nh:] = msk[:, nh:2 * nh]
    if geometry in ("closed", "xchannel"):
        msk[:nh, :] = 0
        msk[-nh:, :] = 0
    if geometry in ("closed", "ychannel"):
        msk[:, :nh] = 0
        msk[:, -nh:] = 0
    return msk


def field(m, n, seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    return scale * rng.standard_normal((m, n))


def corner_mask(msk):
    """The GMG level-0 mask of core/operators.py:47-67 (via the oracle)."""
    from oracle import oracle as K
    work = np.zeros(msk.shape)
    K.celltocorner(msk * 1., work)
    work[work < 1.] = 0.
    return work.astype(np.int8)


def oracle_model(wl, **kw):
    """The oracle stepper model for a workloads.* dict (mask, fields, psi)."""
    from oracle import stepper
    return stepper.from_workload(wl, **kw)


def island_workload():
    """Euler, closed 96x64 box (dx = dy) with two circular islands."""
    from fluid2d_gb300 import workloads as W
    wl = W.dipole(96, 64, seed=13)
    wl["Lx"], wl["Ly"] = 1.5, 1.
    xr, yr = W.cell_coords(96, 64, 1.5, 1.)
    msk = W.base_mask(96, 64, "closed")
    for cx, cy, r in ((0.35, 0.3, 0.08), (1.1, 0.65, 0.1)):
        msk[(xr - cx) ** 2 + (yr - cy) ** 2 < r * r] = 0
    wl["msk"] = msk
    w = (np.exp(-((xr - 0.7) ** 2 + (yr - 0.5) ** 2) / 0.05 ** 2)
         - np.exp(-((xr - 0.85) ** 2 + (yr - 0.5) ** 2) / 0.05 ** 2))
    wl["fields"] = {"vorticity": w * msk}
    return wl
