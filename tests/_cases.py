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
