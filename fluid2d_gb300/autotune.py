"""Autotuning of the launch structure by timing it on the device.

* ``tune_coarse_level(model)``: the level from which the multigrid's coarse
  part runs as one unit: the shared-memory CTA of the cycle (exact build), or
  its precomputed linear map (product build, at most 1024 points).  A finer
  switch level means a longer one-SM chain or a larger operator, a coarser
  one adds small latency-bound launches; the best split depends on the grid
  and the precision, so every allowed level is timed on the model's
  captured step.  Results do not depend on the choice beyond rounding.
* ``tune_level_tiles(model)``: the CTA tile shape and block size of the
  multigrid level kernels (process-wide settings read at graph capture).
* ``tune_ensemble(ens)``: the instances' coarse-switch offset (their
  operators' total size against the L2 cache), the number of batched groups
  and the merge policy of an Ensemble's batched launches, against the
  per-instance stream replay.

Timings use CUDA events on the launching stream after warm-up steps; the
model's state advances while it is tuned, so tune on a copy when the
trajectory matters.  Choices are cached per (kind, grid, precision) for the
process.
"""
import torch

_cache = {}


def _time(run, steps, warmup):
    s = torch.cuda.current_stream()
    run(warmup)
    s.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    run(steps)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def tune_coarse_level(model, steps=5, warmup=2, use_cache=True):
    """Time the captured step for every allowed coarse level, keep the
    fastest; returns (best level, {level: ms per step})."""
    key = (model.modelname, model.desc.nx, model.desc.ny, model.desc.precision)
    if use_cache and key in _cache:
        model.coarse_switch(_cache[key][0])
        return _cache[key]
    cur, first, nlev = model.coarse_switch()
    times = {}
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for level in range(first, nlev + 1):
            model.coarse_switch(level)
            times[level] = _time(lambda n: model.run(n, graph=True), steps, warmup)
    torch.cuda.current_stream().wait_stream(side)
    best = min(times, key=times.get)
    model.coarse_switch(best)
    _cache[key] = (best, times)
    return best, times


def tune_level_tiles(model, steps=5, warmup=2, use_cache=True):
    """The CTA tile shape and block size of the multigrid level kernels:
    the CTA count a level's grid aims at before its tile stops shrinking
    (f2d_set_level_tiles: 0 the largest tile, else a multiple of the SM
    count) and the fused smoother's threads (f2d_set_level_threads: one per
    tile point, or one per input point on small grids).  Both are process
    settings read when a graph is captured; the fastest pair on the model's
    captured step is kept set.  Returns ((target, threads), {pair: ms})."""
    from . import _lib
    L = _lib.lib(model.variant)
    key = ("tiles", model.modelname, model.desc.nx, model.desc.ny, model.desc.precision)
    if use_cache and key in _cache:
        best = _cache[key][0]
        L.f2d_set_level_tiles(best[0])
        L.f2d_set_level_threads(best[1])
        model.reset_graphs()
        return _cache[key]
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    times = {}
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for pair in ((0, 0), (2 * sms, 0), (4 * sms, 0), (0, 1), (2 * sms, 1)):
            L.f2d_set_level_tiles(pair[0])
            L.f2d_set_level_threads(pair[1])
            model.reset_graphs()
            times[pair] = _time(lambda n: model.run(n, graph=True), steps, warmup)
    torch.cuda.current_stream().wait_stream(side)
    best = min(times, key=times.get)
    L.f2d_set_level_tiles(best[0])
    L.f2d_set_level_threads(best[1])
    model.reset_graphs()
    _cache[key] = (best, times)
    return best, times


def tune_ensemble(ens, candidates=((1, 1), (2, 1), (4, 1), (8, 1), (16, 1), (16, 0)),
                  offsets=(0, 1), steps=5, warmup=2):
    """Pick the coarse-switch offset of the instances (Ensemble.coarse_offset:
    the sum of the instances' coarse operators against the L2 cache) and the
    batched grouping and merge policy (groups 0: every instance's own graph
    replayed on streams) with the shortest ensemble step; returns
    ((offset, groups, policy), {choice: ms})."""
    times = {}
    for off in offsets:
        ens.free_batch()
        ens.coarse_offset(off)
        ens.capture()
        times[(off, 0, None)] = _time(ens.run, steps, warmup)
        for groups, policy in candidates:
            ens.build_batch(groups, policy)
            times[(off, groups, policy)] = _time(ens.run, steps, warmup)
    best = min(times, key=times.get)
    ens.free_batch()
    ens.coarse_offset(best[0])
    if best[1] != 0:
        ens.build_batch(best[1], best[2])
    return best, times
