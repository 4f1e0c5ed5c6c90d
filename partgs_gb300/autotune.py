"""Workload autotuning of the rasteriser's launch shape.

Four knobs change speed but not results:

* the cell size.  Each blend CTA streams the list of the cell that holds its
  tile and keeps the entries whose rectangle holds the tile
  (sgr_binning.cu, sgr_blend.cu).  Small cells mean short, dense lists but
  more (record, cell) entries to bin; large cells the reverse.
* the warp footprint (``blend_shape``): 16-pixel-wide strips or 8-pixel-wide
  patches of the 16x16 tile per warp.  Compact patches let a warp skip more
  entries whose splats miss it and keep more lanes busy on those that hit
  it, at the price of more per-entry reach tests.
* the tile schedule: one CTA per tile, or persistent CTAs taking tiles from
  a device queue in decreasing order of estimated cost (uneven scenes).
* the staged batch (``stage_entries``): how many list entries the blends
  copy into shared memory between two CTA barriers, 256, 128 or 64.  Larger
  batches mean fewer barriers; smaller ones less shared memory per CTA and
  less waiting at each barrier for the warp with the most work.

The best choice depends on the surfels' screen sizes, the image and the
scene mix.  ``tune_cells`` times whole training steps of a ``SurfelTrainer``
for each candidate cell edge, ``tune_blend`` then each footprint, schedule
and staged batch at that edge (parameters and optimiser state restored after each
trial); results are cached per workload shape for the process.
"""
from __future__ import annotations

import torch

from . import _lib as L

CANDIDATES = (2, 4, 8, 16)
SHAPES = (L.SGR_BLEND_STRIP16, L.SGR_BLEND_PATCH8)
SCHEDULES = (L.SGR_SCHEDULE_GRID, L.SGR_SCHEDULE_QUEUE)
STAGES = (L.SGR_STAGE_DEFAULT, L.SGR_STAGE_SMALL, L.SGR_STAGE_TINY)
_CACHE: dict = {}


def workload_key(trainer) -> tuple:
    r = trainer.raster
    return (int(trainer.xyz.shape[0]), r.num_views, r.viewset.height, r.viewset.width)


def _time_steps(trainer, targets, steps):
    trainer.step(targets)                      # first use of this configuration
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        trainer.step(targets)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def tune_cells(trainer, targets, candidates=CANDIDATES, steps: int = 3, log=None) -> int:
    """Sets ``trainer.raster.cell_tiles`` to the fastest candidate for this
    workload and returns it, with {edge: ms per step} in ``last_timings``."""
    key = ("cells",) + workload_key(trainer)
    if key in _CACHE:
        trainer.raster.cell_tiles = _CACHE[key]
        return _CACHE[key]
    state = trainer.snapshot()
    saved_capacity = trainer.raster.bin_capacity
    timings = {}
    # two rounds, the second in reverse order, the faster time of each kept:
    # a single short timing picked up clock and cache transients
    for order in (list(candidates), list(candidates)[::-1]):
        for edge in order:
            trainer.raster.cell_tiles = edge
            trainer.raster.set_capacity(None)          # eager steps size the lists exactly
            t = _time_steps(trainer, targets, steps)
            timings[edge] = min(t, timings.get(edge, t))
            trainer.restore(state)
            if log:
                log(f"cell edge {edge}: {t:.2f} ms per step")
    best = min(timings, key=timings.get)
    trainer.raster.cell_tiles = best
    trainer.raster.set_capacity(saved_capacity)
    tune_cells.last_timings = timings
    _CACHE[key] = best
    return best


tune_cells.last_timings = {}


def tune_blend(trainer, targets, shapes=SHAPES, schedules=SCHEDULES, stages=STAGES, steps: int = 3,
               log=None) -> tuple:
    """Sets ``trainer.raster.blend_shape``, ``tile_schedule`` and
    ``stage_entries`` to the fastest combination for this workload (at the
    current cell edge) and returns it, with {(shape, schedule, stage): ms per
    step} in ``last_timings``."""
    key = ("blend", trainer.raster.cell_tiles) + workload_key(trainer)
    r = trainer.raster
    if key in _CACHE:
        r.blend_shape, r.tile_schedule, r.stage_entries = _CACHE[key]
        return _CACHE[key]
    state = trainer.snapshot()
    saved_capacity = r.bin_capacity
    timings = {}
    combos = [(shape, sched, stage) for shape in shapes for sched in schedules for stage in stages]
    for order in (combos, combos[::-1]):               # two rounds, as tune_cells
        for combo in order:
            r.blend_shape, r.tile_schedule, r.stage_entries = combo
            r.set_capacity(None)
            t = _time_steps(trainer, targets, steps)
            timings[combo] = min(t, timings.get(combo, t))
            trainer.restore(state)
            if log:
                log(f"blend shape {combo[0]}, schedule {combo[1]}, stage {combo[2]}: {t:.2f} ms per step")
    best = min(timings, key=timings.get)
    r.blend_shape, r.tile_schedule, r.stage_entries = best
    r.set_capacity(saved_capacity)
    tune_blend.last_timings = timings
    _CACHE[key] = best
    return best


tune_blend.last_timings = {}
