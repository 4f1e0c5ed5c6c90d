"""Workload autotuning of the rasteriser's cell size.

Each blend CTA streams the list of the cell that holds its tile and keeps
the entries whose rectangle holds the tile (sgr_binning.cu, sgr_blend.cu).
Small cells mean short, dense lists but more (record, cell) entries to bin;
large cells the reverse, and the best edge depends on the surfels' screen
sizes and on the image.  ``tune_cells`` times whole training steps of a
``SurfelTrainer`` for each candidate edge (parameters and optimiser state
restored after each trial) and keeps the fastest; results are cached per
workload shape for the process.
"""
from __future__ import annotations

import torch

CANDIDATES = (2, 4, 8, 16)
_CACHE: dict = {}


def workload_key(trainer) -> tuple:
    r = trainer.raster
    return (int(trainer.xyz.shape[0]), r.num_views, r.viewset.height, r.viewset.width)


def tune_cells(trainer, targets, candidates=CANDIDATES, steps: int = 3, log=None) -> int:
    """Sets ``trainer.raster.cell_tiles`` to the fastest candidate for this
    workload and returns it, with {edge: ms per step} in ``last_timings``."""
    key = workload_key(trainer)
    if key in _CACHE:
        trainer.raster.cell_tiles = _CACHE[key]
        return _CACHE[key]
    state = trainer.snapshot()
    saved_capacity = trainer.raster.bin_capacity
    timings = {}
    for edge in candidates:
        trainer.raster.cell_tiles = edge
        trainer.raster.set_capacity(None)          # eager steps size the lists exactly
        trainer.step(targets)                      # first use of this edge
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            trainer.step(targets)
        e1.record()
        torch.cuda.synchronize()
        timings[edge] = e0.elapsed_time(e1) / steps
        trainer.restore(state)
        if log:
            log(f"cell edge {edge}: {timings[edge]:.2f} ms per step")
    best = min(timings, key=timings.get)
    trainer.raster.cell_tiles = best
    trainer.raster.set_capacity(saved_capacity)
    tune_cells.last_timings = timings
    _CACHE[key] = best
    return best


tune_cells.last_timings = {}
