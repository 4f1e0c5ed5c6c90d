"""The checked training loop: an overflow of the cell lists inside a captured
step is caught, the interval is undone and run again after a re-capture with
room for the entries, and the run ends where a run with enough room from the
start ends."""
import math

import pytest
import torch

pytestmark = pytest.mark.gpu


def test_train_recovers_from_a_cell_list_overflow(sgr_lib):
    from partgs_gb300 import _lib as L
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    from partgs_gb300.surfel_step import SurfelTrainer
    scene, cams = random_surfels(3000, seed=6), orbit_cameras(3, 3.0, 64, 80, 55.0, seed=3)
    targets = torch.rand(len(cams), 3, 64, 80, generator=torch.Generator().manual_seed(5)).cuda()
    tr = SurfelTrainer(scene, cams)
    tr.capture(targets, warmup=2)
    start = tr.snapshot()
    loss_ok = float(tr.train(6, check_every=3).detach())
    assert tr.recaptures == 0
    ok = [p.detach().clone() for p in tr.params()]
    _, _, entries = tr.raster.counts()
    tr.restore(start)                                   # a second clean run: the natural spread
    tr.train(6, check_every=3)
    again = [p.detach().clone() for p in tr.params()]

    tr.restore(start)
    tr.raster.set_capacity(max(1, entries // 3))        # far too small for this scene
    tr.capture(targets, warmup=1)
    tr.restore(start)
    tr.replay()
    flags, _ = tr.raster.sticky_counts(reset=True)
    assert flags & L.SGR_FLAG_BIN_OVERFLOW                # the captured step overflows
    tr.restore(start)
    loss = float(tr.train(6, check_every=3).detach())
    assert tr.recaptures >= 1 and math.isfinite(loss)
    assert tr.raster.bin_capacity >= entries
    # Runs differ only in the order of the gradient atomics.  Adam's first
    # steps move every element by about +-lr whatever its gradient's size, so
    # an element whose gradient is near zero may step the other way.  The
    # recovered run must be as close to the clean run as two clean runs are.
    assert abs(loss - loss_ok) <= 1e-3 * abs(loss_ok)

    def off(a, b):
        return float(((a - b).abs() > 1e-5 * max(float(a.abs().max()), 1.0)).float().mean())

    for a, c, b in zip(ok, again, tr.params()):
        assert off(a, b.detach()) <= 3 * off(a, c) + 0.005


def test_fused_step_gradients_equal_the_autograd_path(sgr_lib):
    """The fused step (loss kernels -> rasteriser backward -> activation
    backward into the .grad buffers, no autograd and no PyTorch kernels)
    gives the loss and parameter gradients the autograd path through the
    same kernels gives (up to the order of the gradient atomics)."""
    from partgs_gb300.cameras import orbit_cameras
    from partgs_gb300.scenes import random_surfels
    from partgs_gb300.surfel_step import SurfelTrainer
    scene, cams = random_surfels(3000, seed=8), orbit_cameras(3, 3.0, 64, 80, 55.0, seed=4)
    targets = torch.rand(len(cams), 3, 64, 80, generator=torch.Generator().manual_seed(6)).cuda()
    tr = SurfelTrainer(scene, cams)
    with torch.no_grad():
        loss_fused = float(tr._fused_step(targets))
    fused = [p.grad.detach().clone() for p in tr.params()]
    for p in tr.params():
        p.grad.zero_()
    loss_ag = tr.loss_fn(targets)
    loss_ag.backward()
    assert abs(float(loss_ag) - loss_fused) <= 1e-6 * abs(loss_fused)
    for a, p in zip(fused, tr.params()):
        b = p.grad
        assert float(a.abs().max()) > 0
        assert float((a - b).abs().max()) <= 1e-5 * float(b.abs().max()), p.shape
