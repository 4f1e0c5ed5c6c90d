"""Every C entry point checks its arguments on the host and returns the
documented status before any device work: null pointers, negative sizes,
sizes past a limit and undersized workspaces give their codes, and empty
inputs return SGR_OK without a launch.  No case here reaches a kernel, a
device copy or a device query (each return below precedes the first CUDA
call of its entry point), so the suite runs without a GPU."""
import ctypes as C

import pytest

OK, INVALID, UNSUPPORTED, WORKSPACE = 0, 1, 2, 4
FAKE = 256          # a non-null address that no case dereferences


@pytest.fixture(scope="module")
def lib(sgr_lib):
    from partgs_gb300 import activations, chamfer_eval, densify, losses, optim, proposal, proposal_gemm, sq_losses
    for bind in (activations._lib, chamfer_eval._lib, densify._lib, losses._lib, optim._lib, proposal._pool_lib,
                 proposal_gemm._lib, sq_losses._lib):
        bind()
    return sgr_lib


def _fields(struct, *names):
    """The names a case assigns are fields of the struct (ctypes would take
    any other name as a plain attribute and the case would test nothing)."""
    have = {f[0] for f in struct._fields_}
    assert set(names) <= have, set(names) - have


@pytest.fixture(autouse=True)
def no_launches(lib):
    before = lib.sgr_kernel_launches()
    yield
    assert lib.sgr_kernel_launches() == before


def test_rasteriser_entry_points(lib):
    from partgs_gb300 import _lib as L
    assert lib.sgr_forward_geometry(None, FAKE, FAKE, 0, None, None) == INVALID
    assert lib.sgr_forward_raster(None, FAKE, FAKE, 0, FAKE, 0, None, None) == INVALID
    assert lib.sgr_backward(None, FAKE, FAKE, 0, FAKE, 0, None, None, None) == INVALID
    assert lib.sgr_tile_lists(None, FAKE, None, 0, FAKE, 0, None) == INVALID
    _fields(L.Batch, "variant", "num_scenes", "num_views", "height", "width", "scenes", "views", "viewmatrix",
            "projmatrix", "campos", "background", "cell_tiles")
    b = L.Batch()
    b.variant, b.num_scenes, b.num_views, b.height, b.width = 0, 1, 1, 8, 8
    b.scenes = b.views = b.viewmatrix = b.projmatrix = b.campos = b.background = FAKE
    assert lib.sgr_forward_geometry(C.byref(b), None, FAKE, 0, None, None) == INVALID     # no geometry buffer
    b.cell_tiles = 3
    assert lib.sgr_forward_geometry(C.byref(b), FAKE, FAKE, 0, None, None) == INVALID     # cell edge not 1..16 pow2
    b.cell_tiles = 0
    out = L.FwdOutputs()
    assert lib.sgr_forward_raster(C.byref(b), FAKE, FAKE, -1, FAKE, 0, C.byref(out), None) == 5   # capacity < 0
    assert lib.sgr_forward_raster(C.byref(b), FAKE, FAKE, 0, FAKE, 0, C.byref(out), None) == INVALID  # no colour
    gin, gout = L.BwdInputs(), L.BwdOutputs()
    assert lib.sgr_backward(C.byref(b), FAKE, None, 4, FAKE, 0, C.byref(gin), C.byref(gout), None) == INVALID
    assert lib.sgr_backward(C.byref(b), FAKE, FAKE, 0, FAKE, 0, C.byref(gin), C.byref(gout), None) == INVALID


def test_binding(lib):
    from partgs_gb300 import _lib as L
    assert lib.sgr_bind_forward(None, None, None, None, None, None) == INVALID
    _fields(L.BindArgs, "B", "V", "F", "N", "sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ", "eta", "omega", "faces",
            "alpha", "scale")
    a = L.BindArgs()
    a.B = -1
    assert lib.sgr_bind_forward(C.byref(a), None, None, None, None, None) == INVALID
    a.B, a.V, a.F, a.N = 2, 9, 9, 1
    assert lib.sgr_bind_forward(C.byref(a), None, None, None, None, None) == INVALID       # no parameters
    a.sq_s = a.sq_r = a.sq_t = a.sq_eps = a.sq_occ = FAKE
    assert lib.sgr_bind_forward(C.byref(a), None, None, None, None, None) == INVALID       # no topology
    a.eta = a.omega = a.faces = a.alpha = a.scale = FAKE
    assert lib.sgr_bind_backward(C.byref(a), *([None] * 9), FAKE, None) == INVALID        # no output gradients
    assert lib.sgr_bind_scratch_bytes(None) == 0
    assert lib.sgr_bind_scratch_bytes(C.byref(a)) == 256 + 2 * 9 * 4           # vertex sums, 256-aligned
    e = L.BindArgs()                                                                      # no blocks: nothing to do
    assert lib.sgr_bind_forward(C.byref(e), None, None, None, None, None) == OK
    assert lib.sgr_bind_backward(C.byref(e), *([None] * 9), None, None) == OK


def test_optimiser_and_activations(lib):
    from partgs_gb300.activations import ActivateArgs
    from partgs_gb300.optim import AdamArgs
    assert lib.sgr_adam_step(None, None, None) == INVALID
    _fields(AdamArgs, "beta1", "beta2", "eps", "count", "tensors")
    _fields(ActivateArgs, "P", "sh_coeffs")
    a = AdamArgs()
    a.beta1, a.beta2, a.eps, a.count = 0.9, 0.999, 1e-15, 17
    assert lib.sgr_adam_step(C.byref(a), FAKE, None) == INVALID                            # above 16 tensors
    a.count, a.beta1 = 1, 1.0
    assert lib.sgr_adam_step(C.byref(a), FAKE, None) == INVALID                            # beta1 not in [0, 1)
    a.beta1 = 0.9
    a.tensors[0].numel = -1
    assert lib.sgr_adam_step(C.byref(a), FAKE, None) == INVALID
    a.tensors[0].numel = 8
    assert lib.sgr_adam_step(C.byref(a), FAKE, None) == INVALID                            # no buffers
    assert lib.sgr_activate_forward(None, None) == INVALID
    s = ActivateArgs()
    for P, coeffs in ((-1, 16), (4, 0), (4, 17)):
        s.P, s.sh_coeffs = P, coeffs
        assert lib.sgr_activate_forward(C.byref(s), None) == INVALID, (P, coeffs)
    s.P, s.sh_coeffs = 4, 16
    assert lib.sgr_activate_forward(C.byref(s), None) == INVALID                           # no tensors
    assert lib.sgr_activate_backward(C.byref(s), None, None, None, None, None) == INVALID
    s.P = 0
    assert lib.sgr_activate_forward(C.byref(s), None) == OK
    assert lib.sgr_activate_backward(C.byref(s), None, None, None, None, None) == OK


def test_block_losses(lib):
    from partgs_gb300.sq_losses import SQLossArgs
    assert lib.sgr_sq_losses_forward(None, None) == INVALID
    assert lib.sgr_sq_scratch_bytes(None) == 0
    _fields(SQLossArgs, "S", "R", "T", "eps1", "eps2", "ratio", "n_blocks", "n_rays", "n_samples", "losses")
    a = SQLossArgs()
    a.S = a.R = a.T = a.eps1 = a.eps2 = FAKE
    a.ratio = 0.25
    for n in (0, 65):                                                                      # 1 .. 64 blocks
        a.n_blocks = n
        assert lib.sgr_sq_losses_forward(C.byref(a), None) == INVALID, n
        assert lib.sgr_sq_scratch_bytes(C.byref(a)) == 0
    a.n_blocks, a.ratio = 4, 0.0
    assert lib.sgr_sq_losses_forward(C.byref(a), None) == INVALID                          # ratio must be > 0
    a.ratio, a.n_rays, a.n_samples = 0.25, 10, 0
    assert lib.sgr_sq_losses_forward(C.byref(a), None) == INVALID                          # rays without samples
    a.n_rays = 0
    assert lib.sgr_sq_losses_forward(C.byref(a), None) == INVALID                          # no loss output
    a.losses = FAKE
    assert lib.sgr_sq_losses_forward(C.byref(a), None) == WORKSPACE                        # no scratch
    assert lib.sgr_sq_losses_backward(C.byref(a), None, None) == INVALID                   # no gradient outputs
    assert lib.sgr_sq_sdf(C.byref(a), None, -1, None, None) == INVALID
    assert lib.sgr_sq_sdf(C.byref(a), None, 0, None, None) == OK


def test_evaluation_densification_network_and_loss(lib):
    from partgs_gb300.losses import LossArgs
    from partgs_gb300.proposal_gemm import GemmArgs
    lo, hi = (C.c_float * 3)(0, 0, 0), (C.c_float * 3)(1, 1, 1)
    assert lib.sgr_nn_search(None, -1, None, 0, None, None, None) == INVALID
    assert lib.sgr_nn_search(None, 0, None, 0, None, None, None) == OK                     # no queries
    assert lib.sgr_nn_search(FAKE, 5, FAKE, 0, FAKE, None, None) == INVALID                # nothing to search
    assert lib.sgr_nn_search(FAKE, 5, FAKE, 1 << 31, FAKE, None, None) == UNSUPPORTED      # int32 indices
    assert lib.sgr_nn_grid_scratch_bytes(-1, 4, lo, hi) == 0
    assert lib.sgr_nn_search_grid(None, 0, None, 0, lo, hi, None, None, None, 0, None) == OK
    assert lib.sgr_downsample_scratch_bytes(-1) == 0
    dlo, dhi = (C.c_double * 3)(0, 0, 0), (C.c_double * 3)(1, 1, 1)
    rounds = C.c_int32()
    assert lib.sgr_radius_downsample(FAKE, 4, dlo, dhi, 0.0, FAKE, FAKE, 1 << 20, C.byref(rounds), None) == INVALID
    assert lib.sgr_radius_downsample(FAKE, 4, dhi, dlo, 0.1, FAKE, FAKE, 1 << 20, C.byref(rounds), None) == UNSUPPORTED
    assert lib.sgr_radius_downsample(FAKE, 4, dlo, dhi, 0.1, FAKE, None, 0, C.byref(rounds), None) == WORKSPACE
    assert lib.sgr_radius_downsample(None, 0, None, None, 0.1, None, None, 0, C.byref(rounds), None) == OK
    assert lib.sgr_densify_stats(FAKE, 1, FAKE, -1, None, None, 1.0, None, None, None, None) == INVALID
    assert lib.sgr_densify_stats(FAKE, 0, FAKE, 4, FAKE, FAKE, 1.0, FAKE, FAKE, FAKE, None) == INVALID
    assert lib.sgr_densify_stats(FAKE, 1, FAKE, 4, None, FAKE, 1.0, FAKE, FAKE, FAKE, None) == INVALID
    assert lib.sgr_densify_stats(FAKE, 1, FAKE, 0, None, None, 1.0, None, None, None, None) == OK
    _fields(GemmArgs, "M", "N", "K", "A", "B", "out", "status", "epilogue", "split_k")
    assert lib.sgr_mlp_gemm(None, None) == INVALID
    g = GemmArgs()
    g.M, g.N, g.K = 8, 8, 16
    assert lib.sgr_mlp_gemm(C.byref(g), None) == INVALID                                   # no status word
    g.status = FAKE
    assert lib.sgr_mlp_gemm(C.byref(g), None) == INVALID                                   # no operands
    g.A = g.B = g.out = FAKE
    g.epilogue = 4
    assert lib.sgr_mlp_gemm(C.byref(g), None) == INVALID                                   # unknown epilogue
    g.epilogue, g.split_k = 0, 5
    assert lib.sgr_mlp_gemm(C.byref(g), None) == INVALID                                   # split not in K chunks
    g.M = 0
    assert lib.sgr_mlp_gemm(C.byref(g), None) == OK                                        # empty product
    assert lib.sgr_mlp_maxpool(FAKE, -1, 4, 4, FAKE, None, FAKE, None) == INVALID
    assert lib.sgr_mlp_maxpool(FAKE, 2, 0, 4, FAKE, None, FAKE, None) == INVALID
    assert lib.sgr_mlp_maxpool(None, 0, 4, 4, None, None, None, None) == OK
    assert lib.sgr_mlp_maxpool_backward(None, None, None, 0, 4, 4, None, None) == OK
    _fields(LossArgs, "V", "H", "W")
    assert lib.sgr_loss_scratch_bytes(None) == 0
    la = LossArgs()
    assert lib.sgr_loss_forward_backward(None, FAKE, FAKE, FAKE, FAKE, None) == INVALID
    assert lib.sgr_loss_forward_backward(C.byref(la), FAKE, FAKE, FAKE, FAKE, None) == INVALID   # V, H, W = 0
    la.V, la.H, la.W = 1, 8, 8
    assert lib.sgr_loss_forward_backward(C.byref(la), FAKE, FAKE, FAKE, FAKE, None) == INVALID   # no inputs
