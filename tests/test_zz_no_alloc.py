"""sgr_bind_backward_static (the binding backward with its scratch in the
library's fixed device array) against sgr_bind_backward (caller scratch),
called through the C ABI on the block-level workload's shapes: 8
superquadrics, 2,500 surfels each.  Two calls in a row check that the fixed
scratch is cleared between calls."""
import ctypes as C

import pytest
import torch

from oracle import binding_oracle as B

pytestmark = pytest.mark.gpu

NAMES = ["sq_s", "sq_r", "sq_t", "sq_eps", "sq_occ"]
# Relative to each gradient's largest magnitude: the bar of the binding
# adjoint test.  The per-vertex sums are float atomics, whose order differs
# from run to run, and the rotation gradient cancels (seen: 2e-5 between two
# runs of the same entry point).
TOL = 1e-4


def _static_fn(lib):
    from partgs_gb300 import _lib as L
    fn = lib.sgr_bind_backward_static
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(L.BindArgs)] + [C.c_void_p] * 10
    return fn


def _setup(seed=0, n_eta=50, n_omega=50):
    from partgs_gb300.binding import SuperquadricBinding
    inp = B.random_binding_inputs(B=8, n_eta=n_eta, n_omega=n_omega, N=1, seed=seed)
    topo = SuperquadricBinding(inp["eta"].cuda(), inp["omega"].cuda(), inp["faces"].cuda(), inp["alpha_raw"].cuda(),
                               inp["scale"].cuda(), inp["ratio_block_scene"], inp["scale_block_min"])
    params = [inp[k].float().cuda().contiguous() for k in NAMES]
    params[4] = params[4].reshape(-1, 1).contiguous()
    n = topo.num_surfels
    g = torch.Generator().manual_seed(seed + 1)
    ups = [torch.randn(n, d, generator=g).cuda() for d in (3, 2, 4, 1)]
    return topo, params, ups


def _grads_like(params):
    return [torch.full_like(p, float("nan")) for p in params]


def test_static_scratch_backward_matches_caller_scratch(sgr_lib):
    from partgs_gb300 import _lib as L
    lib = L.load()
    fn = _static_fn(lib)
    topo, params, ups = _setup()
    a, keep = topo.args(*params)
    st = torch.cuda.current_stream().cuda_stream
    ref = _grads_like(params)
    scratch = torch.empty(lib.sgr_bind_scratch_bytes(C.byref(a)), dtype=torch.uint8, device="cuda")
    assert scratch.numel() <= 4 << 20
    L.check(lib.sgr_bind_backward(C.byref(a), *(u.data_ptr() for u in ups), *(g.data_ptr() for g in ref),
                                  scratch.data_ptr(), st), "sgr_bind_backward")
    for call in range(2):
        mine = _grads_like(params)
        rc = fn(C.byref(a), *(u.data_ptr() for u in ups), *(g.data_ptr() for g in mine), st)
        assert rc == 0, lib.sgr_last_error_message()
        torch.cuda.synchronize()
        for k, m, r in zip(NAMES, mine, ref):
            assert torch.isfinite(m).all(), (call, k)
            scale = float(r.abs().max())
            err = float((m - r).abs().max()) / max(scale, 1e-30)
            assert err <= TOL, (call, k, err)
    del keep


def test_static_scratch_rejects_shapes_beyond_its_size(sgr_lib):
    from partgs_gb300 import _lib as L
    lib = L.load()
    fn = _static_fn(lib)
    topo, params, ups = _setup(seed=2, n_eta=200, n_omega=200)    # 8 x 40,000 vertices: 5.1 MB of scratch
    a, keep = topo.args(*params)
    assert lib.sgr_bind_scratch_bytes(C.byref(a)) > 4 << 20
    out = _grads_like(params)
    rc = fn(C.byref(a), *(u.data_ptr() for u in ups), *(g.data_ptr() for g in out),
            torch.cuda.current_stream().cuda_stream)
    assert rc == 4                                         # SGR_ERR_WORKSPACE
    msg = lib.sgr_last_error_message().decode()
    assert "sgr_bind_backward_static" in msg and str(4 << 20) in msg
    torch.cuda.synchronize()
    assert all(torch.isnan(g).all() for g in out)          # nothing ran
    del keep
