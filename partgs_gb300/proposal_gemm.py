"""Host side of the proposal network's BF16 tensor-core GEMM (libsgr.so
``sgr_mlp_gemm``): C[M, N] = A[M, K] . B[N, K]^T with a fused epilogue."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L

STORE_F32, ADD_F32, RELU_BF16, MASK_BF16 = 0, 1, 2, 3
TIMEOUT = 1
_p = C.c_void_p


class GemmArgs(C.Structure):
    _fields_ = [("M", C.c_int64), ("N", C.c_int64), ("K", C.c_int64), ("A", _p), ("lda", C.c_int64),
                ("a_trans", C.c_int32), ("B", _p), ("ldb", C.c_int64), ("b_trans", C.c_int32), ("bias", _p),
                ("epilogue", C.c_int32), ("out", _p), ("ldo", C.c_int64), ("mask", _p), ("ldmask", C.c_int64),
                ("split_k", C.c_int64), ("status", _p), ("skip_loads", C.c_int32)]


_STATUS: dict = {}


def _lib():
    lib = L.load()
    fn = lib.sgr_mlp_gemm
    fn.restype, fn.argtypes = C.c_int, [C.POINTER(GemmArgs), _p]
    return lib


def status_word(device) -> torch.Tensor:
    """The device status word every GEMM on ``device`` ORs its flags into."""
    key = torch.device(device)
    if key not in _STATUS:
        _STATUS[key] = torch.zeros(1, dtype=torch.int32, device=key)
    return _STATUS[key]


def check_status(device) -> None:
    """Raises if any GEMM on ``device`` since the last check ran out of time
    waiting for the tensor cores or a copy (its output is then incomplete),
    and clears the word.  Synchronises with the device."""
    w = status_word(device)
    flags = int(w.item())
    if flags:
        w.zero_()
        raise RuntimeError(f"tensor-core GEMM status {flags:#x}: a wait ran out (SGR_MLP_TIMEOUT); "
                           "the outputs of the calls since the last check are incomplete")


def gemm(a, b, out, epilogue, bias=None, mask=None, trans=False, split_k=0, skip_loads=False):
    """out (+)= epilogue(a . b^T + bias).  Without ``trans``: a [M, K], b
    [N, K] (bf16, K contiguous).  With it: a [K, M], b [K, N] (the reduction
    runs over their rows).  ``out`` is [M, N] (fp32, or bf16 for the ReLU
    epilogues)."""
    if a.dtype != torch.bfloat16 or b.dtype != torch.bfloat16:
        raise TypeError("gemm operands are bf16")
    if not (a.is_contiguous() and b.is_contiguous() and out.is_contiguous()):
        raise ValueError("gemm operands must be contiguous")
    if trans:
        K, M = a.shape
        K2, N = b.shape
    else:
        M, K = a.shape
        N, K2 = b.shape
    if K != K2 or tuple(out.shape) != (M, N):
        raise ValueError("gemm shapes do not agree")
    want = torch.float32 if epilogue in (STORE_F32, ADD_F32) else torch.bfloat16
    if out.dtype != want:
        raise TypeError(f"epilogue {epilogue} writes {want}")
    args = GemmArgs(M, N, K, a.data_ptr(), a.shape[1], int(trans), b.data_ptr(), b.shape[1], int(trans),
                    bias.data_ptr() if bias is not None else None, epilogue, out.data_ptr(), N,
                    mask.data_ptr() if mask is not None else None, mask.shape[1] if mask is not None else 0,
                    split_k, status_word(out.device).data_ptr(), int(bool(skip_loads)))
    L.check(_lib().sgr_mlp_gemm(C.byref(args), torch.cuda.current_stream().cuda_stream), "sgr_mlp_gemm")
    return out


def main():
    """python -m partgs_gb300.proposal_gemm: CUDA-event timings of the
    network's per-point layer shapes at 128 and 256 scenes of 2,048 points
    (262,144 and 524,288 rows), this GEMM (bias + ReLU fused, bf16 out)
    against PyTorch's cuBLAS GEMM with the bias (F.linear) followed by ReLU,
    both as device time inside a CUDA graph.  One JSON line per shape.  Operands larger than the 129 MB L2 are read
    from HBM every launch; the smaller ones partly stay in L2 for both."""
    import json

    def timed(fn, n=20):
        """Device time per call: n calls captured in one CUDA graph, the
        replay timed with CUDA events (so host launch overhead, which is
        larger than the small layers' device time, is not measured)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(3):
                fn()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for _ in range(n):
                fn()
        graph.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        graph.replay()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n * 1e-3
    g = torch.Generator().manual_seed(0)
    for M in (262144, 524288):
        for N, K in ((64, 16), (128, 64), (256, 128)):
            a = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
            b = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
            bias = torch.randn(N, generator=g).cuda()
            bias16 = bias.to(torch.bfloat16)
            out = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
            t = timed(lambda: gemm(a, b, out, RELU_BF16, bias=bias))
            t_ref = timed(lambda: torch.relu(torch.nn.functional.linear(a, b, bias16)))
            check_status(out.device)
            nbytes = (M * K + N * K + M * N) * 2
            print(json.dumps({"M": M, "N": N, "K": K, "us": round(t * 1e6, 2), "tflops": round(2 * M * N * K / t / 1e12, 1),
                              "gbs": round(nbytes / t / 1e9), "cublas_linear_relu_us": round(t_ref * 1e6, 2),
                              "speedup_vs_cublas": round(t_ref / t, 3)}), flush=True)


if __name__ == "__main__":
    main()
