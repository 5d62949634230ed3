"""FP32 storage (s2let_gpu_*_batch_f32, s2let_gpu_{px2wav,wav2px}_multi_f32 and
float32 / complex64 tensors in the torch operators): maps and coefficients in
single precision, the transforms computed as in the FP64-storage path, the
outputs rounded to single precision.  Each result must equal the FP64-storage
result on the same (single-precision) inputs to within FP32 rounding:
normwise relative max error <= 2e-7 (2^-24 = 6e-8 per value, plus the
rounding of the compared FP64 result).  The unused tail of an f_wav row (a
scale with N_j < N) keeps what the caller wrote."""
import ctypes as C

import pytest

from s2let_gb300.capi import make_parameters

TOL32 = 2e-7
torch = pytest.importorskip("torch")


def _rel(a, b):
    """Normwise relative max error; an all-zero reference (the scaling
    coefficients of a spin signal) compares absolutely."""
    d = float((a.to(b.dtype) - b).abs().max())
    s = float(b.abs().max())
    return d / s if s > 0 else d


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


CASES = [  # L, N, J_min, spin, real, upsample
    (64, 4, 2, 0, True, 0),
    (48, 3, 1, 2, False, 0),
    (32, 5, 2, 0, True, 1),
    (16, 8, 0, 0, True, 0),  # small scales with N_j < N: an unused f_wav tail
]


@pytest.mark.gpu
@pytest.mark.parametrize("L,N,J_min,spin,real,up", CASES)
def test_batch_f32_equals_fp64_rounded(gpu, L, N, J_min, spin, real, up):
    lib = gpu.lib
    p = make_parameters(L, 2.0, J_min, N, spin, up)
    s = gpu.sizes(p)
    nb = 5
    g = torch.Generator().manual_seed(L + N)
    d32 = torch.float32 if real else torch.complex64
    d64 = torch.float64 if real else torch.complex128
    sfx = "_real_batch" if real else "_batch"
    f = torch.randn((nb, s["n_px"]), generator=g, dtype=d32).cuda()
    # analysis: FP32 storage against FP64 storage on the same inputs
    w32 = torch.full((nb, s["n_wav"]), 7.0, dtype=d32, device="cuda")
    s32 = torch.empty((nb, s["n_scal"]), dtype=d32, device="cuda")
    assert getattr(lib, "s2let_gpu_analysis_px2wav" + sfx + "_f32")(_vp(w32), _vp(s32), _vp(f), nb, C.byref(p),
                                                                     _stream()) == 0
    w64 = torch.full((nb, s["n_wav"]), 7.0, dtype=d64, device="cuda")
    s64 = torch.empty((nb, s["n_scal"]), dtype=d64, device="cuda")
    f64 = f.to(d64)
    assert getattr(lib, "s2let_gpu_analysis_px2wav" + sfx)(_vp(w64), _vp(s64), _vp(f64), nb, C.byref(p),
                                                            _stream()) == 0
    torch.cuda.synchronize()
    assert _rel(w32, w64) < TOL32 and _rel(s32, s64) < TOL32
    # the unused tail (if any) still holds the caller's 7.0
    used = int((w64 != 7.0).any(dim=0).nonzero().max()) + 1 if (w64 != 7.0).any() else 0
    assert (w32[:, used:] == 7.0).all()
    # synthesis and both adjoints
    r32 = torch.empty_like(f)
    assert getattr(lib, "s2let_gpu_synthesis_wav2px" + sfx + "_f32")(_vp(r32), _vp(w32), _vp(s32), nb, C.byref(p),
                                                                      _stream()) == 0
    r64 = torch.empty_like(f64)
    w32w, s32w = w32.to(d64), s32.to(d64)
    assert getattr(lib, "s2let_gpu_synthesis_wav2px" + sfx)(_vp(r64), _vp(w32w), _vp(s32w), nb, C.byref(p),
                                                             _stream()) == 0
    torch.cuda.synchronize()
    assert _rel(r32, r64) < TOL32
    a32 = torch.empty_like(f)
    assert getattr(lib, "s2let_gpu_analysis_adjoint_wav2px" + sfx + "_f32")(_vp(a32), _vp(w32), _vp(s32), nb,
                                                                             C.byref(p), _stream()) == 0
    a64 = torch.empty_like(f64)
    assert getattr(lib, "s2let_gpu_analysis_adjoint_wav2px" + sfx)(_vp(a64), _vp(w32w), _vp(s32w), nb,
                                                                    C.byref(p), _stream()) == 0
    bw32 = torch.zeros_like(w32)
    bs32 = torch.empty_like(s32)
    assert getattr(lib, "s2let_gpu_synthesis_adjoint_px2wav" + sfx + "_f32")(_vp(bw32), _vp(bs32), _vp(f), nb,
                                                                              C.byref(p), _stream()) == 0
    bw64 = torch.zeros_like(w64)
    bs64 = torch.empty_like(s64)
    assert getattr(lib, "s2let_gpu_synthesis_adjoint_px2wav" + sfx)(_vp(bw64), _vp(bs64), _vp(f64), nb,
                                                                     C.byref(p), _stream()) == 0
    torch.cuda.synchronize()
    assert _rel(a32, a64) < TOL32
    assert _rel(bw32, bw64) < TOL32 and _rel(bs32, bs64) < TOL32
    assert lib.s2let_gpu_last_error() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [0, 1])
def test_multi_f32_equals_fp64_rounded(gpu, use_graph):
    """Maps with their own parameters (two sharing one set), FP32 storage
    against the FP64 multi-map entry point, three calls in a row (with
    use_graph the second captures a CUDA graph, the third replays it)."""
    lib = gpu.lib
    spec = [(32, 3, 0, True), (48, 5, 2, False), (32, 3, 0, True), (24, 4, 0, True)]
    n = len(spec)
    params = (type(make_parameters(8)) * n)()
    real = (C.c_int * n)()
    bufs32, bufs64 = [], []
    g = torch.Generator().manual_seed(5)
    for k, (L, N, spin, re) in enumerate(spec):
        params[k] = make_parameters(L, 2.0, 1, N, spin, 0)
        real[k] = int(re)
        s = gpu.sizes(params[k])
        d32 = torch.float32 if re else torch.complex64
        d64 = torch.float64 if re else torch.complex128
        f = torch.randn(s["n_px"], generator=g, dtype=d32).cuda()
        bufs32.append([f, torch.zeros(s["n_wav"], dtype=d32, device="cuda"),
                       torch.zeros(s["n_scal"], dtype=d32, device="cuda"), torch.zeros_like(f)])
        bufs64.append([f.to(d64), torch.zeros(s["n_wav"], dtype=d64, device="cuda"),
                       torch.zeros(s["n_scal"], dtype=d64, device="cuda"), torch.zeros_like(f.to(d64))])
    arr = lambda bufs, i: (C.c_void_p * n)(*[b[i].data_ptr() for b in bufs])
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        for _ in range(3):
            assert lib.s2let_gpu_px2wav_multi_f32(arr(bufs32, 1), arr(bufs32, 2), arr(bufs32, 0), params, real, n,
                                                  use_graph, C.c_void_p(st.cuda_stream)) == 0
            assert lib.s2let_gpu_wav2px_multi_f32(arr(bufs32, 3), arr(bufs32, 1), arr(bufs32, 2), params, real, n,
                                                  use_graph, C.c_void_p(st.cuda_stream)) == 0
        assert lib.s2let_gpu_px2wav_multi(arr(bufs64, 1), arr(bufs64, 2), arr(bufs64, 0), params, real, n, 0,
                                          C.c_void_p(st.cuda_stream)) == 0
        assert lib.s2let_gpu_wav2px_multi(arr(bufs64, 3), arr(bufs64, 1), arr(bufs64, 2), params, real, n, 0,
                                          C.c_void_p(st.cuda_stream)) == 0
    st.synchronize()
    for b32, b64 in zip(bufs32, bufs64):
        assert _rel(b32[1], b64[1]) < TOL32 and _rel(b32[2], b64[2]) < TOL32
        # synthesis from the rounded coefficients: FP32 rounding of its inputs and output
        assert _rel(b32[3], b64[3]) < 1e-6
    assert lib.s2let_gpu_last_error() == 0


@pytest.mark.gpu
def test_torch_f32_gradient_matches_fp64():
    """float32 tensors through px2wav -> wav2px with autograd: forward values
    and the gradient of a quadratic loss equal the float64 ones to FP32
    rounding."""
    from s2let_gb300 import torch_ops as T

    p = make_parameters(64, 2.0, 2, 4, 0, 0)
    n = T.sizes(p)["n_px"]
    g = torch.Generator().manual_seed(3)
    x64 = torch.randn((4, n), generator=g, dtype=torch.float64).cuda()
    grads = {}
    for dt in (torch.float32, torch.float64):
        x = x64.to(dt).clone().requires_grad_(True)
        w, s = T.px2wav(x, p)
        loss = 0.5 * (T.wav2px(w * 0.5, s, p) ** 2).sum() + (w ** 2).sum()
        loss.backward()
        grads[dt] = (w.detach(), x.grad.detach())
    assert grads[torch.float32][0].dtype == torch.float32
    assert grads[torch.float32][1].dtype == torch.float32
    assert _rel(grads[torch.float32][0], grads[torch.float64][0]) < 1e-6
    assert _rel(grads[torch.float32][1], grads[torch.float64][1]) < 1e-5
