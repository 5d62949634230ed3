"""PyTorch autograd operators over the batched device entry points.

``px2wav(f, p)`` and ``wav2px(f_wav, f_scal, p)`` take CUDA tensors with a
leading batch dimension: f is (batch, n_px), f_wav (batch, n_wav), f_scal
(batch, n_scal) in the reference's MW / wavelet layouts
(src/c/s2let_analysis.c:456-523, src/c/s2let_synthesis.c:472-539).  Real
signals use float64 tensors, spin / complex signals complex128; float32 /
complex64 tensors select the FP32-storage entry points (the same transforms on
FP64 copies made on the device, the outputs rounded to single precision), and
the outputs and gradients keep the input's precision.

Backward passes run the hand-written adjoint kernels
(s2let_gpu_analysis_adjoint_wav2px*_batch, s2let_gpu_synthesis_adjoint_px2wav*_batch),
not the inverse transform: MW quadrature is not self-adjoint, so the inverse
is not the transpose.  For complex tensors PyTorch passes dL/d(conj y) and the
adjoint A^H maps it to dL/d(conj x), which is what these functions return.

Precision: ``precision="fp64"`` (default) or ``"mixed"`` (split-precision
tensor-core contraction, within 1e-10 of FP64) for forward and backward; the
choice is applied on the thread that runs each pass (autograd runs backward on
its own thread).  There is no CPU path: the library raises when no GPU is
present.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .capi import S2letParameters, make_parameters

__all__ = ["px2wav", "wav2px", "Px2Wav", "Wav2Px", "make_parameters", "sizes"]

_PREC = {"fp64": 0, "mixed": 1}


def _lib_handle():
    return _lib.load()


def sizes(p: S2letParameters) -> dict:
    lib = _lib_handle()
    r = C.byref(p)
    return dict(n_px=lib.s2let_n_px(r), n_wav=lib.s2let_n_wav(r), n_scal=lib.s2let_n_scal(r))


def _single(t: torch.Tensor) -> bool:
    return t.dtype in (torch.float32, torch.complex64)


def _dtype(real: bool, single: bool):
    if single:
        return torch.float32 if real else torch.complex64
    return torch.float64 if real else torch.complex128


def _check(t: torch.Tensor, name: str, n: int, real: bool, single: bool = False) -> torch.Tensor:
    want = _dtype(real, single)
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dim() != 2 or t.shape[1] != n:
        raise ValueError(f"{name} must have shape (batch, {n}), got {tuple(t.shape)}")
    if t.dtype != want:
        t = t.to(want)
    return t.contiguous()


def _call(fn: str, args, precision: str, device) -> None:
    """One library call at the given precision; the calling thread's precision
    mode is restored afterwards, so C-ABI calls made later on the same thread
    keep their own setting."""
    lib = _lib_handle()
    if precision not in _PREC:
        raise ValueError(f"precision must be one of {list(_PREC)}")
    with torch.cuda.device(device):
        stream = C.c_void_p(torch.cuda.current_stream(device).cuda_stream)
        old = lib.s2let_gpu_get_precision()
        lib.s2let_gpu_set_precision(_PREC[precision])
        try:
            rc = getattr(lib, fn)(*args, stream)
        finally:
            lib.s2let_gpu_set_precision(old)
    if rc != 0:
        raise RuntimeError(f"{fn}: {lib.s2let_gpu_last_error_string().decode()}")


def _ptr(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _suffix(real: bool, single: bool = False) -> str:
    return ("_real_batch" if real else "_batch") + ("_f32" if single else "")


class Px2Wav(torch.autograd.Function):
    """f -> (f_wav, f_scal); backward: the adjoint of analysis."""

    @staticmethod
    def forward(ctx, f, p: S2letParameters, real: bool, precision: str):
        s = sizes(p)
        single = _single(f)
        f = _check(f, "f", s["n_px"], real, single)
        nb = f.shape[0]
        w = torch.empty((nb, s["n_wav"]), dtype=f.dtype, device=f.device)
        sc = torch.empty((nb, s["n_scal"]), dtype=f.dtype, device=f.device)
        _call("s2let_gpu_analysis_px2wav" + _suffix(real, single), (_ptr(w), _ptr(sc), _ptr(f), nb, C.byref(p)),
              precision, f.device)
        ctx.p, ctx.real, ctx.precision, ctx.sizes, ctx.single = p, real, precision, s, single
        return w, sc

    @staticmethod
    def backward(ctx, gw, gsc):
        p, real, s, single = ctx.p, ctx.real, ctx.sizes, ctx.single
        dev = gw.device if gw is not None else gsc.device
        dt = _dtype(real, single)
        nb = (gw if gw is not None else gsc).shape[0]
        gw = (torch.zeros((nb, s["n_wav"]), dtype=dt, device=dev) if gw is None
              else _check(gw, "grad f_wav", s["n_wav"], real, single))
        gsc = (torch.zeros((nb, s["n_scal"]), dtype=dt, device=dev) if gsc is None
               else _check(gsc, "grad f_scal", s["n_scal"], real, single))
        gf = torch.empty((nb, s["n_px"]), dtype=dt, device=dev)
        _call("s2let_gpu_analysis_adjoint_wav2px" + _suffix(real, single),
              (_ptr(gf), _ptr(gw), _ptr(gsc), nb, C.byref(p)), ctx.precision, dev)
        return gf, None, None, None


class Wav2Px(torch.autograd.Function):
    """(f_wav, f_scal) -> f; backward: the adjoint of synthesis."""

    @staticmethod
    def forward(ctx, f_wav, f_scal, p: S2letParameters, real: bool, precision: str):
        s = sizes(p)
        single = _single(f_wav)
        f_wav = _check(f_wav, "f_wav", s["n_wav"], real, single)
        f_scal = _check(f_scal, "f_scal", s["n_scal"], real, single)
        nb = f_wav.shape[0]
        if f_scal.shape[0] != nb:
            raise ValueError("f_wav and f_scal batch sizes differ")
        f = torch.empty((nb, s["n_px"]), dtype=f_wav.dtype, device=f_wav.device)
        _call("s2let_gpu_synthesis_wav2px" + _suffix(real, single),
              (_ptr(f), _ptr(f_wav), _ptr(f_scal), nb, C.byref(p)), precision, f_wav.device)
        ctx.p, ctx.real, ctx.precision, ctx.sizes, ctx.single = p, real, precision, s, single
        return f

    @staticmethod
    def backward(ctx, gf):
        p, real, s, single = ctx.p, ctx.real, ctx.sizes, ctx.single
        gf = _check(gf, "grad f", s["n_px"], real, single)
        nb = gf.shape[0]
        gw = torch.empty((nb, s["n_wav"]), dtype=gf.dtype, device=gf.device)
        gsc = torch.empty((nb, s["n_scal"]), dtype=gf.dtype, device=gf.device)
        _call("s2let_gpu_synthesis_adjoint_px2wav" + _suffix(real, single),
              (_ptr(gw), _ptr(gsc), _ptr(gf), nb, C.byref(p)), ctx.precision, gf.device)
        return gw, gsc, None, None, None


def px2wav(f: torch.Tensor, p: S2letParameters, real: bool | None = None, precision: str = "fp64"):
    """Batched differentiable analysis; real defaults to (f is real)."""
    if real is None:
        real = not torch.is_complex(f)
    return Px2Wav.apply(f, p, real, precision)


def wav2px(f_wav: torch.Tensor, f_scal: torch.Tensor, p: S2letParameters, real: bool | None = None,
           precision: str = "fp64"):
    """Batched differentiable synthesis; real defaults to (f_wav is real)."""
    if real is None:
        real = not torch.is_complex(f_wav)
    return Wav2Px.apply(f_wav, f_scal, p, real, precision)
