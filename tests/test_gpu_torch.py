"""torch.autograd operators (s2let_gb300.torch_ops) over the batched device API.

Backward passes are the hand-written adjoint kernels.  Checked three ways, as
the reference's own adjoint tests do (test/c/s2let_test_adjoint.c: dot products
<A x, y> = <x, A* y>, relative 1e-12 in FP64), plus central finite differences
of a wavelet-sparsity loss and the mixed-precision gradient against FP64."""
import pytest

torch = pytest.importorskip("torch")

from s2let_gb300 import torch_ops as T  # noqa: E402
from s2let_gb300.capi import make_parameters  # noqa: E402

DEV = "cuda"


def _inner(a, b):
    """Real inner product Re <a, b> over all entries (complex: sum a conj b)."""
    a, b = a.detach(), b.detach()
    return float(torch.sum(a * b.conj()).real) if torch.is_complex(a) else float(torch.sum(a * b))


def _rand(shape, complex_, gen):
    x = torch.rand(shape, dtype=torch.float64, generator=gen) * 2 - 1
    if complex_:
        x = torch.complex(x, torch.rand(shape, dtype=torch.float64, generator=gen) * 2 - 1)
    return x.to(DEV)


@pytest.mark.gpu
@pytest.mark.parametrize("L,N,spin,real", [(16, 4, 0, True), (24, 3, 2, False), (17, 5, 0, True)])
def test_adjoint_dot_products(L, N, spin, real):
    p = make_parameters(L, 2.0, 1, N, spin, 0)
    s = T.sizes(p)
    g = torch.Generator().manual_seed(L)
    x = _rand((3, s["n_px"]), not real, g).requires_grad_(True)
    vw, vs = _rand((3, s["n_wav"]), not real, g), _rand((3, s["n_scal"]), not real, g)
    w, sc = T.px2wav(x, p, real=real)
    lhs = _inner(w, vw) + _inner(sc, vs)
    (gx,) = torch.autograd.grad((torch.sum((w * vw.conj()).real) + torch.sum((sc * vs.conj()).real)) if not real
                                else (torch.sum(w * vw) + torch.sum(sc * vs)), x)
    rhs = _inner(x.detach(), gx)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)

    a = _rand((3, s["n_wav"]), not real, g).requires_grad_(True)
    b = _rand((3, s["n_scal"]), not real, g).requires_grad_(True)
    v = _rand((3, s["n_px"]), not real, g)
    f = T.wav2px(a, b, p, real=real)
    lhs = _inner(f, v)
    ga, gb = torch.autograd.grad(torch.sum((f * v.conj()).real) if not real else torch.sum(f * v), (a, b))
    rhs = _inner(a.detach(), ga) + _inner(b.detach(), gb)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


def _sparsity_loss(x, y, p, lam, thr, precision):
    w, sc = T.px2wav(x, p, precision=precision)
    ws = torch.sign(w) * torch.clamp(w.abs() - thr, min=0.0)
    r = T.wav2px(ws, sc, p, precision=precision) - y
    return 0.5 * torch.sum(r * r) + lam * torch.sum(w.abs())


def _fd_check(L, lam, thr, seed):
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    s = T.sizes(p)
    g = torch.Generator().manual_seed(seed)
    y = _rand((2, s["n_px"]), False, g)
    x = (y + 0.1 * _rand((2, s["n_px"]), False, g)).requires_grad_(True)
    loss = _sparsity_loss(x, y, p, lam, thr, "fp64")
    (gx,) = torch.autograd.grad(loss, x)
    d = _rand((2, s["n_px"]), False, g)
    h = 1e-3
    with torch.no_grad():
        lp = _sparsity_loss(x + h * d, y, p, lam, thr, "fp64")
        lm = _sparsity_loss(x - h * d, y, p, lam, thr, "fp64")
    fd = float((lp - lm) / (2 * h))
    an = float(torch.sum(gx * d))
    return fd, an


@pytest.mark.gpu
def test_quadratic_loss_finite_differences():
    """No threshold, no L1 term: the loss is quadratic in x, so the central
    difference (h = 1e-3) equals the directional derivative up to rounding."""
    fd, an = _fd_check(24, 0.0, 0.0, 5)
    assert abs(fd - an) <= 1e-9 * max(abs(an), 1.0)


@pytest.mark.gpu
def test_sparsity_loss_finite_differences():
    """Soft threshold and L1 term: the loss is piecewise quadratic, and the
    coefficients that cross a kink inside +-h leave an O(h) difference; the
    tolerance is set by that, not by the adjoints (checked exactly above)."""
    fd, an = _fd_check(24, 1e-3, 1e-2, 5)
    assert abs(fd - an) <= 5e-3 * max(abs(an), 1.0)


@pytest.mark.gpu
def test_mixed_gradient_matches_fp64():
    L = 256
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    s = T.sizes(p)
    g = torch.Generator().manual_seed(8)
    y = _rand((2, s["n_px"]), False, g)
    x0 = y + 0.1 * _rand((2, s["n_px"]), False, g)
    grads = {}
    for prec in ("fp64", "mixed"):
        x = x0.clone().requires_grad_(True)
        loss = _sparsity_loss(x, y, p, 1e-3, 1e-2, prec)
        (grads[prec],) = torch.autograd.grad(loss, x)
    err = float((grads["mixed"] - grads["fp64"]).abs().max() / grads["fp64"].abs().max())
    assert err < 1e-10


@pytest.mark.gpu
def test_batch_equals_single():
    L = 20
    p = make_parameters(L, 2.0, 1, 3, 0, 0)
    s = T.sizes(p)
    g = torch.Generator().manual_seed(2)
    x = _rand((3, s["n_px"]), False, g)
    w, sc = T.px2wav(x, p)
    for b in range(3):
        wb, sb = T.px2wav(x[b:b + 1], p)
        assert torch.equal(wb[0], w[b]) and torch.equal(sb[0], sc[b])


@pytest.mark.gpu
def test_rejects_bad_shapes():
    p = make_parameters(16, 2.0, 1, 4, 0, 0)
    with pytest.raises(ValueError):
        T.px2wav(torch.zeros((2, 7), dtype=torch.float64, device=DEV), p)
    with pytest.raises(ValueError):
        T.px2wav(torch.zeros((2, T.sizes(p)["n_px"]), dtype=torch.float64), p)


@pytest.mark.gpu
def test_precision_mode_restored(gpu):
    """A mixed-precision torch call leaves the thread's precision mode as it
    found it, so later C-ABI calls on the thread keep their own setting."""
    lib = gpu.lib
    old = lib.s2let_gpu_get_precision()
    assert lib.s2let_gpu_set_precision(0) == 0
    try:
        p = make_parameters(160, 2.0, 2, 3, 0, 0)
        x = _rand((2, T.sizes(p)["n_px"]), False, torch.Generator().manual_seed(3))
        w, s = T.px2wav(x, p, precision="mixed")
        T.wav2px(w, s, p, precision="mixed")
        assert lib.s2let_gpu_get_precision() == 0
        with pytest.raises(ValueError):
            T.px2wav(x, p, precision="fp16")
        assert lib.s2let_gpu_get_precision() == 0
    finally:
        lib.s2let_gpu_set_precision(old)
