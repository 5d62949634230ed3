"""Heterogeneous batches (s2let_gpu_px2wav_multi / s2let_gpu_wav2px_multi): maps
with their own band-limit, direction count, spin and reality in one call, as
in the uneven-workload configuration (L log-uniform, N in {1, 3, 5}, spin in
{0, 2}, B = 2, J_min = 1).  Every map must equal the oracle's transform of that
map alone (FP64 path, normwise relative max error <= 1e-12), eagerly, when the
call is captured into a CUDA graph, and when the graph is replayed on new
inputs written to the same buffers."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from s2let_gb300.capi import S2letParameters, make_parameters

TOL = 1e-12


def uneven_maps(seed, n, lmin=16, lmax=64):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        L = int(2 * round(np.exp(rng.uniform(np.log(lmin), np.log(lmax))) / 2))
        N = int(rng.choice([1, 3, 5]))
        spin = int(rng.choice([0, 2]))
        out.append((L, N, spin))
    out.append(out[0])  # a repeated parameter set runs as a batch of two
    out.append(out[1])
    return out


@pytest.mark.gpu
def test_multi_matches_oracle_eager_graph_and_replay(gpu, oracle_port):
    torch = pytest.importorskip("torch")
    lib = gpu.lib
    maps = uneven_maps(4, 8)
    n = len(maps)
    params = (S2letParameters * n)()
    real = (C.c_int * n)()
    px, wav, scal, host_f = [], [], [], []
    rng = np.random.default_rng(5)
    for k, (L, N, spin) in enumerate(maps):
        params[k] = make_parameters(L, 2.0, 1, N, spin, 0)
        real[k] = 1 if spin == 0 else 0
        s = gpu.sizes(params[k])
        dt = torch.float64 if real[k] else torch.complex128
        f = rng.normal(size=s["n_px"]) if real[k] else rng.normal(size=s["n_px"]) + 1j * rng.normal(size=s["n_px"])
        host_f.append(f)
        px.append(torch.from_numpy(f).cuda())
        wav.append(torch.zeros(s["n_wav"], dtype=dt, device="cuda"))
        scal.append(torch.zeros(s["n_scal"], dtype=dt, device="cuda"))
    ptrs = lambda ts: (C.c_void_p * n)(*[t.data_ptr() for t in ts])
    P, W, S = ptrs(px), ptrs(wav), ptrs(scal)
    stream = torch.cuda.Stream()

    def check(fs):
        for k in range(n):
            w0, s0 = oracle_port.px2wav(fs[k], params[k], real=bool(real[k]))
            assert rel_err(wav[k].cpu().numpy(), w0) < TOL, k
            assert rel_err(scal[k].cpu().numpy(), s0) < TOL, k

    for call in range(3):  # eager (plans), capture + launch, replay
        assert lib.s2let_gpu_px2wav_multi(W, S, P, params, real, n, 1, C.c_void_p(stream.cuda_stream)) == 0
        stream.synchronize()
        check(host_f)
    # replay on new inputs written into the same buffers
    for k in range(n):
        host_f[k] = host_f[k] * -0.5 + 0.25
        px[k].copy_(torch.from_numpy(host_f[k]))
    torch.cuda.synchronize()
    assert lib.s2let_gpu_px2wav_multi(W, S, P, params, real, n, 1, C.c_void_p(stream.cuda_stream)) == 0
    stream.synchronize()
    check(host_f)
    # synthesis of the same coefficients: per map against the oracle
    out = [torch.zeros_like(t) for t in px]
    O = ptrs(out)
    for call in range(3):
        assert lib.s2let_gpu_wav2px_multi(O, W, S, params, real, n, 1, C.c_void_p(stream.cuda_stream)) == 0
        stream.synchronize()
        for k in range(n):
            r0 = oracle_port.wav2px(wav[k].cpu().numpy(), scal[k].cpu().numpy(), params[k], real=bool(real[k]))
            assert rel_err(out[k].cpu().numpy(), r0) < TOL, k
    assert lib.s2let_gpu_device_fault() == 0
    gpu.lib.s2let_gpu_release_plans()


@pytest.mark.gpu
def test_multi_rejects_bad_parameters(gpu):
    lib = gpu.lib
    params = (S2letParameters * 1)(make_parameters(16, 1.0, 1, 3, 0, 0))  # B must exceed 1
    real = (C.c_int * 1)(1)
    null = (C.c_void_p * 1)(None)
    assert lib.s2let_gpu_px2wav_multi(null, null, null, params, real, 1, 0, None) == 1
