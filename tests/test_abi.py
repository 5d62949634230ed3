"""CPU tests of the C-ABI library libs2let_gpu.so: it loads without a GPU,
exports every function include/s2let_gpu.h declares, lays out
s2let_parameters_t as the reference does, computes the host-side helpers
(sizes, band-limits, tilings) exactly as the oracle, and reports errors through
its status API instead of exiting."""
import ctypes as C
import os
import shutil
import re
import subprocess
import tempfile

import numpy as np
import pytest

from s2let_gb300.capi import S2letParameters, make_parameters, ptr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "s2let_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(s2let_\w+|binomial_coefficient)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import s2let_gb300

    return s2let_gb300.load()


def test_exports_every_declared_function(lib):
    names = declared_functions()
    assert len(names) > 100
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_parameters_struct_layout_matches_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "s2let_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(s2let_parameters_t),
    offsetof(s2let_parameters_t, verbosity), offsetof(s2let_parameters_t, reality),
    offsetof(s2let_parameters_t, upsample), offsetof(s2let_parameters_t, B),
    offsetof(s2let_parameters_t, L), offsetof(s2let_parameters_t, J_min),
    offsetof(s2let_parameters_t, N), offsetof(s2let_parameters_t, spin),
    offsetof(s2let_parameters_t, original_spin), offsetof(s2let_parameters_t, sampling_scheme),
    offsetof(s2let_parameters_t, dl_method));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-std=c99", f"-I{ROOT}/include", c, "-o", exe], check=True)
        vals = list(map(int, subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()))
    f = S2letParameters
    py = [C.sizeof(f)] + [getattr(f, n).offset for n, _ in f._fields_]
    assert vals == py


PARAMS = [(16, 4, 2.0, 2, 0, 0), (16, 4, 2.0, 2, 2, 1), (17, 3, 2.5, 1, 1, 0), (12, 5, 2.0, 0, 0, 0),
          (1024, 4, 2.0, 2, 0, 0), (100, 7, 1.7, 3, 3, 0), (64, 1, 3.0, 0, 0, 1)]


@pytest.mark.parametrize("case", PARAMS)
def test_host_helpers_match_oracle(lib, oracle_port, case):
    L, N, B, J_min, spin, up = case
    for real in (0, 1):
        p = make_parameters(L, B, J_min, N, spin, up, reality=real)
        r = C.byref(p)
        for fn in ("s2let_n_phi", "s2let_n_theta", "s2let_n_px", "s2let_n_lm", "s2let_n_lm_scal",
                   "s2let_n_lmn_wav", "s2let_n_gamma", "s2let_n_scal", "s2let_n_wav", "s2let_j_max"):
            assert getattr(lib, fn)(r) == getattr(oracle_port.lib, fn)(r), fn
        J = lib.s2let_j_max(r)
        for j in range(-1, J + 2):
            assert lib.s2let_bandlimit(j, r) == oracle_port.lib.s2let_bandlimit(j, r)
            assert lib.s2let_L0(j, r) == oracle_port.lib.s2let_L0(j, r)
            assert lib.s2let_n_wav_j(j, r) == oracle_port.lib.s2let_n_wav_j(j, r)


@pytest.mark.parametrize("case", PARAMS[:4] + [(64, 3, 2.0, 1, 0, 0)])
@pytest.mark.parametrize("kernel", [1, 2, 3])
def test_tiling_matches_oracle_bitwise(lib, oracle_port, case, kernel):
    from s2let_gb300.capi import S2let

    L, N, B, J_min, spin, up = case
    p = make_parameters(L, B, J_min, N, spin, up, original_spin=1 if spin else 0)
    try:
        lib.s2let_switch_wavtype(kernel)
        oracle_port.lib.s2let_switch_wavtype(kernel)
        a = S2let(lib).tiling(p)
        b = oracle_port.tiling(p)
    finally:
        lib.s2let_switch_wavtype(1)
        oracle_port.lib.s2let_switch_wavtype(1)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def test_invalid_parameters_report_status(lib):
    f = np.zeros(16 * 31)
    w = np.zeros(10)
    s = np.zeros(10)
    for bad in (make_parameters(0, 2.0, 0, 1), make_parameters(16, 1.0, 0, 1), make_parameters(16, 2.0, 0, 0),
                make_parameters(16, 2.0, 9, 1), make_parameters(16, 2.0, 0, 1, spin=16)):
        lib.s2let_analysis_px2wav_real(ptr(w), ptr(s), ptr(f), C.byref(bad))
        assert lib.s2let_gpu_last_error() == 1, lib.s2let_gpu_last_error_string()
    # MW and MWSS are the two schemes; anything else is "not supported"
    # (src/c/s2let_analysis.c:244-245)
    unknown = make_parameters(16, 2.0, 0, 1, sampling_scheme=2)
    lib.s2let_analysis_px2wav_real(ptr(w), ptr(s), ptr(f), C.byref(unknown))
    assert lib.s2let_gpu_last_error() == 2
    assert np.all(w == 0) and np.all(s == 0)


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_no_device_reports_status_and_leaves_outputs(lib):
    p = make_parameters(16, 2.0, 2, 4)
    f = np.ones(16 * 31)
    w = np.full(lib.s2let_n_wav(C.byref(p)), 7.0)
    s = np.full(lib.s2let_n_scal(C.byref(p)), 7.0)
    lib.s2let_analysis_px2wav_real(ptr(w), ptr(s), ptr(f), C.byref(p))
    assert lib.s2let_gpu_last_error() == 5
    assert b"no CUDA device" in lib.s2let_gpu_last_error_string()
    assert np.all(w == 7.0) and np.all(s == 7.0)


def test_precision_mode_switch(lib):
    assert lib.s2let_gpu_set_precision(1) == 0
    assert lib.s2let_gpu_get_precision() == 1
    assert lib.s2let_gpu_set_precision(5) == 1
    assert lib.s2let_gpu_set_precision(0) == 0


def test_double_float_contraction_switches(lib):
    """The batch limit of the double-float contraction (0-4 maps) and the
    double-float table copies (0/1): out-of-range values are refused with
    S2LET_GPU_ERR_INVALID and leave the setting unchanged."""
    old_max, old_tab = lib.s2let_gpu_get_df_max_maps(), lib.s2let_gpu_get_split_tables()
    try:
        for n in (0, 4, 2):
            assert lib.s2let_gpu_set_df_max_maps(n) == 0
            assert lib.s2let_gpu_get_df_max_maps() == n
        assert lib.s2let_gpu_set_df_max_maps(5) == 1 and lib.s2let_gpu_set_df_max_maps(-1) == 1
        assert lib.s2let_gpu_get_df_max_maps() == 2
        for on in (0, 1):
            assert lib.s2let_gpu_set_split_tables(on) == 0
            assert lib.s2let_gpu_get_split_tables() == on
        assert lib.s2let_gpu_set_split_tables(2) == 1
        assert lib.s2let_gpu_get_split_tables() == 1
    finally:
        lib.s2let_gpu_set_df_max_maps(old_max)
        lib.s2let_gpu_set_split_tables(old_tab)


RELINK = r"""
/* A caller written against the reference's API (s2let.h), relinked against
   libs2let_gpu: allocation helpers, sizes, the tiling, and a transform whose
   status it reads back.  S2LET_HEADER is <s2let.h> or <s2let/s2let.h>. */
#include <string.h>
#include <stdio.h>
#include <stdlib.h>
#include S2LET_HEADER
int main(void) {
  s2let_parameters_t p;
  memset(&p, 0, sizeof p);
  p.L = 16; p.B = 2.0; p.J_min = 1; p.N = 3; p.reality = 1;
  p.sampling_scheme = S2LET_SAMPLING_MW;
  double *f, *f_wav, *f_scal;
  s2let_allocate_mw_real(&f, p.L);
  s2let_allocate_f_wav_real(&f_wav, &f_scal, &p);
  for (int i = 0; i < p.L * (2 * p.L - 1); ++i) f[i] = 0.01 * i;
  s2let_analysis_px2wav_real(f_wav, f_scal, f, &p);
  printf("%d %d %d %d\n", s2let_n_px(&p), s2let_j_max(&p), s2let_bandlimit(2, &p), s2let_gpu_last_error());
  free(f); free(f_wav); free(f_scal);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_reference_style_c_caller_relinks(lib, tmp_path):
    """The drop-in claim at the C level: a program using only reference
    names and the reference's header (s2let.h, forwarding to
    include/s2let_gpu.h) builds unchanged and links -ls2let_gpu; sizes and
    band-limits come out as the reference computes them, and the transform's
    status is 0 with a GPU, S2LET_GPU_ERR_NO_DEVICE without."""
    import s2let_gb300

    libdir = os.path.dirname(s2let_gb300.LIB_PATH)
    # the reference's own include forms: <s2let.h> with -I.../include/s2let, and
    # <s2let/s2let.h> with -I.../include; as C99 and as C++ (std::complex)
    builds = [("gcc", "c", "-std=c99", "<s2let.h>", f"-I{ROOT}/include/s2let"),
              ("gcc", "c", "-std=c99", "<s2let/s2let.h>", f"-I{ROOT}/include"),
              ("g++", "cpp", "-std=c++17", "<s2let.h>", f"-I{ROOT}/include/s2let")]
    for k, (cc, ext, std, header, inc) in enumerate(builds):
        if shutil.which(cc) is None:
            continue
        src, exe = tmp_path / f"caller{k}.{ext}", tmp_path / f"caller{k}"
        src.write_text(RELINK.replace("S2LET_HEADER", header))
        subprocess.run([cc, std, "-Wall", "-Werror", inc, str(src), f"-L{libdir}", "-ls2let_gpu",
                        f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
        n_px, j_max, bl2, status = map(int, out)
        assert n_px == 16 * 31 and j_max == 4 and bl2 == 8
        assert status == (0 if _has_gpu() else 5)


def test_device_binding_guard():
    """One device per process: the first device (named explicitly here, as no
    GPU is present) is kept; naming another is refused with
    S2LET_GPU_ERR_UNSUPPORTED and leaves the binding unchanged.  Runs in a
    fresh interpreter so that no earlier call has bound the library."""
    code = r'''
import s2let_gb300
lib = s2let_gb300.load()
out = [lib.s2let_gpu_bound_device(), lib.s2let_gpu_bind_device(-1), lib.s2let_gpu_bound_device(),
       lib.s2let_gpu_bind_device(0), lib.s2let_gpu_bound_device(), lib.s2let_gpu_bind_device(0),
       lib.s2let_gpu_bind_device(1), lib.s2let_gpu_last_error(), lib.s2let_gpu_bound_device()]
print(" ".join(map(str, out)))
'''
    r = subprocess.run([os.sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in r.stdout.split()]
    #      unbound, bind(-1) invalid, still unbound, bind(0), bound 0, again ok, bind(1) refused, status, still 0
    assert got == [-1, 1, -1, 0, 0, 0, 2, 2, 0]
    assert "already serves CUDA device 0" in r.stderr
