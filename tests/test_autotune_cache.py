"""The autotuner's cache file, read on the CPU (no GPU needed): lines of other
GPU models are ignored, a later line for a key replaces an earlier one, and
s2let_gpu_autotune_entries lists the choices with their timings.  Without a
device the GPU model reads as "unknown", which the lines below name.  Runs in
a child process because the file is read once per process."""
import os
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import ctypes as C, sys
    sys.path.insert(0, %r)
    import s2let_gb300
    lib = s2let_gb300.load()
    keys = (C.c_int * 50)()
    ms = (C.c_double * 20)()
    n = lib.s2let_gpu_autotune_entries(keys, ms, 10)
    print(n)
    for i in range(n):
        print(*[keys[5 * i + j] for j in range(5)], ms[2 * i], ms[2 * i + 1])
    old = lib.s2let_gpu_autotune(1)
    print("mode", old, lib.s2let_gpu_autotune(0))
""") % ROOT


def test_cache_file_is_read(tmp_path):
    import pytest

    lib_path = os.path.join(ROOT, "s2let_gb300", "lib", "libs2let_gpu.so")
    if not os.path.exists(lib_path):
        pytest.skip("library not built")
    cache = tmp_path / "tune.txt"
    cache.write_text(
        "unknown 1 0 1024 16 3 1.5 2.0\n"
        "Other_GPU 1 0 1024 16 0 9.0 9.0\n"
        "unknown 4 1024 64 1 6 12.25 12.25\n"
        "unknown 1 0 1024 16 2 1.25 2.0\n")
    env = dict(os.environ, S2LET_GPU_AUTOTUNE_CACHE=str(cache), CUDA_VISIBLE_DEVICES="")
    env.pop("S2LET_GPU_AUTOTUNE", None)
    out = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.split("\n")
    assert lines[0] == "2"
    got = sorted(tuple(float(x) for x in ln.split()) for ln in lines[1:3])
    # (family, a, b, c, choice, best ms, built-in ms); the later line of key (1, 0, 1024, 16) wins
    assert got == [(1, 0, 1024, 16, 2, 1.25, 2.0), (4, 1024, 64, 1, 6, 12.25, 12.25)]
    assert lines[3] == "mode 0 1"  # off by default; the setter returns the previous mode
