"""ORACLE / TEST INFRASTRUCTURE ONLY.

Loads the CPU checkers built by oracle/Makefile:

* ``port()``  -> oracle/_build/liboracle.so, the project's C restatement of the
  reference's S2LET layer over a restatement of the SSHT/SO3 transforms it calls.
  Builds and runs anywhere (this is the checker on GPU machines).
* ``ref()``   -> oracle/_ref/libs2let_ref.so, the reference's own S2LET C sources
  compiled in place over the same SSHT/SO3 restatement.  Exists only where the
  reference tree was available at build time; used to generate and pin golden
  vectors.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this module, and only as a checker or a timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libs2let_ref.so")


def build(ref_dir: str | None = None) -> None:
    """Compile the port (always) and, when a reference checkout is named
    (``ref_dir``, else the S2LET_REFERENCE_DIR environment variable) and holds
    src/c, the in-place reference build."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    ref_dir = ref_dir or os.environ.get("S2LET_REFERENCE_DIR")
    if ref_dir and os.path.isdir(os.path.join(ref_dir, "src", "c")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_dir}"], check=True)


def _load(path):
    from s2let_gb300.capi import S2let, bind

    lib = C.CDLL(path, mode=os.RTLD_LOCAL)
    bind(lib)
    return S2let(lib)


_cache = {}


def port():
    if "port" not in _cache:
        if not os.path.exists(PORT_SO):
            build()
        _cache["port"] = _load(PORT_SO)
    return _cache["port"]


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    if "ref" not in _cache:
        _cache["ref"] = _load(REF_SO)
    return _cache["ref"]
