#!/usr/bin/env python3
"""Build ``mmd/_lib/libmmdg.so`` (the C-ABI of include/mmdg.h) for sm_103a.

1. ``csrc/gen_md.py`` generates the per-class shell-quartet code
   (``_build/md_gen.cuh``), the instantiation units ``_build/md_inst*.cu`` and the
   dispatch table ``_build/md_dispatch.cuh``;
2. every unit is compiled by nvcc in parallel
   (``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``);
3. the objects are linked into a shared library with nvcc.

Outputs stay in-tree and are git-ignored: ``_build/`` and ``mmd/_lib/``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "mmd", "_lib")
LIB = os.path.join(LIBDIR, "libmmdg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr", "-I", CSRC, "-I", BUILD, "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    sys.path.insert(0, CSRC)
    try:
        import gen_md
    finally:
        sys.path.pop(0)
    os.makedirs(BUILD, exist_ok=True)
    gen_md.generate(os.path.join(BUILD, "md_gen.cuh"))
    inst = gen_md.generate_instances(BUILD)
    return [os.path.join(CSRC, "capi.cu"), os.path.join(CSRC, "noalloc.cu"), os.path.join(CSRC, "mlp.cu"), os.path.join(CSRC, "grad.cu"), os.path.join(CSRC, "ao2mo.cu")] + inst


def _deps():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".py")):
                out.append(os.path.join(d, f))
    return out


def build(verbose: bool = False, extra_flags=None, force: bool = False) -> str:
    srcs = _sources()
    newest_dep = max(os.path.getmtime(p) for p in _deps() + srcs)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest_dep:
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    flags = ARCH + NVCC_FLAGS + list(extra_flags or [])
    t0 = time.time()
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if not force and os.path.exists(o) and os.path.getmtime(o) >= newest_dep:
            continue
        cmd = [nvcc(), "-c", s, "-o", o] + flags
        procs.append((s, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for s, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            print(out)
        if p.returncode != 0:
            failed.append((s, out))
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB} in {time.time() - t0:.1f}s")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv,
          extra_flags=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
