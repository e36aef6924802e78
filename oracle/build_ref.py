#!/usr/bin/env python3
"""Build recipe for ``oracle/_ref``: the reference's own Cython integral modules.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this file or
anything it builds; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs
of ``bench.py`` use ``oracle/``, and only to check results or as the timed CPU baseline.

What it does
------------
The reference (jjgoings/McMurchie-Davidson) keeps its two-electron hot path in
Cython: ``cython/twoe.pyx`` (``doERIs``, ``ERI``, ``electron_repulsion``),
``cython/util.pxi`` (``E``, ``R``, ``boys``), ``cython/basis.pxi`` (``Basis``) and
``cython/fock.pyx`` (``formPT``).  This script compiles those modules *from the
reference's own sources, where they lie*, after three mechanical shims that the
current toolchain needs (applied to a temporary copy, never to the original):

1. ``cython/basis.pxi:29``  ``long(view)`` -> ``int(view)`` (Cython 3 has no ``long``).
2. ``cython/onee.pyx:184`` (and ``grad.pyx``) ``xrange`` -> ``range``.
3. ``scipy.special.factorial2(-1)`` returns 0.0 in SciPy >= 1.11 while the
   reference was written against the old gamma-formula value 1.0; every s/p
   normalisation (``basis.pxi:102-110``) would divide by zero.  The shim binds
   ``fact2 = factorial2(n, extend="complex")`` which gives 1, 1, 3 at -1, 1, 3.

Outputs go only under ``oracle/_ref/`` (git-ignored, but copied with the tree to the machine with the GPU):

* ``oracle/_ref/gen/*.c``          Cython-generated C (portable; rebuilt per host)
* ``oracle/_ref/mmd/integrals/*.so`` the compiled modules, importable as
  ``mmd.integrals.twoe`` / ``mmd.integrals.fock`` / ``mmd.integrals.onee`` when
  ``oracle/_ref`` is first on ``sys.path`` (``fock.pyx`` imports
  ``mmd.integrals.twoe`` by that absolute name).

Modes
-----
``python oracle/build_ref.py``            cythonize from the reference (needs the
                                           reference tree and Cython) and compile.
``python oracle/build_ref.py --compile``  compile the already-generated C (the
                                           GPU machine has neither the reference nor
                                           Cython; it only needs gcc, Python.h and
                                           NumPy's headers).
``python oracle/build_ref.py --full DIR`` additionally lay out a complete shimmed
                                           copy of the reference package in DIR
                                           (Python modules + basis data + all four
                                           compiled modules), used only by
                                           ``tests/golden/make_golden.py`` here.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import sysconfig
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
GEN_DIR = os.path.join(REF_OUT, "gen")
PKG_DIR = os.path.join(REF_OUT, "mmd", "integrals")
# the reference tree: --reference or $MMD_REFERENCE (required to cythonize)
DEFAULT_REFERENCE = os.environ.get("MMD_REFERENCE")

# modules on the hot path (plus onee, whose ``_boys`` hook test012 uses)
HOT_MODULES = ("twoe", "fock", "onee")
ALL_MODULES = ("twoe", "fock", "onee", "grad")

FACT2_SHIM = (
    "from scipy.special import factorial2 as _fact2_raw\n"
    "def fact2(n):\n"
    "    return _fact2_raw(n, extend=\"complex\")\n"
)


def _shim_text(name: str, text: str) -> str:
    if name == "basis.pxi":
        text = text.replace("return long(view)", "return int(view)")
    if name in ("onee.pyx", "grad.pyx"):
        text = text.replace("xrange(", "range(")
    if name in ("basis.pxi", "onee.pyx", "reference.py"):
        text = text.replace("from scipy.special import factorial2 as fact2", FACT2_SHIM)
    return text


def shim_cython_sources(reference: str, dst: str) -> None:
    """Copy ``cython/*.pyx|pxi`` of the reference into ``dst`` with the shims."""
    os.makedirs(dst, exist_ok=True)
    src = os.path.join(reference, "cython")
    for name in sorted(os.listdir(src)):
        if not name.endswith((".pyx", ".pxi")):
            continue
        with open(os.path.join(src, name)) as f:
            text = f.read()
        with open(os.path.join(dst, name), "w") as f:
            f.write(_shim_text(name, text))


def cythonize(shimmed: str, modules=HOT_MODULES) -> None:
    os.makedirs(GEN_DIR, exist_ok=True)
    for m in modules:
        out = os.path.join(GEN_DIR, m + ".c")
        cmd = [sys.executable, "-m", "cython", "-3", "--module-name", "mmd.integrals." + m,
               "-o", out, os.path.join(shimmed, m + ".pyx")]
        subprocess.check_call(cmd)


def compile_generated(modules=HOT_MODULES, out_dir: str = PKG_DIR) -> list[str]:
    import numpy
    os.makedirs(out_dir, exist_ok=True)
    for d in (os.path.join(REF_OUT, "mmd"), out_dir):
        init = os.path.join(d, "__init__.py")
        if not os.path.exists(init):
            open(init, "w").close()
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    inc = sysconfig.get_paths()["include"]
    built = []
    procs = []
    for m in modules:
        src = os.path.join(GEN_DIR, m + ".c")
        if not os.path.exists(src):
            raise FileNotFoundError(f"{src} missing: run build_ref.py where the reference is present")
        so = os.path.join(out_dir, m + suffix)
        cmd = ["gcc", "-shared", "-fPIC", "-O2", "-fno-strict-aliasing", "-w",
               "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
               "-I", inc, "-I", numpy.get_include(), src, "-o", so, "-lm"]
        procs.append((so, subprocess.Popen(cmd)))
    for so, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"compiling {so} failed")
        built.append(so)
    return built


def full_copy(reference: str, dst: str) -> str:
    """Lay out a complete shimmed reference package under ``dst`` (golden generation only)."""
    pkg = os.path.join(dst, "mmd")
    if os.path.exists(pkg):
        shutil.rmtree(pkg)
    shutil.copytree(os.path.join(reference, "mmd"), pkg,
                    ignore=shutil.ignore_patterns("__pycache__", "backup"))
    ref_py = os.path.join(pkg, "integrals", "reference.py")
    with open(ref_py) as f:
        text = f.read()
    with open(ref_py, "w") as f:
        f.write(_shim_text("reference.py", text))
    compile_generated(ALL_MODULES, out_dir=os.path.join(pkg, "integrals"))
    return dst


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    ap.add_argument("--compile", action="store_true", help="only compile oracle/_ref/gen/*.c")
    ap.add_argument("--full", metavar="DIR", help="also lay out a full shimmed reference package in DIR")
    args = ap.parse_args(argv)

    modules = ALL_MODULES if args.full else HOT_MODULES
    if (not args.compile or args.full) and not args.reference:
        if args.full or not os.path.isdir(GEN_DIR):
            ap.error("the reference tree is required: pass --reference DIR or set MMD_REFERENCE")
        print("no reference tree given (--reference / MMD_REFERENCE); compiling generated C only", file=sys.stderr)
        args.compile = True
    if not args.compile:
        if not os.path.isdir(os.path.join(args.reference, "cython")):
            print(f"reference not found at {args.reference}; compiling generated C only", file=sys.stderr)
        else:
            with tempfile.TemporaryDirectory() as tmp:
                shim_cython_sources(args.reference, tmp)
                cythonize(tmp, modules)
    built = compile_generated(HOT_MODULES)
    if args.full:
        full_copy(args.reference, args.full)
    for b in built:
        print("built", os.path.relpath(b, HERE))
    return 0


if __name__ == "__main__":
    sys.exit(main())
