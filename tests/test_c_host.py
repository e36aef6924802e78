"""A plain C host against the C ABI: a C99 program that includes include/mmdg.h and
links libmmdg.so compiles with gcc, and its calls behave as the header states
without a GPU -- argument errors and the missing device come back as status codes
with text from mmdg_last_error(), and the host-side Boys table is readable."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(REPO, "mcmurchie-davidson_gb300", "mmd", "_lib")

PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "mmdg.h"

int main(void) {
    /* host-only entry point: the tabulated F_m(k/16) rows */
    long long n = mmdg_boys_table(NULL, 0);
    double* tab = (double*)malloc(sizeof(double) * (size_t)n);
    if (mmdg_boys_table(tab, n) != n) return 2;
    printf("boys %lld %.17g\n", n, tab[0]);          /* F_0(0) = 1 */
    free(tab);
    /* an argument error is reported before any device work */
    int rc = mmdg_eri_tensor_noalloc(0, NULL, NULL, NULL, NULL, NULL, NULL, 0, NULL, NULL);
    printf("noalloc %d %s\n", rc, mmdg_last_error());
    /* a context: a GPU gives MMDG_OK, no GPU gives a CUDA status with its text */
    mmdg_context* h = NULL;
    rc = mmdg_create(&h, 0);
    printf("create %d %s\n", rc, rc == MMDG_OK ? "ok" : mmdg_last_error());
    if (rc == MMDG_OK) mmdg_destroy(h);
    return 0;
}
"""


def test_c_program_compiles_links_and_reports_status(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lib = os.path.join(LIBDIR, "libmmdg.so")
    if not os.path.exists(lib):
        pytest.skip("libmmdg.so not built (run __graft_entry__.build())")
    src = tmp_path / "host.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "host"
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"), str(src),
                           "-o", str(exe), "-L", LIBDIR, "-lmmdg", f"-Wl,-rpath,{LIBDIR}"])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = dict(line.split(" ", 1) for line in out.stdout.strip().splitlines())
    n, f00 = lines["boys"].split()
    assert int(n) > 0 and float(f00) == 1.0
    rc, msg = lines["noalloc"].split(" ", 1)
    assert int(rc) == -1 and "mmdg_eri_tensor_noalloc" in msg          # MMDG_E_ARG
    rc, msg = lines["create"].split(" ", 1)
    assert (int(rc) == 0 and msg == "ok") or (int(rc) == -3 and msg)    # MMDG_OK or MMDG_E_CUDA
