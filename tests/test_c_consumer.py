"""The C ABI consumed from plain C: the header compiles as C99 and the
library links and answers from a C program (what a Julia ccall, cgo or JNI
shim sees).  Runs without a GPU: version, device count, a host table builder
and the no-device error path of pcl_create."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_SRC = r"""
#include <stdio.h>
#include <string.h>
#include "particulator_gb300.h"

int main(void) {
    const char* v = pcl_version();
    if (!v || !strstr(v, "sm_103a")) return 1;
    int ndev = pcl_device_count();
    /* Moller (Z = 7, tcut = 10 keV): total cross section at 1 MeV, host FP64 */
    pcl_process m;
    memset(&m, 0, sizeof(m));
    m.kind = PCL_PROC_MOLLER;
    m.Z = 7;
    m.coef = 1.0;
    m.param[0] = 1e4 * 1.6021766208e-19;
    m.nparam = 1;
    double e = 1e6 * 1.6021766208e-19, cs = -1.0;
    if (pcl_totalcs(&m, 1, &e, &cs) != PCL_OK || !(cs > 0.0)) return 2;
    if (ndev == 0) {
        pcl_config cfg;
        memset(&cfg, 0, sizeof(cfg));
        void* ctx = NULL;
        if (pcl_create(&cfg, &ctx) != PCL_ERR_CUDA || ctx != NULL) return 3;
    }
    printf("ok %d %.6e\n", ndev, cs);
    return 0;
}
"""


def test_header_compiles_as_c99_and_links(pcl, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.join(ROOT, "particulator.jl_gb300", "_build")
    src = tmp_path / "consumer.c"
    src.write_text(C_SRC)
    exe = tmp_path / "consumer"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-L", libdir, "-lparticulator_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), (r.returncode, r.stdout, r.stderr)
