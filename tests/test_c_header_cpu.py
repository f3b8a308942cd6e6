"""include/fluid2d_gb300.h is a plain C header: a C99 program (as another
host language's FFI would see the library) compiles against it, links
libfluid2d_gb300.so and gets the host-side answers of the ABI -- version,
a switch query, the halo check's error code and message, a refused model
description -- without touching a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "fluid2d_gb300.h"

int main(void) {
    double dummy[1];
    int8_t m1[1];
    f2d_model_desc d;
    void *model = NULL;
    int rc;
    printf("version %d\n", f2d_version());
    printf("pdl %d\n", f2d_set_pdl(-1));
    rc = f2d_adv_upwind(m1, dummy, dummy, dummy, dummy, dummy, 2, 1, 5, 38, 38, NULL);
    printf("nh %d %s\n", rc, rc == F2D_ERR_NH ? "F2D_ERR_NH" : "?");
    printf("msg %s\n", f2d_last_error());
    memset(&d, 0, sizeof d);
    d.model = F2D_EULER;
    d.nx = 2;
    d.ny = 32;
    d.Lx = d.Ly = 1.;
    rc = f2d_model_create(&d, m1, &model);
    printf("create %d %s\n", rc, rc == F2D_ERR_SHAPE && model == NULL ? "F2D_ERR_SHAPE" : "?");
    return 0;
}
"""


def test_c_program_uses_the_header(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    from fluid2d_gb300 import _lib
    _lib.build()
    so = _lib.so_path("product")
    src = tmp_path / "use_header.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "use_header"
    cmd = [gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
           "-o", str(exe), so, "-Wl,-rpath," + os.path.dirname(so)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ)
    cudalib = "/usr/local/cuda/lib64"
    if os.path.isdir(cudalib):
        env["LD_LIBRARY_PATH"] = cudalib + ":" + env.get("LD_LIBRARY_PATH", "")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert int(out["version"]) > 0
    assert out["pdl"] in ("0", "1")
    assert out["nh"] == "1 F2D_ERR_NH" and "NHALO = 3" in out["msg"]
    assert out["create"] == "2 F2D_ERR_SHAPE"
