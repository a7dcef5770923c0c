"""The C ABI is plain C: include/nbx.h compiles as C99 with every warning an
error, and the example of the integration guide (section 2, the native
pipeline) compiles and links against libnbx.so (no GPU: nothing runs)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

EXAMPLE = r"""
#include "nbx.h"

/* the integration guide's native-pipeline example, as a function */
int run(float *d_x, float *d_y, float *d_z, float *d_vx, float *d_vy, float *d_vz, float *d_ax,
        float *d_ay, float *d_az, float *d_m, int n, void *stream) {
    nbx_params prm;
    nbx_params_default(&prm);
    prm.max_bodies = n; prm.theta = 0.5f; prm.eps = 0.005f; prm.dt = 5e-4f;
    nbx_ctx *ctx;
    int rc = nbx_create(&prm, &ctx);
    if (rc) return rc;
    int64_t off[2] = {0, n};
    rc = nbx_set_systems(ctx, 1, off);
    nbx_state s = {d_x, d_y, d_z, d_vx, d_vy, d_vz, d_ax, d_ay, d_az, d_m};
    if (!rc) rc = nbx_step(ctx, &s, 100, stream);
    if (!rc) rc = nbx_sync_status(ctx, stream);
    nbx_destroy(ctx);
    return rc;
}

int main(void) { return 0; }
"""


def test_header_is_plain_c(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "example.c"
    src.write_text(EXAMPLE)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_example_links_against_the_library(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    lib = os.path.join(ROOT, "nns_gb300", "libnbx.so")
    if cc is None or not os.path.exists(lib):
        pytest.skip("no C compiler or library not built")
    src = tmp_path / "example.c"
    src.write_text(EXAMPLE)
    exe = tmp_path / "example"
    r = subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", os.path.dirname(lib), "-lnbx", "-Wl,--no-as-needed"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
