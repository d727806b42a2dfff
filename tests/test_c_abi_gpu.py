"""A C host program drives a whole simulation through the C ABI alone -- what
a cgo shim does: Normalize, create, seed on the host, upload the padded
fields, apply the velocity BC, Step, read MaxDivergence and the fields back,
close.  Its results must be bit-identical to the same run through the Python
binding, and a NaN it plants must come back as the reference's fault text."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from aeroflux_gb300 import Config, New
from aeroflux_gb300.workloads import taylor_green

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "aeroflux_cuda.h"

static int fail(const char* what, af_engine* e) {
    printf("FAIL %s: %s\n", what, e ? af_last_error(e) : "");
    return 1;
}

int main(int argc, char** argv) {
    const int nan_case = argc > 2 && argv[2][0] == '1';
    char err[256];
    af_config c;
    memset(&c, 0, sizeof c);
    c.nx = 20; c.ny = 14; c.nz = 12; c.h = 1.0 / 20; c.dt = 0.003; c.viscosity = 1e-4; c.density = 1.0;
    c.gauss_seidel_iters = 40;
    if (af_config_normalize(&c, err, sizeof err) != AF_OK) { printf("FAIL normalize %s\n", err); return 1; }
    af_engine* e = NULL;
    if (af_create(&c, &e, err, sizeof err) != AF_OK) { printf("FAIL create %s\n", err); return 1; }
    af_field_desc du, dv, dw;
    af_field_info(e, AF_FIELD_U, &du); af_field_info(e, AF_FIELD_V, &dv); af_field_info(e, AF_FIELD_W, &dw);
    double* u = (double*)calloc((size_t)du.count, 8);
    double* v = (double*)calloc((size_t)dv.count, 8);
    double* w = (double*)calloc((size_t)dw.count, 8);
    if (af_seed_taylor_green(&c, 1.0, 0.01, 42, 0, u, v, w) != AF_OK) return fail("seed", e);
    if (nan_case) u[4 + 4 * du.sy + 4 * du.sz] = NAN;
    if (af_field_upload(e, AF_FIELD_U, u, (size_t)du.count) != AF_OK) return fail("upload U", e);
    if (af_field_upload(e, AF_FIELD_V, v, (size_t)dv.count) != AF_OK) return fail("upload V", e);
    if (af_field_upload(e, AF_FIELD_W, w, (size_t)dw.count) != AF_OK) return fail("upload W", e);
    if (af_apply_velocity_bc(e) != AF_OK) return fail("bc", e);
    int rc = af_step(e, 3);
    if (nan_case) {
        printf("rc=%d\nmsg=%s\n", rc, af_last_error(e));
        af_destroy(e);
        return 0;
    }
    if (rc != AF_OK) return fail("step", e);
    double md = 0;
    if (af_max_divergence(e, &md) != AF_OK) return fail("maxdiv", e);
    if (af_field_download(e, AF_FIELD_U, u, (size_t)du.count) != AF_OK) return fail("download", e);
    FILE* f = fopen(argv[1], "wb");
    fwrite(&md, 8, 1, f);
    fwrite(u, 8, (size_t)du.count, f);
    fclose(f);
    af_close(e);
    af_close(e);  /* Close is idempotent (aeroflux.go:419-439) */
    af_destroy(e);
    printf("ok %.17g\n", md);
    return 0;
}
"""


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("needs gcc")
    d = tmp_path_factory.mktemp("chost")
    src = d / "host.c"
    src.write_text(PROGRAM)
    exe = d / "host"
    lib = os.path.join(ROOT, "aeroflux_gb300", "libaeroflux_cuda.so")
    subprocess.run(["gcc", "-std=c11", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), lib,
                    "-lm", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], check=True, capture_output=True,
                   text=True)
    return exe, d


def test_c_host_run_matches_python_binding(host):
    exe, d = host
    out = d / "u.bin"
    r = subprocess.run([str(exe), str(out), "0"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
    raw = out.read_bytes()
    md_c = struct.unpack("<d", raw[:8])[0]
    u_c = np.frombuffer(raw[8:], dtype=np.float64)
    cfg = Config(NX=20, NY=14, NZ=12, H=1 / 20, DT=0.003, Viscosity=1e-4, Density=1.0, GaussSeidelIters=40)
    e = New(cfg)
    for n, a in zip(("U", "V", "W"), taylor_green(e.Cfg, 1.0, 0.01, 42, 0)):
        e.upload(n, a)
    e.applyVelocityBC()
    e.Step(3)
    assert e.MaxDivergence() == md_c
    assert np.array_equal(e.download("U").view(np.uint64), u_c.view(np.uint64))
    e.Close()


def test_c_host_sees_the_reference_fault_text(host):
    exe, d = host
    r = subprocess.run([str(exe), str(d / "unused.bin"), "1"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(l.split("=", 1) for l in r.stdout.splitlines() if "=" in l)
    assert int(lines["rc"]) == -3  # AF_ERR_FAULT
    assert lines["msg"].startswith("aeroflux: guard-page fault contained: runtime error: index out of range [")
