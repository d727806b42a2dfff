"""The boundary as a cgo shim sees it: include/aeroflux_cuda.h must compile
as C11 (cgo hands it to a C compiler), and a C host program must link the
library and use its device-free entry points (Normalize with the
reference's messages, MACBytes, the ABI version, a failed create reporting
its error) without a GPU."""
import os
import shutil
import subprocess

import pytest

from aeroflux_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "aeroflux_cuda.h"

int main(void) {
    char err[256];
    af_config c;
    memset(&c, 0, sizeof c);
    c.nx = 64; c.ny = 64; c.nz = 64;
    if (af_config_normalize(&c, err, sizeof err) != AF_OK) { printf("normalize: %s\n", err); return 1; }
    printf("ghost=%lld h=%.17g dt=%.17g gsi=%lld\n", (long long)c.ghost, c.h, c.dt, (long long)c.gauss_seidel_iters);
    af_config bad;
    memset(&bad, 0, sizeof bad);
    bad.nx = 0; bad.ny = 4; bad.nz = 4;
    int rc = af_config_normalize(&bad, err, sizeof err);
    printf("bad=%d msg=%s\n", rc, err);
    printf("mac=%lld abi=%d\n", (long long)af_mac_bytes(64, 64, 64, 1), af_abi_version());
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_header_compiles_as_c11_and_a_c_host_links(tmp_path):
    lib = L.lib_path() if hasattr(L, "lib_path") else os.path.join(ROOT, "aeroflux_gb300", "libaeroflux_cuda.so")
    assert os.path.exists(lib), "build the library first"
    src = tmp_path / "host.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "host"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                    str(src), lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(tok.split("=", 1) for line in r.stdout.splitlines() for tok in line.split(" ") if "=" in tok)
    assert lines["ghost"] == "1" and float(lines["h"]) == 1 / 64 and lines["gsi"] == "24"
    assert int(lines["bad"]) == L.AF_ERR_CONFIG
    assert r.stdout.split("msg=", 1)[1].startswith("aeroflux:")
    assert int(lines["mac"]) == L.lib().af_mac_bytes(64, 64, 64, 1)
    assert int(lines["abi"]) == L.lib().af_abi_version()
