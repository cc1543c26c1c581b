"""The C boundary as a C caller sees it (no GPU): a C99 program that
includes include/natgpu.h, compiled with -pedantic -Werror, linked against
libnatgpu.so the way the integration notes show, calls the entry points
that return before touching CUDA and checks their results."""
import os
import shutil
import subprocess

import pytest

import natrium_gb300 as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "natgpu.h"

int main(void) {
  char buf[64];
  nat_spec spec;
  nat_solver* h = NULL;
  uint64_t ticket = 0;
  double x[4] = {0, 0, 0, 0};
  if (!nat_version() || !nat_version()[0]) return 10;
  if (nat_last_error(NULL, buf, sizeof buf) != NAT_OK || strcmp(buf, "null handle") != 0) return 11;
  memset(&spec, 0, sizeof spec);
  spec.dim = 2;
  spec.stencil = NAT_D2Q9;
  spec.order = 0; /* invalid: rejected before any CUDA call */
  spec.cells[0] = spec.cells[1] = spec.cells[2] = 4;
  spec.length[0] = spec.length[1] = spec.length[2] = 1.0;
  spec.periodic[0] = spec.periodic[1] = spec.periodic[2] = 1;
  spec.scaling = 1.0;
  spec.viscosity = 0.1;
  spec.cfl = 0.4;
  spec.collision = NAT_BGK_STANDARD;
  spec.precision = NAT_FP64;
  spec.vertices = NULL;
  if (nat_create(&spec, &h) != NAT_ERR_INVALID_ARG) return 12;
  if (nat_step(NULL, 1) != NAT_ERR_INVALID_ARG) return 13;
  if (nat_upload_f(NULL, x) != NAT_ERR_INVALID_ARG) return 14;
  if (nat_download_macro_async(NULL, x, x, &ticket) != NAT_ERR_INVALID_ARG) return 15;
  if (nat_wait(NULL, 1) != NAT_ERR_INVALID_ARG) return 16;
  if (nat_destroy(NULL) != NAT_OK) return 17;
  {
    /* the server statistics the Python mirror reads field by field: twelve int64 */
    nat_server_stats_t st;
    if (sizeof st != 12 * sizeof(int64_t)) return 18;
    if (nat_server_stats(NULL, &st) != NAT_ERR_INVALID_ARG) return 19;
  }
  printf("ok %s\n", nat_version());
  return 0;
}
"""


def test_c99_program_includes_header_and_links(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = N.load_library()._name
    libdir = os.path.dirname(lib)
    src = tmp_path / "caller.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "caller"
    cmd = [cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(src), "-o", str(exe), "-L", libdir, "-lnatgpu", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("ok ")


def test_server_stats_layout_matches_python_mirror():
    """natrium_gb300.serving reads nat_server_stats_t through ctypes: the same
    twelve int64 fields in the same order as include/natgpu.h."""
    import ctypes
    from natrium_gb300 import serving as SV
    names = [f for f, _ in SV._Stats._fields_]
    assert ctypes.sizeof(SV._Stats) == 12 * 8
    hdr = open(os.path.join(ROOT, "include", "natgpu.h")).read()
    body = hdr[hdr.index("typedef struct nat_server_stats_t {"):hdr.index("} nat_server_stats_t;")]
    decl = " ".join(l.split("/*")[0] for l in body.splitlines()[1:] if "int64_t" in l)
    fields = [f.strip(" ;") for f in decl.replace("int64_t", "").replace(";", ",").split(",") if f.strip(" ;")]
    assert fields == names
