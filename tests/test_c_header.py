"""The C ABI from C: include/cpmd_gb300.h compiles as strict C99, and a C program
linked against libcpmd_gb300.so writes and reads a RESTART file through
gbcp_restart_write / gbcp_restart_read (host-only entry points, no GPU)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include <math.h>
#include <stdio.h>
#include <string.h>
#include "cpmd_gb300.h"

int main(int argc, char** argv) {
  if (argc < 2) return 9;
  enum { NGW = 40, NS = 3 };
  double c0[2 * NGW * NS], back[2 * NGW * NS];
  for (int i = 0; i < 2 * NGW * NS; ++i) c0[i] = sin(0.37 * i) * (i % 7 == 0 ? 2.0 : 0.1);
  int32_t na[1] = {2};
  double tau0[6] = {0, 0, 0, 1, 1, 1};
  gbcp_restart w;
  memset(&w, 0, sizeof w);
  w.ibrav = 1;
  w.celldm[0] = 10.0; w.celldm[1] = 1.0; w.celldm[2] = 1.0;
  w.nsp = 1; w.nat = 2; w.na = na; w.tau0 = tau0;
  w.ecut = 20.0; w.cdual = 4.0; w.nel = 6; w.nr1s = w.nr2s = w.nr3s = 24;
  w.nstate = NS; w.ngwks = NGW; w.c0 = c0; w.ldc = NGW; w.ngw = NGW; w.icompr = 1;
  int rc = gbcp_restart_write(argv[1], &w);
  if (rc != GBCP_OK) { printf("write %d\n", rc); return 1; }
  gbcp_restart r;
  memset(&r, 0, sizeof r);
  rc = gbcp_restart_read(argv[1], &r);  /* sizes */
  if (rc != GBCP_OK || r.nstate != NS || r.ngwks != NGW || r.nat != 2) { printf("size %d\n", rc); return 2; }
  int32_t na2[1];
  double t2[6];
  memset(&r, 0, sizeof r);
  r.na = na2; r.tau0 = t2; r.c0 = back; r.ldc = NGW; r.ngw = NGW; r.nstate_cap = NS;
  rc = gbcp_restart_read(argv[1], &r);
  if (rc != GBCP_OK || r.nstate_read != NS) { printf("read %d\n", rc); return 3; }
  if (memcmp(back, c0, sizeof c0) != 0 || memcmp(t2, tau0, sizeof tau0) != 0 || na2[0] != 2) return 4;
  if (gbcp_restart_read("/nonexistent/RESTART", &r) != GBCP_ERR_IO) return 5;
  printf("ok\n");
  return 0;
}
"""


def test_header_is_c99_and_restart_round_trips_from_c(tmp_path):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not available")
    from cpmd_gb300 import build as B
    lib = B.build()
    src = tmp_path / "prog.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "prog"
    cuda_lib = Path("/usr/local/cuda/lib64")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", str(ROOT / "include"), str(src),
           "-o", str(exe), "-L", str(lib.parent), "-lcpmd_gb300", "-lm", f"-Wl,-rpath,{lib.parent}"]
    if cuda_lib.exists():
        cmd += ["-L", str(cuda_lib), f"-Wl,-rpath,{cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ)
    run = subprocess.run([str(exe), str(tmp_path / "RESTART")], capture_output=True, text=True, env=env)
    assert run.returncode == 0 and run.stdout.strip() == "ok", run.stdout + run.stderr
