"""A plain C host links against the library through include/lh.h alone and gets the
library's error convention (negative codes, lh_last_error(NULL) on the calling thread) for
configurations it rejects before touching a GPU."""
import os
import subprocess

from rnl_multiblock_nofft_gb300 import build_native

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

SRC = r'''
#include <stdio.h>
#include <string.h>
#include "lh.h"
int main(void) {
  lh_config cfg;
  lh_handle *h = 0;
  memset(&cfg, 0, sizeof cfg);
  cfg.abi_version = LH_ABI_VERSION + 1;
  int rc1 = lh_create(&cfg, &h);
  printf("%d %s\n", rc1, lh_last_error(NULL));
  cfg.abi_version = LH_ABI_VERSION;
  cfg.precision = 7;
  int rc2 = lh_create(&cfg, &h);
  printf("%d %s\n", rc2, lh_last_error(NULL));
  cfg.precision = LH_PREC_MIXED;
  cfg.N1 = 30; cfg.N2 = 32; cfg.Ngal1 = 48; cfg.Ngal2 = 48;  /* N1 != 2 (Ngal1 / 3) */
  cfg.N1c = 30; cfg.N2c = 32; cfg.Ngal1c = 48; cfg.Ngal2c = 48;
  int rc3 = lh_create(&cfg, &h);
  printf("%d %s\n", rc3, lh_last_error(NULL));
  printf("%d %d\n", lh_destroy(0), h == 0);
  return 0;
}
'''


def test_c_host_links_and_gets_errors(tmp_path):
    lib = build_native.build()
    src = tmp_path / "host.c"
    src.write_text(SRC)
    exe = tmp_path / "host"
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-l:" + os.path.basename(lib), "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    assert out[0].startswith("-1 ") and "abi_version" in out[0]
    assert out[1].startswith("-1 ") and "precision" in out[1]
    assert out[2].startswith("-1 ")
    assert out[3] == "-1 1"
