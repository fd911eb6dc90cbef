"""The C ABI from a plain C99 program: include/lbm_gb300.h compiles as C,
and a program linked against the library runs its host-only entry points
(no GPU call), as a cgo or JNI binding would link it."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "lbm_gb300.h"

int main(void) {
  int k = 0;
  if (lbm_plan_checkpoints(2000, 100, &k) != LBM_OK) return 1;
  if (lbm_plan_checkpoints(2000, 10, &k) != LBM_ERR_NOMEM) return 2;
  if (strcmp(lbm_status_string(LBM_ERR_ARG), "LBM_ERR_ARG") != 0) return 3;
  if (lbm_struct_size(0) != sizeof(lbm_params)) return 4;
  if (lbm_struct_size(1) != sizeof(lbm_sphere)) return 5;
  if (lbm_struct_size(2) != sizeof(lbm_xla_desc)) return 6;
  if (lbm_struct_size(3) != sizeof(lbm_xla_fused_desc)) return 7;
  if (lbm_create(NULL, NULL) != LBM_ERR_ARG) return 8;
  printf("api %d segment %d\n", lbm_api_version(), k);
  return 0;
}
"""


@pytest.fixture(scope="module")
def libdir():
    from lbm_jax_autodiff_gb300 import build
    return os.path.dirname(build.build())


def test_c_program_links_and_runs(libdir, tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "consumer.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "consumer"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-llbm_gb300",
                    "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    api, seg = out.stdout.split()[1], int(out.stdout.split()[3])
    assert int(api) >= 1 and 1 <= seg <= 2000
