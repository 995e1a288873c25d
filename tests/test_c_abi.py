"""The C ABI from a C caller: include/sem_b200.h compiles as C99 with every
warning enabled, a program that takes the address of every declared entry
point links against libsem_b200.so, and its host-only calls run without a GPU
(the version, argument checks and the BDF coefficients of src/time.jl:31-53)."""
import os
import re
import shutil
import subprocess

import pytest

from semgb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _functions():
    src = open(os.path.join(ROOT, "include", "sem_b200.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sem_[a-z0-9_]+)\s*\(", src)))


PROGRAM = r"""
#include <stdio.h>
#include <math.h>
#include "sem_b200.h"

typedef void (*any_fn)(void);

int main(void) {
  const any_fn table[] = {
%s
  };
  int missing = 0;
  for (size_t i = 0; i < sizeof(table) / sizeof(table[0]); ++i) missing += table[i] == 0;
  if (missing) return 10;
  if (sem_abi_version() != SEM_ABI_VERSION) return 11;
  /* host-only: BDF3 on the history [3h, 2h, h, 0] */
  const double h = 0.1, t[4] = {3 * h, 2 * h, h, 0.0};
  double a[3], b[4];
  if (sem_bdf_coeffs(3, t, a, b) != SEM_OK) return 12;
  const double want_b[4] = {11.0 / 6.0 / h, -3.0 / h, 1.5 / h, -1.0 / 3.0 / h};
  for (int i = 0; i < 4; ++i)
    if (fabs(b[i] - want_b[i]) > 1e-12 * fabs(want_b[i])) return 13;
  if (fabs(a[0] - 3.0) > 1e-12 || fabs(a[1] + 3.0) > 1e-12 || fabs(a[2] - 1.0) > 1e-12) return 14;
  /* argument checks run before any device work */
  if (sem_mesh_create(NULL, NULL) != SEM_ERR_BAD_ARG) return 15;
  if (sem_bdf_run(NULL, NULL, NULL, NULL, NULL, NULL, NULL) != SEM_ERR_BAD_ARG) return 16;
  if (sem_last_error() == NULL || sem_last_error()[0] == 0) return 17;
  printf("ok %%d\n", (int)(sizeof(table) / sizeof(table[0])));
  return 0;
}
"""


@pytest.fixture(scope="module")
def lib_path():
    _lib.build()
    return _lib.LIB_PATH


def test_header_is_c99_and_every_entry_links(lib_path, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = _functions()
    entries = ",\n".join(f"    (any_fn){n}" for n in names)
    src = tmp_path / "abi.c"
    src.write_text(PROGRAM % entries)
    exe = tmp_path / "abi"
    lib_dir = os.path.dirname(lib_path)
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-Wno-cast-function-type",
           "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", lib_dir, "-lsem_b200", f"-Wl,-rpath,{lib_dir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    assert run.stdout.strip() == f"ok {len(names)}"
