"""The C++ host layer (include/qbg.hpp) compiles against the C ABI, links to
libqbg.so and runs its host-side parts without a GPU: the basis it builds
equals the Python mirror's, and a failing C call surfaces as a qbg::Error
carrying the status and the library's message (on a machine without a GPU,
plan creation is that failing call)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import qball_gb300 as Q

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

PROGRAM = r'''
#include <cstdio>
#include "qbg.hpp"

int main() {
  const double L = 12.0;
  qbg::Basis b({L, 0, 0, 0, L, 0, 0, 0, L}, 10.0);
  double s = 0.0;
  for (double v : b.kpg2) s += v;
  std::printf("basis %d %d %d %d %d %.17g %.17g\n", b.ngw, b.nrods, b.np[0], b.np[1], b.np[2],
              b.omega, s);
  try {
    qbg::Plan plan(b, 32, 32, 32, QBG_PREC_FP64);
    std::printf("plan ok %d\n", plan.ngw());
  } catch (const qbg::Error& e) {
    std::printf("plan error %d\n", (int)e.status());
  }
  try {
    qbg::Basis bad({0, 0, 0, 0, 0, 0, 0, 0, 0}, 10.0);
    std::printf("bad basis accepted\n");
  } catch (const qbg::Error& e) {
    std::printf("bad basis error %d\n", (int)e.status());
  }
  return 0;
}
'''


def test_cpp_layer_builds_and_runs_host_side():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    Q.lib()  # the library is built
    out = os.path.join(ROOT, "qball_gb300", "_build", "cpp_host")
    os.makedirs(out, exist_ok=True)
    src = os.path.join(out, "host.cc")
    exe = os.path.join(out, "host")
    with open(src, "w") as f:
        f.write(PROGRAM)
    lib_dir = os.path.join(ROOT, "qball_gb300")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        src, "-o", exe, "-L", lib_dir, "-lqbg", f"-Wl,-rpath,{lib_dir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    import torch
    if torch.cuda.is_available():
        pytest.skip("host-side run is checked where no GPU is present")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    basis = lines[0].split()
    b = Q.Basis(12.0, 10.0)
    assert basis[0] == "basis" and int(basis[1]) == b.ngw
    assert abs(float(basis[6]) - 12.0 ** 3) < 1e-9
    assert abs(float(basis[7]) - float(np.sum(b.kpg2))) <= 1e-12 * float(np.sum(b.kpg2))
    # no GPU here: plan creation fails with a CUDA status, as a qbg::Error
    assert lines[1] == "plan error 4", r.stdout
    # a singular cell is rejected as an invalid argument
    assert lines[2] == "bad basis error 1", r.stdout
