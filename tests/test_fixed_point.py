"""The float64 -> 64-bit fixed-point conversion of state uploads
(fixed_from_double in csrc/kernels.cuh) is exact: compiled for the host and
checked against rational arithmetic (periodic: round(frac(x/L) 2^64) with
halves up, mod 2^64; reflecting: llround(x/L S), S = 2^62)."""
import math
import os
import shutil
import subprocess
from fractions import Fraction as F

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = r'''
#include <cstdio>
#include "kernels.cuh"
int main() {
  double x, L;
  int per;
  const long long Si = (long long)(1ULL << 62);
  while (std::scanf("%la %la %d", &x, &L, &per) == 3) {
    unsigned long long X = 0;
    bool ok = rd::fixed_from_double(x, L, per != 0, Si, &X);
    std::printf("%d %llu\n", ok ? 1 : 0, X);
  }
  return 0;
}
'''


def exact(x, L, per):
    Si = 2 ** 62
    if per:
        f = F(math.fmod(x, L))
        return math.floor(f * 2 ** 64 / F(L) + F(1, 2)) % 2 ** 64
    y = F(x) * Si / F(L)
    q = math.floor(abs(y) + F(1, 2))
    return (q if y >= 0 else -q) % 2 ** 64


@pytest.fixture(scope="module")
def converter(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("fx")
    src = d / "fx.cu"
    src.write_text(SRC)
    exe = d / "fx"
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-I", os.path.join(ROOT, "pyrdsim_gb300", "csrc"), str(src), "-o",
                           str(exe)])
    return str(exe)


def test_fixed_from_double_is_exact(converter):
    rng = np.random.default_rng(4)
    cases = []
    for _ in range(4000):
        L = float(1.0 + 500.0 * rng.random())
        per = int(rng.integers(0, 2))
        x = float((rng.random() * 4 - 2) * L) if per else float((rng.random() * 2 - 1) * L)
        cases.append((x, L, per))
    for L in (7.0, 404.77, 1e-3, 3.0e5):
        cases += [(L / 2, L, 1), (-L / 4, L, 1), (L, L, 1), (0.0, L, 1), (-0.0, L, 1),
                  (math.nextafter(L, 0.0), L, 1), (-1e-300, L, 1), (L, L, 0), (-L, L, 0),
                  (1e-310, L, 0), (math.nextafter(0.5 * L, L), L, 0)]
    text = "\n".join(f"{x.hex()} {L.hex()} {p}" for x, L, p in cases) + "\n"
    out = subprocess.run([converter], input=text, capture_output=True, text=True, check=True)
    got = [tuple(map(int, line.split())) for line in out.stdout.strip().splitlines()]
    assert len(got) == len(cases)
    for (x, L, p), (ok, X) in zip(cases, got):
        assert ok == 1
        assert X == exact(x, L, p), (x, L, p, X, exact(x, L, p))
    # non-finite positions are refused
    out = subprocess.run([converter], input=f"{float('inf').hex()} 1.0 1\n", capture_output=True,
                         text=True, check=True)
    assert out.stdout.split()[0] == "0"
