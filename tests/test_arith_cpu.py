"""Host checks of the lazy modular arithmetic the recursion kernels use (three-partial
Shoup estimate, widened Montgomery reduction, 32-bit Shoup products) and of the
inverse-twiddle identity the special_modulus kernel derives its inverse ladders from."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "inspire-rs_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"


def test_lazy_bounds_against_exact_arithmetic():
    gxx = shutil.which("g++")
    if gxx is None or not os.path.isdir(CUDA_INC):
        pytest.skip("needs g++ and the CUDA headers")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "arith_bounds")
        subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, "-I", CUDA_INC,
                        os.path.join(ROOT, "tests", "arith_bounds.cpp"), "-o", exe], check=True)
        out = subprocess.run([exe, "1000000"], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr


def _brv(k, bits):
    return int(format(k, "0%db" % bits)[::-1], 2)


@pytest.mark.parametrize("m", [536_813_569, 2_147_389_441, 1_152_921_504_606_830_593])
def test_inverse_twiddles_from_forward_ladder(m):
    """psi^-brv(j) = m - psi^brv(3 2^s - 1 - j) for 2^s <= j < 2^(s+1), and the Shoup
    companion of m - w is the complement of w's: the identity both respond kernels use to
    take the inverse ladder from the forward one."""
    n, bits = 2048, 11
    psi = next(c for c in (pow(g, (m - 1) // (2 * n), m) for g in range(2, 200)) if pow(c, n, m) == m - 1)
    psi_inv = pow(psi, 2 * n - 1, m)
    word = 32 if m < 2**32 else 64
    full = (1 << word) - 1
    for j in range(1, n):
        s = j.bit_length() - 1
        f = pow(psi, _brv(3 * (1 << s) - 1 - j, bits), m)
        want = pow(psi_inv, _brv(j, bits), m)
        assert m - f == want, j
        assert (~((f << word) // m)) & full == (want << word) // m, j
