"""Compensated reductions (energy.f90:67-165 sums, the norm and mu).

Every sum the kernels return goes through the primitives of
eff_pot_gb300/csrc/ep_reduce.cuh: Neumaier per thread, TwoSum pairs across
warps, blocks and the finalising block.  tests/cuda/reduce_harness.cu runs
them on a GPU beside a plain FP64 reduction of the same shape.  On a sum
whose terms cancel (2^21 terms of magnitude up to 1e3 adding up to about
1e-7, condition number ~1e16) the plain sum keeps at most a few digits and
the compensated one keeps ten; on a well-conditioned positive sum both are
exact to a few ulp.
"""
import ctypes as C
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("reduce") / "libreduce_harness.so")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-o", out, os.path.join(HERE, "cuda", "reduce_harness.cu")], check=True)
    lib = C.CDLL(out)
    lib.harness_sum.restype = C.c_int
    lib.harness_sum.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(C.c_double)]

    def run(x, compensated):
        x = np.ascontiguousarray(x, dtype=np.float64)
        r = C.c_double()
        assert lib.harness_sum(x.ctypes.data, x.size, 1 if compensated else 0, C.byref(r)) == 0
        return r.value
    return run


def test_compensated_sum_keeps_the_digits_a_plain_sum_loses(harness):
    rng = np.random.default_rng(7)
    x = rng.uniform(-1e3, 1e3, 1 << 21)
    x[0] -= math.fsum(x)
    x[1] += 1.234567e-7
    exact = math.fsum(x)
    assert 1e-7 < abs(exact) < 2e-7
    plain = harness(x, False)
    comp = harness(x, True)
    err_plain = abs(plain - exact) / abs(exact)
    err_comp = abs(comp - exact) / abs(exact)
    print(f"REDUCE cancelling sum: exact {exact:.17g}, plain rel err {err_plain:.2e}, "
          f"compensated rel err {err_comp:.2e}")
    assert err_comp < 1e-9
    assert err_plain > 1e-6


def test_well_conditioned_sums_agree(harness):
    rng = np.random.default_rng(8)
    x = rng.uniform(0.0, 0.02, 1 << 21) ** 2
    exact = math.fsum(x)
    for comp in (False, True):
        assert abs(harness(x, comp) - exact) <= 8 * np.finfo(float).eps * exact
