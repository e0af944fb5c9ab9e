"""The double-single spin master (precisions 2 and 4) on the CPU: tests/ds_harness.cu,
compiled as host code against uppasd_gb300/csrc/common.cuh, applies ds_add_renorm to
updates that keep |e| = 1 to FP32 rounding (rotations formed in FP32, as the Depondt,
midpoint and SIB kernels form them) and ds_add_renorm_wide to first-order updates (Heun,
LLGI), and compares the hi + lo pairs in long double with the exactly normalised sums.
The pair keeps the state to about 2^-48 per component; the second-order form alone would
leave first-order updates off the sphere by ~1e-5, which is why those take the wide form.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    if not os.path.exists(NVCC):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("ds") / "ds_harness")
    subprocess.run([NVCC, "-O2", "-std=c++17", "-x", "cu", os.path.join(ROOT, "tests", "ds_harness.cu"), "-o", exe],
                   check=True)
    out = subprocess.run([exe, "100000"], check=True, capture_output=True, text=True).stdout
    return {ln.split()[0]: [float(x) for x in ln.split()[1:]] for ln in out.splitlines()}


def test_rotations_keep_double_single_precision(results):
    norm, err, lo = results["narrow"]
    assert norm < 1e-13 and err < 5e-14
    assert lo <= 0.5  # |lo| within half an ulp of hi: normalised pairs


def test_first_order_updates_take_the_wide_form(results):
    norm, err, lo = results["wide"]
    assert norm < 5e-13 and err < 2e-13
    assert lo <= 0.5
    # the second-order series alone on the same updates
    assert results["narrow_on_first_order"][0] > 1e-6
