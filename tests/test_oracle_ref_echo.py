"""The oracle's echo against the reference's own code.

tests/golden/ref_echo.npz holds echoes computed by the reference's
generateEchoKernel (code/SAR_BP/CUDA/BPA_CUDA_kernels.cu:3-45) itself,
compiled from the reference source as host code (oracle/ref) and run in FP32,
for its default SARParams with a record and aperture that hold the targets.
The oracle restates the same formula (BPA_SAR.m:80-89: phase
pi Kr t^2 - 4 pi R / lambda, gates 0 < t < Tr and |Az| < La/2) in FP64, so:
  * every gate decision agrees (the same samples are non-zero);
  * the relative L2 difference is within one FP32 ulp of the reference's
    largest phase (its own rounding: -42 dB at 300 m range, -12 dB at the
    default 11 km).
"""
import numpy as np
import pytest

from ref_echo_case import load, oracle_echo, phase_ulp_db
from sar_cambrianaccelerationcard_gb300 import metrics


@pytest.mark.parametrize("name", ["near", "default"])
def test_oracle_echo_matches_reference_kernel(orc, name):
    case = load(name)
    ref = case["echo"]
    mine = oracle_echo(orc, case)
    assert np.count_nonzero(ref) > 0
    assert np.array_equal(np.abs(ref) > 0, np.abs(mine) > 0), "gate decisions differ"
    err = metrics.rel_l2_db(mine, ref)
    bound = phase_ulp_db(case["params"])
    print(name, f"oracle vs reference kernel {err:.1f} dB (FP32 phase ulp {bound:.1f} dB)")
    assert err <= bound
