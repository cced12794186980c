"""FP32 fused stepper vs an FP64 run of the reference's own spin-1 kernels
(oracle/ref_cuda_drift.py) on a 24^3 version of the spin-1 workload, 400 steps:
relative energy difference <= 1e-6 and max |psi_fp32 - psi_ref| <= 1e-4 max|psi|.
The full-size run (96^3, 10^4 steps) is `python -m oracle.ref_cuda_drift`."""
import pytest

from oracle import ref_cuda

pytestmark = pytest.mark.gpu


def test_fp32_vs_reference_fp64(gpu):
    if not ref_cuda.available("spin1_bcc"):
        pytest.skip("reference cubins not built (oracle/build_ref_cuda.sh needs the reference tree)")
    from oracle.ref_cuda_drift import run

    r = run(cells=24, steps=400, every=100)
    assert r["energy_rel_diff_max"] <= 1e-6, r
    assert r["norm_rel_diff_max"] <= 1e-6, r
    assert r["psi_max_abs_err"] <= 1e-4 * r["psi_max_abs"], r


def test_scalar_fp32_vs_reference_fp64(gpu):
    if not ref_cuda.available("scalar_bcc"):
        pytest.skip("reference cubins not built (oracle/build_ref_cuda.sh needs the reference tree)")
    from oracle.ref_cuda_drift import run_scalar

    r = run_scalar(cells=16, steps=300, every=100)
    assert r["energy_rel_diff_max"] <= 1e-6, r
    assert r["psi_max_abs_err"] <= 1e-4 * r["psi_max_abs"], r
