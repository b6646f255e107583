"""The FP64 fast-path device math (logmean with a shared reciprocal, the
two-point flux contracted with its metric vector, log/exp entropy maps)
against the reference's formulas, compiled by nvcc as host code (no GPU)."""
import json
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.fail("nvcc is required")
    exe = str(tmp_path_factory.mktemp("devmath") / "device_math_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", os.path.join(HERE, "device_math_check.cu"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def test_logmeans(results):
    assert results["logmean"] < 5e-15
    assert results["inv_logmean"] < 5e-15


def test_contracted_ec_flux(results):
    # relative to the largest flux-tensor entry; the contraction sums D terms
    assert results["ec_flux_dot"] < 2e-14


def test_halved_metric_vector_flux_is_bitwise(results):
    # ec_flux_dot_half(G / 2) takes the 1/2 factors inside the halved vector;
    # scaling by 1/2 is exact, so the mass and momentum fluxes are bitwise
    # those of ec_flux_dot(G); the energy flux is associated differently
    # (igm1 inside the inverse logmean's series) and agrees to rounding
    assert results["ec_flux_half_mismatches"] == 0
    assert results["ec_flux_half_energy"] < 1e-15


def test_mixed_reduced_flux(results):
    # FP32 flux on perturbations vs the FP64 flux reduced the same way,
    # relative to the largest reduced flux component, for low-Mach states
    # with 30 % density variation (temperature terms of ~50 cancel to ~1)
    assert results["mixed_reduced_flux"] < 1e-4


def test_adjoint_derivatives(results):
    # hand-written transposes against central differences (h = 1e-6); the
    # worst cases are directional derivatives ~1e-8 of fluxes ~1e2, where the
    # difference quotient's own round-off is ~1e-6 relative
    assert results["flux_vjp_vs_fd"] < 1e-5
    assert results["entropy_jvp_vs_fd"] < 1e-6
    # the entropy maps are gradients / inverse gradients: symmetric Jacobians
    assert results["entropy_jacobian_symmetry"] < 1e-13


def test_mixed_adjoint_derivatives(results):
    # FP32 transpose of the reduced flux (cotangent ob_rho + H_ref ob_E, ...)
    # mapped to conservative cotangents vs the FP64 transpose of the full
    # flux, relative to the largest cotangent, low-Mach states
    assert results["mixed_flux_vjp"] < 1e-5


def test_entropy_variable_maps(results):
    assert results["cons_to_entropy"] < 5e-14
    assert results["entropy_to_cons"] < 5e-14


def test_fp32_perturbation_entropy_maps(results):
    # the mixed form's FP32 entropy maps on perturbations from the reference
    # state against the FP64 maps, relative to the largest perturbation
    # component, for 0.1 %, 3 % and 30 % density and pressure perturbations
    # (the maps they replaced, FP64 algebra with FP32 log1p / expm1 and FP32
    # outputs, measured 1.1e-5 and 2.2e-5 on the same states)
    assert results["cons_to_entropy_pert"] < 3e-5
    assert results["entropy_to_cons_pert"] < 1e-4


def test_fp32_entropy_map_jvps(results):
    # the mixed-form VJP's FP32 Jacobian-vector products of both entropy maps
    # at absolute FP32 states against the FP64 ones, relative to the largest
    # component
    assert results["cons_to_entropy_jvp_f"] < 1e-5
    assert results["entropy_to_cons_jvp_f"] < 1e-5


def test_table_driven_log_and_exp(results):
    # sse_log / sse_exp (Tang's table-driven methods) against the C library
    # in extended precision: within 2 ulp of the result (for |log| < 1,
    # 2 ulp of 1: the entropy maps need absolute accuracy there), and every
    # out-of-range argument handed to the library functions (NaN logs of
    # negative pressures, which the non-physical flag relies on)
    assert results["table_log_ulps"] < 2.0
    assert results["table_exp_ulps"] < 2.0
    assert results["table_logexp_special_mismatches"] == 0
