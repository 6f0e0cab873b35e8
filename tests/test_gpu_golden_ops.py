"""The CUDA fine-level kernels against the reference's own applyK, residual and
Gauss-Seidel kernels (golden vectors from tests/golden/make_ref_ops_golden.py,
see tests/test_golden_ref_ops.py): every form of the fine operator (modal FP64,
dense-row FP64, double-float, FP32), the FP64 residual and two forward
point-block Gauss-Seidel sweeps, through the C ABI."""
import numpy as np
import pytest

from topoptspline3d_gb300 import capi
from tests.helpers import rel
from tests.test_golden_ref_ops import CASES, golden_case

pytestmark = pytest.mark.gpu


def _problem(c):
    p = capi.Problem(c["nx"], c["ny"], c["nz"], 1.0, 1e6, 0.4, 3.0, 1e-3, eactive=c["eactive"])
    p.set_bc(c["fixed"], np.zeros(3 * c["nv"]))
    assert rel(p.get("ke"), c["ke"]) < 1e-13
    p.put("rho", c["rho"])
    return p


@pytest.mark.parametrize("name", CASES)
def test_fine_operator_forms_match_reference(name):
    c = golden_case(name)
    p = _problem(c)
    fr = c["free"]
    for prec, tol in ((0, 1e-12), (2, 1e-12), (3, 1e-12), (1, 1e-5)):
        ku = p.apply_fine(c["u"], prec)
        assert rel(ku[fr], c["Ku"][fr]) < tol, prec
    p.close()


@pytest.mark.parametrize("name", CASES)
def test_residual_and_gauss_seidel_match_reference(name):
    c = golden_case(name)
    p = _problem(c)
    p.update_operators()
    p.put("u", c["u"])
    p.put("f", c["f"])
    p.residual(0)
    assert rel(p.get("r"), c["r"]) < 1e-12
    p.put("u", c["u"])
    p.smooth(0, 2)
    assert rel(p.get("u"), c["gs2"]) < 1e-12
    p.close()
