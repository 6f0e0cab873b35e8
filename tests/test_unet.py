"""The learned preconditioner's U-Net: the numpy oracle's backward pass against
finite differences (CPU), and the CUDA forward, loss and parameter gradients
against the oracle (GPU).

Tolerances: the CUDA kernels store bf16 activations and accumulate in fp32 in a
different order than the oracle; with the oracle rounding at the same points,
outputs agree to ~1e-2 relative and gradients to a few 1e-2 (an occasional
bf16 rounding flip of an intermediate value is the main source)."""
import numpy as np
import pytest

from oracle import unet_oracle as uo


def _inputs(shape, seed):
    rng = np.random.default_rng(seed)
    nb, Z, Y, X = shape
    x = rng.standard_normal((nb, Z, Y, X, 8))
    x[..., 6] = rng.uniform(-0.5, 0.5, (nb, Z, Y, X))
    x[..., 7] = 0.0
    t = rng.standard_normal((nb, Z, Y, X, 3)) * 0.3
    m = rng.integers(0, 16, (nb, Z, Y, X)).astype(np.uint8) | 7
    return x, t, m


def test_parameter_count():
    assert uo.effective_params() == 246_931
    from topoptspline3d_gb300 import capi
    assert capi.Problem.unet_num_params() == uo.num_params()


def test_oracle_backward_matches_finite_differences():
    p = uo.random_params(3)
    x, t, m = _inputs((1, 8, 8, 8), 0)
    L, g = uo.UNetOracle(p, bf16_round=False).loss_grad(x, t, m)
    rng = np.random.default_rng(1)
    wo, bo, _ = uo.offsets()
    # one weight and one bias from every layer
    idx = []
    for l, (cin, cout, _, ci, co) in enumerate(uo.LAYERS):
        idx.append(wo[l] + (rng.integers(co) * 27 + rng.integers(27)) * cin + rng.integers(ci))
        idx.append(bo[l] + rng.integers(co))
    for i in idx:
        e = 1e-6
        pp = p.copy(); pp[i] += e
        pm = p.copy(); pm[i] -= e
        fd = (uo.UNetOracle(pp, False).loss_grad(x, t, m)[0] - uo.UNetOracle(pm, False).loss_grad(x, t, m)[0]) / (2 * e)
        assert abs(g[i] - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(g).max()), (i, g[i], fd)


def test_bf16_rounding_helper():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-30])
    b = uo.bf16(a)
    assert b[0] == 1.0 and b[1] == 1.0  # tie to even
    assert b[2] == 1.0078125
    assert abs(b[3] + 3.140625) < 1e-12


def _gpu_problem(kernel=None):
    from topoptspline3d_gb300 import capi
    p = capi.Problem(8, 8, 8)
    p.unet_enable(5)
    if kernel is not None:
        p.unet_set_conv_kernel(kernel)
    return p


KERNELS = pytest.mark.parametrize("kernel", [1, 0], ids=["tcgen05", "mma_sync"])


@pytest.mark.gpu
@KERNELS
@pytest.mark.parametrize("shape", [(2, 16, 16, 16), (1, 8, 16, 24), (1, 8, 24, 40)])
def test_forward_matches_oracle(shape, kernel):
    prm = uo.random_params(7).astype(np.float32)
    g = _gpu_problem(kernel)
    g.unet_set_params(prm)
    assert np.array_equal(g.unet_params(), prm)
    x, _, _ = _inputs(shape, 2)
    y = g.unet_forward(x.astype(np.float32))
    yo = uo.UNetOracle(prm.astype(np.float64)).forward(x.astype(np.float32).astype(np.float64))
    err = np.linalg.norm(y - yo) / np.linalg.norm(yo)
    assert err < 1e-2, err


@pytest.mark.gpu
@KERNELS
def test_loss_and_gradients_match_oracle(kernel):
    prm = uo.random_params(9).astype(np.float32)
    g = _gpu_problem(kernel)
    g.unet_set_params(prm)
    x, t, m = _inputs((2, 16, 16, 16), 4)
    x32, t32 = x.astype(np.float32), t.astype(np.float32)
    loss, grad = g.unet_loss_grad(x32, t32, m)
    lo, go = uo.UNetOracle(prm.astype(np.float64)).loss_grad(x32.astype(np.float64), t32.astype(np.float64), m)
    assert abs(loss - lo) <= 1e-3 * lo
    wo, bo, _ = uo.offsets()
    for l, (cin, cout, *_r) in enumerate(uo.LAYERS):
        for a, b in ((wo[l], wo[l] + cout * 27 * cin), (bo[l], bo[l] + cout)):
            ref = go[a:b]
            err = np.linalg.norm(grad[a:b] - ref) / max(np.linalg.norm(ref), 1e-30)
            assert err < 3e-2, (l, a, err)


@pytest.mark.gpu
def test_zero_last_layer_is_identity_correction():
    """A freshly enabled network has a zero last layer: its output is exactly 0."""
    g = _gpu_problem()
    x, _, _ = _inputs((1, 16, 16, 16), 8)
    assert np.count_nonzero(g.unet_forward(x.astype(np.float32))) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(2, 16, 16, 16), (1, 8, 24, 40), (3, 8, 8, 32)])
def test_tcgen05_convolutions_match_mma_sync(shape):
    """The tcgen05 + TMA convolutions against the mma.sync ones on the same
    weights and inputs: the two differ only in the fp32 summation order (and
    in the bf16 roundings of activations that order can flip), so the network
    output and the parameter gradient agree to 5e-3."""
    prm = uo.random_params(11).astype(np.float32)
    x, t, m = _inputs(shape, 12)
    x32, t32 = x.astype(np.float32), t.astype(np.float32)
    out = {}
    for kernel in (1, 0):
        g = _gpu_problem(kernel)
        g.unet_set_params(prm)
        y = g.unet_forward(x32)
        loss, grad = g.unet_loss_grad(x32, t32, m)
        out[kernel] = (y, loss, grad)
    (y1, l1, g1), (y0, l0, g0) = out[1], out[0]
    assert np.linalg.norm(y1 - y0) <= 5e-3 * np.linalg.norm(y0)
    assert abs(l1 - l0) <= 5e-3 * abs(l0)
    assert np.linalg.norm(g1 - g0) <= 5e-3 * np.linalg.norm(g0)
