"""The network's convolutions on the 5th-generation tensor cores (tcgen05.mma,
TMEM accumulators, tiled tensor-copy staging) against a float64 PyTorch CPU
reference of the same network and against the legacy mma.sync kernels: forward
outputs and per-layer weight gradients, on grids whose coarse levels do not fill
the 8 x 4 x 4 voxel tiles (partial tiles, zero-filled halos)."""
import numpy as np
import pytest

from am_ml_suite_gb300 import _native as nat

from test_precond import SPEC, _random_params, _rel, _split, _unet_reference

pytestmark = pytest.mark.gpu


@pytest.fixture
def kernels():
    yield nat.set_conv_kernels
    nat.set_conv_kernels(nat.CONV_TCGEN05)


@pytest.mark.parametrize("shape", [(2, 16, 8, 8), (1, 8, 24, 40)])
def test_tcgen05_forward_and_gradients_match_reference(kernels, shape):
    torch = pytest.importorskip("torch")
    n, gz, gy, gx = shape
    pre = nat.Preconditioner(seed=1, capacity=0)
    ws = _random_params(pre, 2)
    rng = np.random.default_rng(3)
    x = rng.normal(size=(n, gz, gy, gx, 4)).astype(np.float32)
    dout = rng.normal(size=(n, gz, gy, gx, 3)).astype(np.float32)
    ref, W = _unet_reference(x.astype(np.float64), ws)
    (ref * torch.tensor(dout, dtype=torch.float64)).sum().backward()
    ref = ref.detach().numpy()
    got, grads = {}, {}
    for impl in (nat.CONV_TCGEN05, nat.CONV_MMA_SYNC):
        kernels(impl)
        got[impl] = pre.forward(x)
        grads[impl] = _split(pre.param_grad(x, dout))
    kernels(nat.CONV_TCGEN05)
    # BF16 weights and activations through 15 layers: ~1 % relative either way
    assert _rel(got[nat.CONV_TCGEN05], ref) <= 3e-2
    assert _rel(got[nat.CONV_TCGEN05], got[nat.CONV_MMA_SYNC]) <= 3e-2
    errs, coss = [], []
    for l, (cin, _) in enumerate(SPEC):
        used = 4 if l == 0 else cin
        gr = W[l].grad.numpy()[:, :, :used]
        gg = grads[nat.CONV_TCGEN05][l][:, :, :used].astype(np.float64)
        errs.append(_rel(gg, gr))
        coss.append(float((gr * gg).sum() / (np.linalg.norm(gr) * np.linalg.norm(gg))))
    print("tcgen05 relative gradient error per layer", np.round(errs, 4), "cosine", np.round(coss, 5))
    assert errs[14] <= 2e-2 and errs[13] <= 6e-2, errs
    assert max(errs) <= 0.2, errs
    assert min(coss) >= 0.98, coss
    assert np.all(grads[nat.CONV_TCGEN05][0][:, :, 4:] == 0.0)


def test_tcgen05_forward_is_deterministic(kernels):
    pre = nat.Preconditioner(seed=5, capacity=0)
    _random_params(pre, 6)
    x = np.random.default_rng(7).normal(size=(1, 16, 16, 24, 4)).astype(np.float32)
    a = pre.forward(x)
    b = pre.forward(x)
    assert np.array_equal(a, b)
