"""The density-predicting U-Net of the reference's am.ai module (TopOptUNet,
AIOptimizer; src/am/ai/model.py:18-67, inference.py:18-133), on the engine's
tensor-core convolutions: the forward pass and the per-layer weight gradients
against a float64 PyTorch CPU reference of the same architecture for both base
widths, the problem encoding, and training / prediction / validation / checkpoint
round trip on a small problem family."""
import numpy as np
import pytest

from am_ml_suite_gb300 import _native as nat
from am_ml_suite_gb300.core import DOF, BoundaryCondition, DistributedLoad, LoadCase, PointLoad, VoxelDomain


def _spec(f0):
    f1, f2, f3 = 2 * f0, 4 * f0, 8 * f0
    return [(16, f0), (f0, f0), (f0, f1), (f1, f1), (f1, f2), (f2, f2), (f2, f3), (f3, f3), (3 * f2, f2), (f2, f2),
            (3 * f1, f1), (f1, f1), (3 * f0, f0), (f0, f0), (f0, 16)]


def _split(w, spec):
    out, o = [], 0
    for cin, cout in spec:
        n = 27 * cout * cin
        out.append(w[o:o + n].reshape(27, cout, cin))
        o += n
    assert o == w.size
    return out


def _reference(x, ws, n_out):
    """float64 CPU reference: x (n, gz, gy, gx, c); ws per layer [27][cout][cin];
    returns the raw outputs (n, gz, gy, gx, n_out) and the weight tensors."""
    torch = pytest.importorskip("torch")
    F = torch.nn.functional
    W = [torch.tensor(w, dtype=torch.float64, requires_grad=True) for w in ws]

    def conv(l, t, relu=True):
        cout = W[l].shape[1]
        cin = t.shape[1]
        k = W[l][:, :, :cin].reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
        y = F.conv3d(t, k, padding=1)
        return F.relu(y) if relu else y

    def up(t):
        return F.interpolate(t, scale_factor=2, mode="nearest")

    t = torch.tensor(x, dtype=torch.float64).permute(0, 4, 1, 2, 3)
    e1 = conv(1, conv(0, t))
    e2 = conv(3, conv(2, F.avg_pool3d(e1, 2)))
    e3 = conv(5, conv(4, F.avg_pool3d(e2, 2)))
    e4 = conv(7, conv(6, F.avg_pool3d(e3, 2)))
    d3 = conv(9, conv(8, torch.cat([up(e4), e3], 1)))
    d2 = conv(11, conv(10, torch.cat([up(d3), e2], 1)))
    d1 = conv(13, conv(12, torch.cat([up(d2), e1], 1)))
    out = conv(14, d1, relu=False)[:, :n_out].permute(0, 2, 3, 4, 1)
    return out, W


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_encoding_and_arguments():
    from am_ml_suite_gb300.ai import AIOptimizer, TopOptUNet
    from am_ml_suite_gb300.ai.inference import element_loads

    shape = (4, 3, 2)
    nx, ny, nz = shape
    grid = np.zeros(shape, np.int8)
    grid[0, 0, 0] = -1
    grid[3, 2, 1] = 1
    dom = VoxelDomain(grid=grid, resolution_mm=1.0)
    node = nx * (ny + 1) * (nz + 1)  # (nx, 0, 0)
    lc = LoadCase(name="t", point_loads=[PointLoad(node_index=node, force_vector=np.array([0.0, 0.0, -8.0]))])
    e = element_loads(dom, [lc])
    assert e.shape == (3, nx, ny, nz)
    assert e[2, nx - 1, 0, 0] == -1.0 and np.count_nonzero(e) == 1  # one corner node: 1/8 of it, rescaled
    x = AIOptimizer(device="cuda").encode_problem(dom, [lc])
    assert x.shape == (4, nx, ny, nz) and np.array_equal(x[0], grid.astype(np.float32))
    # 7 channels: the constrained DOFs of the x = 0 face (component z only) on the elements
    fixed_nodes = np.array([j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)])
    lc.boundary_conditions = [BoundaryCondition(node_indices=fixed_nodes, constrained_dofs=[DOF.UZ])]
    x7 = AIOptimizer().encode_problem(dom, [lc], channels=7)
    assert x7.shape == (7, nx, ny, nz) and np.array_equal(x7[:4], x)
    assert np.all(x7[4] == 0) and np.all(x7[5] == 0)
    assert np.all(x7[6][0] == 0.5) and np.all(x7[6][1:] == 0)  # half of an x = 0 element's nodes
    with pytest.raises(ValueError):
        AIOptimizer().encode_problem(dom, [lc], channels=5)
    with pytest.raises(ValueError):
        TopOptUNet(features=(32, 64, 128, 512))
    with pytest.raises(ValueError):
        AIOptimizer(device="cpu")


@pytest.mark.gpu
@pytest.mark.parametrize("f0,shape", [(16, (2, 16, 8, 8)), (32, (1, 8, 24, 16))])
def test_unet_forward_and_gradients_match_reference(f0, shape):
    torch = pytest.importorskip("torch")
    n, gz, gy, gx = shape
    net = nat.UNet(4, 1, f0, seed=1)
    spec = _spec(f0)
    rng = np.random.default_rng(2)
    ws = []
    for l, (cin, cout) in enumerate(spec):
        used_in = 4 if l == 0 else cin
        used_out = 1 if l == len(spec) - 1 else cout
        w = np.zeros((27, cout, cin), np.float32)
        w[:, :used_out, :used_in] = rng.uniform(-1, 1, size=(27, used_out, used_in)) * np.sqrt(6.0 / (27 * used_in))
        ws.append(w)
    net.set_params(np.concatenate([w.ravel() for w in ws]))
    ws = [w.astype(np.float64) for w in _split(net.get_params(), spec)]
    x = rng.normal(size=(n, gz, gy, gx, 4)).astype(np.float32)
    dout = rng.normal(size=(n, gz, gy, gx, 1)).astype(np.float32)
    ref, W = _reference(x.astype(np.float64), ws, 1)
    got = net.forward(x, sigmoid=False)
    assert _rel(got, ref.detach().numpy()) <= 3e-2
    sig = net.forward(x, sigmoid=True)
    assert np.allclose(sig, 1.0 / (1.0 + np.exp(-got.astype(np.float64))), atol=1e-6)
    (ref * torch.tensor(dout, dtype=torch.float64)).sum().backward()
    g = _split(net.param_grad(x, dout), spec)
    errs, coss = [], []
    for l, (cin, cout) in enumerate(spec):
        used_in = 4 if l == 0 else cin
        used_out = 1 if l == len(spec) - 1 else cout
        gr = W[l].grad.numpy()[:, :used_out, :used_in]
        gg = g[l][:, :used_out, :used_in].astype(np.float64)
        errs.append(_rel(gg, gr))
        coss.append(float((gr * gg).sum() / (np.linalg.norm(gr) * np.linalg.norm(gg))))
    print("relative gradient error per layer", np.round(errs, 4))
    assert errs[14] <= 2e-2 and max(errs) <= 0.2, errs
    assert min(coss) >= 0.98, coss


def _cantilever_family(rng, shape=(16, 8, 8)):
    nx, ny, nz = shape
    base = np.array([j * (nz + 1) + k for j in range(ny + 1) for k in range(nz + 1)])
    j0 = int(rng.integers(1, ny))
    nodes = np.array([nx * (ny + 1) * (nz + 1) + j * (nz + 1) + nz // 2 for j in (j0 - 1, j0)])
    th = rng.uniform(-0.6, 0.6)
    return LoadCase(name="c", boundary_conditions=[BoundaryCondition(node_indices=base)],
                    distributed_loads=[DistributedLoad(node_indices=nodes,
                                                       total_force=np.array([0.0, np.sin(th), -np.cos(th)]))])


@pytest.mark.gpu
def test_train_predict_validate_and_checkpoint(tmp_path):
    from am_ml_suite_gb300.ai import AIOptimizer, TopOptUNet, load_pretrained
    from am_ml_suite_gb300.ai.train import padded
    from am_ml_suite_gb300.numerical.fem import MaterialProperties
    from am_ml_suite_gb300.numerical.topopt import SIMPOptimizer, SIMPParams

    rng = np.random.default_rng(7)
    shape = (16, 8, 8)
    dom = VoxelDomain(grid=np.zeros(shape, np.int8), resolution_mm=1000.0)
    prm = SIMPParams(volume_fraction=0.3, filter_radius=1.5, max_iterations=15, convergence_tol=0.0,
                     precision=nat.PREC_MIXED, cg_tol=1e-6)
    enc = AIOptimizer()
    X, T, cases = [], [], []
    for _ in range(12):
        lc = _cantilever_family(rng, shape)
        X.append(enc.encode_problem(dom, [lc]))
        T.append(SIMPOptimizer(dom, [lc], MaterialProperties(E=1.0, nu=0.3), prm, verbose=False).run().density)
        cases.append(lc)
    x, t, m = padded(dom, np.stack(X[:10]), np.stack(T[:10]))
    model = TopOptUNet(4, 1, (16, 32, 64, 128), seed=3)
    model.net.set_data(x, t, m)
    before = model.net.eval()
    losses = model.net.train(epochs=40, batch=5, lr=2e-3, seed=1)
    after = model.net.eval()
    assert np.all(np.isfinite(losses)) and after < 0.5 * before, (before, after)
    model.meta = {"volume_fraction": 0.3, "filter_radius": 1.5, "simp_iterations": 15}
    ai = AIOptimizer()
    ai.model = model
    pred = ai.predict(dom, [cases[10]])
    assert pred.shape == shape and set(np.unique(pred)) <= {0.0, 1.0}
    v = ai.validate_against_numerical(dom, [cases[10]], numerical_density=T[10])
    assert 0.0 <= v["iou"] <= 1.0 and np.isfinite(v["compliance_error"]) and abs(v["volume_error"]) < 0.5
    path = str(tmp_path / "unet.npz")
    model.save(path)
    again = load_pretrained(path)
    assert again.features == (16, 32, 64, 128) and again.meta["volume_fraction"] == 0.3
    assert np.array_equal(again.predict(enc.encode_problem(dom, [cases[11]])),
                          model.predict(enc.encode_problem(dom, [cases[11]])))


@pytest.mark.gpu
def test_seven_channel_model_predicts_and_round_trips(tmp_path):
    """The 7-channel encoding (constrained DOFs on channels 4-6) through a
    TopOptUNet(7, ...): prediction shape and range, checkpoint round trip, and the
    optimizer encoding for the loaded model's channel count."""
    from am_ml_suite_gb300.ai import AIOptimizer, TopOptUNet, load_pretrained

    shape = (16, 8, 8)
    nx, ny, nz = shape
    dom = VoxelDomain(grid=np.zeros(shape, np.int8), resolution_mm=1000.0)
    lc = _cantilever_family(np.random.default_rng(5), shape)
    model = TopOptUNet(7, 1, (16, 32, 64, 128), seed=2)
    x = AIOptimizer().encode_problem(dom, [lc], channels=7)
    rho = model.predict(x)
    assert rho.shape == shape and np.all((rho > 0) & (rho < 1))
    path = str(tmp_path / "u7.npz")
    model.save(path)
    ai = AIOptimizer(model_path=path)
    assert ai.model.in_channels == 7 and ai.encode_problem(dom, [lc]).shape == (7, nx, ny, nz)
    assert np.array_equal(ai.model.predict(x), load_pretrained(path).predict(x))
