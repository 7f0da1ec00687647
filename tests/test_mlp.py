"""The grid pruner's network: the numpy oracle pinned by finite differences (CPU), and the CUDA
forward / gradient / Adam kernels against it (GPU)."""

import numpy as np
import pytest

from oracle import mlp_ref as R


def _problem(seed, n=37):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, R.N_PARAMS)
    X = rng.normal(size=(n, 16))
    T = rng.normal(size=(n, 16))
    M = (rng.random((n, 16)) > 0.3).astype(float)
    return p, X, T, M


def test_oracle_gradient_matches_finite_differences():
    p, X, T, M = _problem(1, 9)
    inv = 1.0 / M.sum()
    _, g = R.loss_grad(p, X, T, M, inv)
    rng = np.random.default_rng(2)
    h = 1e-6
    for i in rng.integers(0, R.N_PARAMS, 40):
        e = np.zeros(R.N_PARAMS)
        e[i] = h
        fd = (R.loss_grad(p + e, X, T, M, inv)[0] - R.loss_grad(p - e, X, T, M, inv)[0]) / (2 * h)
        assert abs(fd - g[i]) < 1e-7 * max(1.0, abs(g[i]))


def test_library_shape_matches_oracle(native_lib):
    import ctypes
    vals = [ctypes.c_int() for _ in range(5)]
    assert native_lib.calchem_mlp_shape(*[ctypes.byref(v) for v in vals]) == 0
    n_in, n_hid, n_out, n_params, work = (v.value for v in vals)
    assert (n_in, n_hid, n_out, n_params) == (R.N_IN, R.N_HID, R.N_OUT, R.N_PARAMS)
    assert work == 4 * n_hid + n_out


def test_mlp_entry_points_reject_bad_arguments(native_lib):
    assert native_lib.calchem_mlp_forward(None, None, 4, None, None) == -1
    assert native_lib.calchem_mlp_adam(None, None, None, None, R.N_PARAMS, 1, 1e-3, 0.9, 0.999, 1e-8, None) == -1


@pytest.mark.gpu
def test_forward_gradient_and_adam_match_oracle(native_lib):
    torch = pytest.importorskip("torch")
    from calchem_gb300 import _native
    dev = torch.device("cuda:0")
    st = torch.cuda.current_stream(dev).cuda_stream
    p, X, T, M = _problem(3, 301)
    p32, X32, T32, M32 = (a.astype(np.float32) for a in (p, X, T, M))
    dp, dx, dt, dm = (torch.from_numpy(a).to(dev) for a in (p32, X32, T32, M32))
    y = torch.zeros((len(X), 16), dtype=torch.float32, device=dev)
    assert native_lib.calchem_mlp_forward(dp.data_ptr(), dx.data_ptr(), len(X), y.data_ptr(), st) == 0
    y_ref, _, _ = R.forward(p32.astype(np.float64), X32.astype(np.float64))
    torch.cuda.synchronize()
    assert np.max(np.abs(y.cpu().numpy() - y_ref)) < 1e-4
    inv = float(1.0 / M32.sum())
    work = torch.zeros(len(X) * (4 * 64 + 16), dtype=torch.float32, device=dev)
    lp = torch.zeros(len(X), dtype=torch.float32, device=dev)
    g = torch.zeros(R.N_PARAMS, dtype=torch.float32, device=dev)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    assert native_lib.calchem_mlp_loss_grad(dp.data_ptr(), dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), len(X), inv,
                                            work.data_ptr(), lp.data_ptr(), g.data_ptr(), loss.data_ptr(), st) == 0
    L_ref, g_ref = R.loss_grad(p32.astype(np.float64), X32.astype(np.float64), T32.astype(np.float64),
                               M32.astype(np.float64), inv)
    torch.cuda.synchronize()
    assert abs(float(loss.item()) - L_ref) < 1e-5 * abs(L_ref)
    gg = g.cpu().numpy()
    assert np.max(np.abs(gg - g_ref)) < 1e-5 * np.max(np.abs(g_ref))
    # deterministic: a second evaluation gives the same bits
    g2 = torch.zeros_like(g)
    native_lib.calchem_mlp_loss_grad(dp.data_ptr(), dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), len(X), inv,
                                     work.data_ptr(), lp.data_ptr(), g2.data_ptr(), loss.data_ptr(), st)
    torch.cuda.synchronize()
    assert np.array_equal(gg, g2.cpu().numpy())
    # one Adam step
    m = torch.zeros_like(dp)
    v = torch.zeros_like(dp)
    assert native_lib.calchem_mlp_adam(dp.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), R.N_PARAMS, 1, 1e-3,
                                       0.9, 0.999, 1e-8, st) == 0
    p_ref, _, _ = R.adam_step(p32.astype(np.float64), gg.astype(np.float64), 0.0, 0.0, 1, 1e-3)
    torch.cuda.synchronize()
    assert np.max(np.abs(dp.cpu().numpy() - p_ref)) < 1e-6
    _native.load()


@pytest.mark.gpu
def test_training_lowers_the_loss(native_lib):
    pytest.importorskip("torch")
    from calchem_gb300 import pruner
    rng = np.random.default_rng(5)
    L = len(pruner.LEVELS)
    X = rng.normal(size=(200, 16))
    Y = -8.0 + X[:, :L] @ rng.normal(0, 0.5, (L, L))  # a learnable map to one value per level
    net = pruner.Network(feature_mean=X.mean(0), feature_std=X.std(0), seed=1)
    hist = net.fit(X, Y, steps=600, lr=3e-3)
    assert hist[-1][1] < 0.1 * hist[0][1]
    pred = net.predict(X)
    assert np.sqrt(np.mean((pred[:, :L - 1] - Y[:, :L - 1]) ** 2)) < 0.5
