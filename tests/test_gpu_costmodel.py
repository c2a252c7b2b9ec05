"""The learned cost model's kernels (tq_mlp_*) against the CPU oracle
(oracle/mlp_oracle.py, float64): forward outputs, loss and every parameter
gradient, and Adam steps.  Tolerances are those of float32 arithmetic against
float64: outputs and loss within 1e-5 relative, gradients within 1e-4 of the
largest gradient, parameters after 5 Adam steps within 1e-4 relative."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

N_IN, WIDTH, N_OUT = 32, 64, 46


def data(seed, n=200):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, N_IN)).astype(np.float32)
    T = rng.standard_normal((n, N_OUT)).astype(np.float32)
    M = (rng.random((n, N_OUT)) < 0.8).astype(np.float32)
    return X, T, M


def test_forward_and_gradients_match_oracle(tq):
    from torque_gb300.costmodel import MLP
    net = MLP(N_IN, WIDTH, N_OUT, seed=3)
    p = net.get_params()
    X, T, M = data(0)
    y = net.forward(X)
    y_ref, _ = mo.forward(p, X, N_IN, WIDTH, N_OUT)
    assert np.max(np.abs(y - y_ref)) <= 1e-5 * np.max(np.abs(y_ref))
    loss, g = net.gradients(X, T, M)
    loss_ref, g_ref = mo.loss_and_grad(p, X, T, N_IN, WIDTH, N_OUT, M)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    gerr = np.max(np.abs(g - g_ref)) / np.max(np.abs(g_ref))
    print("gradient max error / max gradient: %.2e" % gerr)
    assert gerr <= 1e-4
    # without a mask every output counts
    loss1, g1 = net.gradients(X, T)
    loss1_ref, g1_ref = mo.loss_and_grad(p, X, T, N_IN, WIDTH, N_OUT)
    assert abs(loss1 - loss1_ref) <= 1e-5 * loss1_ref
    assert np.max(np.abs(g1 - g1_ref)) <= 1e-4 * np.max(np.abs(g1_ref))


def test_adam_steps_match_oracle(tq):
    import ctypes

    import torch

    from torque_gb300 import _lib
    from torque_gb300.costmodel import MLP
    net = MLP(N_IN, WIDTH, N_OUT, seed=5)
    p = net.get_params().astype(np.float64)
    X, T, M = data(1, 64)
    x, t, m = (torch.as_tensor(a).cuda() for a in (X, T, M))
    mom, vel = np.zeros_like(p), np.zeros_like(p)
    lr = 1e-3
    for step in range(1, 6):
        _lib.check(_lib.load().tq_mlp_train_step(net._h, ctypes.c_void_p(x.data_ptr()),
                                                 ctypes.c_void_p(t.data_ptr()),
                                                 ctypes.c_void_p(m.data_ptr()), 64,
                                                 ctypes.c_float(lr), None, None))
        _, g = mo.loss_and_grad(p, X, T, N_IN, WIDTH, N_OUT, M)
        p, mom, vel = mo.adam_step(p, g, mom, vel, step, lr)
    torch.cuda.synchronize()
    got = net.get_params()
    err = np.max(np.abs(got - p)) / np.max(np.abs(p))
    print("params after 5 Adam steps: max rel error %.2e" % err)
    assert err <= 1e-4


def test_training_is_deterministic_and_learns(tq):
    from torque_gb300.costmodel import MLP
    rng = np.random.default_rng(2)
    X = rng.standard_normal((300, N_IN)).astype(np.float32)
    W = rng.standard_normal((N_IN, N_OUT)).astype(np.float32) / np.sqrt(N_IN)
    T = np.tanh(X @ W).astype(np.float32)  # a smooth target the network can fit
    a, b = MLP(N_IN, WIDTH, N_OUT, seed=9), MLP(N_IN, WIDTH, N_OUT, seed=9)
    l0, _ = a.gradients(X, T)
    ca = a.fit(X, T, steps=400, lr=3e-3, log_every=100)
    b.fit(X, T, steps=400, lr=3e-3)
    assert np.array_equal(a.get_params(), b.get_params())
    l1, _ = a.gradients(X, T)
    print("loss %.4f -> %.4f" % (l0, l1), ca)
    assert l1 < 0.2 * l0


def test_plan_features(tq):
    from torque_gb300 import workloads
    c = workloads.small_u1()
    A = tq.BlockSparseTensor(c.A.dimension, c.a_data, c.A.begin.T, c.A.end.T)
    B = tq.BlockSparseTensor(c.B.dimension, c.b_data, c.B.begin.T, c.B.end.T)
    P = tq.ContractionPlan(A, B, c.pairs, precision="ozaki", layout="reduced")
    f = P.features(1e-10)
    assert f.shape == (32,)
    assert abs(f[0] - 10 / 16) < 1e-6
    assert f[1] == 0.5 and f[2] == 0.5 and f[3] == 0.5
    assert abs(f[4] - np.log2(24 * 24) / 32) < 1e-6
    assert abs(f[5] - np.log2(c.flops() + 1) / 48) < 1e-6
    for g in range(3):
        assert abs(f[8 + 8 * g:16 + 8 * g].sum() - 1.0) < 1e-5
    # m = n = k = products of two sector sizes in {3,5,8}: 9..64, bins 1..4
    assert f[8] == 0.0 and f[8 + 5:16].sum() == 0.0


def test_trained_model_regret_and_gain(tq):
    """Trained on the tuner's measurements of 1,800 random contractions (library
    kernels only), evaluated on the 200 held out: the model's proposals stay close
    to the exhaustive tuner (mean regret = mean of ms_pick / ms_best - 1) and
    beat the schedule the library takes without the model (5 slices for 1e-10,
    4 for 1e-8, tile width 96, no grouping) by a wide margin."""
    from torque_gb300 import costmodel as cm
    recs = cm.load_records(cm.DATASET)
    train, test = cm.split(recs)
    net, curve = cm.train(train, steps=3000)
    for eps in (1e-8, 1e-10):
        m = cm.regret_report(test, cm.model_choices(net, test, eps), eps)
        d = cm.regret_report(test, [cm.default_choice(eps)] * len(test), eps)
        gain = d["ms_total"] / m["ms_total"]
        print("target %g: model mean regret %.3f (median %.3f, p90 %.3f), misses %.3f; "
              "default mean regret %.3f; gain over default %.2fx"
              % (eps, m["mean_regret"], m["median_regret"], m["p90_regret"], m["miss_rate"],
                 d["mean_regret"], gain))
        assert m["mean_regret"] <= 0.15
        assert m["miss_rate"] <= 0.02
        assert gain >= 1.5
