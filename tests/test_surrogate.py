"""Green-function surrogate (k_mlp.cu): the network's own forward/backward kernels
against the CPU oracle (oracle/mlp_oracle.py), training on samples from the plain
integrator, and what the trained network gains over the closed form it replaces."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def _rand_params(seed=1):
    rng = np.random.default_rng(seed)
    p = []
    for l in range(len(mo.DIMS) - 1):
        i, n = mo.DIMS[l], mo.DIMS[l + 1]
        p.append(rng.uniform(-1, 1, n * i) * np.sqrt(6.0 / (i + n)))
        p.append(rng.normal(0, 0.1, n))
    return np.concatenate(p)


def test_oracle_gradient_finite_differences():
    """The oracle's backward pass against central differences (unquantised weights)."""
    rng = np.random.default_rng(0)
    p = _rand_params()
    x = rng.normal(size=(7, 2))
    t = rng.normal(size=(7, 6))
    loss, g = mo.loss_and_grad(p, x, t, quantize=False)
    idx = rng.choice(p.size, 40, replace=False)
    for k in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mo.loss_and_grad(pp, x, t, False)[0] - mo.loss_and_grad(pm, x, t, False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 0.0], dtype=np.float32)
    q = mo.bf16(v)
    assert q[0] == 1.0 and q[1] == 1.0  # ties to even
    assert q[2] == np.float32(1.0078125)
    assert abs(q[3] + 3.140625) < 1e-7


@pytest.mark.gpu
def test_gpu_forward_backward_match_oracle():
    import bemuse_gb300 as bg
    s = bg.HavelockSurrogate(seed=3)
    p = _rand_params(5)
    s.set_params(p)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(300, 2))
    t = rng.normal(size=(300, 6))
    # identity normalisation: eval sees x, y directly
    s.set_normalization([0, 0], [1, 1], np.zeros(6), np.ones(6))
    y_gpu = s.eval(x)
    y_ref = mo.forward(p, x)[0]
    err = np.max(np.abs(y_gpu - y_ref)) / np.max(np.abs(y_ref))
    print("surrogate forward vs oracle:", err)
    assert err < 2e-5
    loss_gpu, g_gpu = s.grad(x, t)
    loss_ref, g_ref = mo.loss_and_grad(p, x, t)
    print("loss", loss_gpu, loss_ref, "grad rel", np.max(np.abs(g_gpu - g_ref)) / np.max(np.abs(g_ref)))
    assert abs(loss_gpu - loss_ref) <= 1e-5 * loss_ref
    assert np.max(np.abs(g_gpu - g_ref)) <= 1e-4 * np.max(np.abs(g_ref))


@pytest.mark.gpu
def test_tensor_core_forward_matches_oracle():
    """The tcgen05 forward (BF16 weights and activations, FP32 accumulation in TMEM)
    against the oracle with BF16-rounded activations, on a sample count that is not a
    multiple of the 128-sample tile.  Differences come from FP32 summation order, the
    hardware tanh in SiLU and the BF16 roundings these shift; a wrong operand layout
    would give O(1) errors."""
    import bemuse_gb300 as bg
    s = bg.HavelockSurrogate(seed=4)
    p = _rand_params(6)
    s.set_params(p)
    s.set_normalization([0, 0], [1, 1], np.zeros(6), np.ones(6))
    rng = np.random.default_rng(9)
    x = rng.normal(size=(1000, 2)) * 1.5
    y_tc = s.eval_tc(x)
    y_ref = mo.forward(p, x, act_bf16=True)[0]
    err = np.max(np.abs(y_tc - y_ref)) / np.max(np.abs(y_ref))
    err32 = np.max(np.abs(y_tc - s.eval(x))) / np.max(np.abs(y_ref))
    print("tensor-core forward vs BF16-activation oracle %.3e, vs FP32-activation kernel %.3e" % (err, err32))
    assert err < 1e-2 and err32 < 2e-2
    # the weights change: the operand image follows
    p2 = _rand_params(7)
    s.set_params(p2)
    err2 = np.max(np.abs(s.eval_tc(x[:130]) - mo.forward(p2, x[:130], act_bf16=True)[0])) / np.max(
        np.abs(mo.forward(p2, x[:130], act_bf16=True)[0]))
    assert err2 < 1e-2


@pytest.mark.gpu
def test_training_and_gain_report():
    """Trains on samples of the plain FP64 integrator in the surrogate's domain (targets
    divided by the per-sample envelope) and reports accuracy and throughput: the
    tensor-core network against the FP32 closed form it would replace.  The closed form
    is expected to be faster and the network's error far above the 1e-6 the solve
    needs; a negative result, reported."""
    import bemuse_gb300 as bg
    x, y, t = bg.HavelockSurrogate.domain_set(1 << 17, seed=0)
    xv, yv, tv = bg.HavelockSurrogate.domain_set(1 << 13, seed=1)
    s = bg.HavelockSurrogate(seed=0)
    s.set_domain_normalization(t)
    losses = [s.train(x, t, epochs=1, batch=4096, lr=2e-3 * (0.93 ** e), seed=e)[0] for e in range(40)]
    print("losses", losses[0], losses[-1])
    assert losses[-1] < 0.2 * losses[0]
    pred = s.predict(xv)
    env = bg.HavelockSurrogate.envelope(10 ** xv[:, 0], xv[:, 1])
    med = np.median(np.abs(pred - yv) / env, axis=0)
    print("median error / envelope per output:", med)
    assert np.all(med < 0.05)
    mlp = s.throughput_tc(1 << 20)
    closed = bg.havelock_throughput(1 << 20, bg.MIXED)
    print("evaluations/s: tensor-core network %.3e, FP32 closed form %.3e" % (mlp, closed))
    assert mlp > 0 and closed > 0
