"""GPU: the learned predictor's tensor-core kernels (tcgen05, BF16 operands,
FP32 accumulation in tensor memory) against the CPU oracle (oracle/gnn):
the product kernel on its own, the network's forward pass, its gradients,
and a short training run."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle", "gnn"))
import gnn_ref as R  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G(built_lib):
    from ngspice_gb300 import gnn
    return gnn


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("M,N,K,splits", [(128, 16, 16, 1), (256, 64, 64, 1), (128, 128, 128, 1),
                                          (384, 64, 192, 1), (128, 64, 1024, 4), (128, 16, 640, 3)])
def test_tensor_core_product(G, M, N, K, splits):
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    ref = R.bf16(A).astype(np.float64) @ R.bf16(B).astype(np.float64).T
    got = G.gemm_test(A, B, splits)
    # FP32 accumulation of exact BF16 products: relative error ~ K * 2^-24
    assert np.max(np.abs(got - ref)) <= 1e-5 * np.sqrt(K) * np.max(np.abs(ref)) + 1e-6


def random_graph(n, seed):
    rng = np.random.default_rng(seed)
    nb = [set() for _ in range(n)]
    for i in range(1, n):                      # a connected, circuit-like graph
        j = int(rng.integers(max(0, i - 20), i))
        nb[i].add(j)
        nb[j].add(i)
    for _ in range(n):
        i, j = rng.integers(0, n, 2)
        if i != j:
            nb[i].add(int(j))
            nb[j].add(int(i))
    ptr = np.zeros(n + 1, np.int32)
    idx = []
    for i in range(n):
        idx += sorted(nb[i])
        ptr[i + 1] = len(idx)
    deg = np.diff(ptr)
    dinv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0).astype(np.float32)
    return ptr, np.array(idx, np.int32), dinv


def sample(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, R.F_IN)).astype(np.float32)
    y = (0.5 * np.tanh(X[:, 1]) - 0.3 * X[:, 2] * X[:, 3]).astype(np.float32)
    w = np.ones(n, np.float32)
    return X, y, w


def test_forward_matches_oracle(G):
    n = 300
    ptr, idx, dinv = random_graph(n, 1)
    p = R.init_params(2)
    net = G.Net(ptr, idx)
    net.set_params(G.flatten(p))
    X, _, _ = sample(n, 3)
    ref, _ = R.forward(p, X, ptr, idx, dinv)
    got = net.forward(X)
    # BF16 re-rounding of activations that differ in the last FP32 bits
    assert rel(got, ref) <= 1e-2


def test_gradients_match_oracle(G):
    n = 500
    ptr, idx, dinv = random_graph(n, 4)
    p = R.init_params(5)
    net = G.Net(ptr, idx)
    net.set_params(G.flatten(p))
    X, y, w = sample(n, 6)
    loss_ref, g_ref, _ = R.loss_and_grad(p, X, ptr, idx, dinv, y, w)
    loss, g = net.train_step(X, y, w, lr=0.0, want_grads=True)
    assert abs(loss - loss_ref) <= 1e-3 * abs(loss_ref)
    got = G.unflatten(g)
    for k in g_ref:
        assert rel(got[k], g_ref[k]) <= 3e-2, k


def test_training_reduces_loss(G):
    n = 800
    ptr, idx, dinv = random_graph(n, 7)
    net = G.Net(ptr, idx)
    net.set_params(G.flatten(R.init_params(8)))
    X, y, w = sample(n, 9)
    first, _ = net.train_step(X, y, w, lr=0.0)
    for _ in range(150):
        last, _ = net.train_step(X, y, w, lr=3e-3)
    assert last < 0.2 * first
