"""TEST INFRASTRUCTURE ONLY -- numpy FP64 restatement of the learned-warm-start network.

The product path runs the network on the GPU (FP32 training kernels, BF16 tensor-core
inference); this module is the checker for its gradients and outputs.  The reference
code has no learned component (its CCD always starts from MP2 amplitudes,
ccm_iter.f90:2329-2368), so there is nothing to pin against the reference: the module
is pinned by finite differences instead (tests/test_mlp_oracle.py).

Network: 18 features -> 128 -> 128 -> 128 -> 1, SiLU after each hidden layer.
Parameter vector (float32 on the device, float64 here), row-major weights [out][in]:
    W1[128][18] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] w4[128] b4
Loss: mean over the batch of (f(x) - y)^2.
"""
import numpy as np

F, W = 18, 128
OFF_W1 = 0
OFF_B1 = OFF_W1 + W * F
OFF_W2 = OFF_B1 + W
OFF_B2 = OFF_W2 + W * W
OFF_W3 = OFF_B2 + W
OFF_B3 = OFF_W3 + W * W
OFF_W4 = OFF_B3 + W
OFF_B4 = OFF_W4 + W
N_PARAMS = OFF_B4 + 1


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(W, F), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(W, W), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3].reshape(W, W), p[OFF_B3:OFF_W4], p[OFF_W4:OFF_B4], p[OFF_B4])


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigmoid(z)


def dsilu(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def forward(p, X):
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p)
    X = np.asarray(X, np.float64)
    Z1 = X @ W1.T + b1
    H1 = silu(Z1)
    Z2 = H1 @ W2.T + b2
    H2 = silu(Z2)
    Z3 = H2 @ W3.T + b3
    H3 = silu(Z3)
    out = H3 @ w4 + b4
    return out, (X, Z1, H1, Z2, H2, Z3, H3)


def loss_grad(p, X, y):
    """Mean squared error and its gradient with respect to the parameter vector."""
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p)
    out, (X, Z1, H1, Z2, H2, Z3, H3) = forward(p, X)
    n = len(out)
    d = out - np.asarray(y, np.float64)
    loss = float(np.mean(d * d))
    dout = 2.0 * d / n
    g = np.zeros(N_PARAMS)
    g[OFF_W4:OFF_B4] = H3.T @ dout
    g[OFF_B4] = dout.sum()
    dZ3 = np.outer(dout, w4) * dsilu(Z3)
    g[OFF_W3:OFF_B3] = (dZ3.T @ H2).ravel()
    g[OFF_B3:OFF_W4] = dZ3.sum(0)
    dZ2 = (dZ3 @ W3) * dsilu(Z2)
    g[OFF_W2:OFF_B2] = (dZ2.T @ H1).ravel()
    g[OFF_B2:OFF_W3] = dZ2.sum(0)
    dZ1 = (dZ2 @ W2) * dsilu(Z1)
    g[OFF_W1:OFF_B1] = (dZ1.T @ X).ravel()
    g[OFF_B1:OFF_W2] = dZ1.sum(0)
    return loss, g
