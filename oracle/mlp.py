"""Float64 numpy restatement of the predictor MLP (test infrastructure).

Same parameter layout and loss as the device kernels: features normalised
by (x - mu) / max(sd, 1e-6); 12 -> 64 -> 64 -> K with ReLU; softmax; loss =
mean over samples of w * sum_k -t_k log p_k.  Used to check the device
forward pass and the hand-written backward pass.
"""
import numpy as np

F, H = 12, 64


def unpack(p, K):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    mu = p[o:o + F]; o += F
    sd = p[o:o + F]; o += F
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + K * H].reshape(K, H); o += K * H
    b3 = p[o:o + K]; o += K
    assert o == len(p)
    return mu, sd, W1, b1, W2, b2, W3, b3


def forward(p, X, K):
    mu, sd, W1, b1, W2, b2, W3, b3 = unpack(p, K)
    x = (np.asarray(X, np.float64) - mu) / np.maximum(sd, 1e-6)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    z = h2 @ W3.T + b3
    z = z - z.max(axis=1, keepdims=True)
    e = np.exp(z)
    return e / e.sum(axis=1, keepdims=True), (x, h1, h2)


def loss_and_grad(p, X, T, W, K):
    n = len(X)
    w = np.ones(n) if W is None else np.asarray(W, np.float64)
    probs, (x, h1, h2) = forward(p, X, K)
    T = np.asarray(T, np.float64)
    loss = float((w[:, None] * -T * np.log(np.maximum(probs, 1e-30)) * (T > 0)).sum() / n)
    mu, sd, W1, b1, W2, b2, W3, b3 = unpack(p, K)
    dz = (probs - T) * w[:, None]
    gW3 = dz.T @ h2
    gb3 = dz.sum(0)
    g2 = (dz @ W3) * (h2 > 0)
    gW2 = g2.T @ h1
    gb2 = g2.sum(0)
    g1 = (g2 @ W2) * (h1 > 0)
    gW1 = g1.T @ x
    gb1 = g1.sum(0)
    grad = np.concatenate([np.zeros(2 * F), gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3]) / n
    return loss, grad
