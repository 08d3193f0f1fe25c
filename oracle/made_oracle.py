"""CPU restatement of the learned proposal's network (test infrastructure only).

An autoregressive masked MLP (MADE: M. Germain, K. Gregor, I. Murray, H. Larochelle, "MADE: Masked
Autoencoder for Distribution Estimation", ICML 2015) over n binary sites: x -> h1 = relu(W1 x + b1)
-> h2 = relu(W2 h1 + b2) -> logits o = W3 h2 + b3, with masks built from degrees so that o_i depends
on x_0..x_{i-1} only; p(x_i = 1 | x_<i) = sigmoid(o_i).  Weights are rounded to bfloat16 for every
product (as the device kernels store them), activations and accumulations are float32.  Training
minimises the mean negative log-likelihood with Adam (D. P. Kingma, J. Ba, ICLR 2015).
"""
import numpy as np


def degrees(n, hidden):
    """Input degrees 1..n and hidden degrees cycling through 1..n-1 (MADE's deterministic choice)."""
    d_in = np.arange(1, n + 1)
    d_h = (np.arange(hidden) % max(1, n - 1)) + 1
    return d_in, d_h


def masks(n, hidden):
    d_in, d_h = degrees(n, hidden)
    m1 = (d_h[:, None] >= d_in[None, :]).astype(np.float32)   # hidden1 x input
    m2 = (d_h[:, None] >= d_h[None, :]).astype(np.float32)    # hidden2 x hidden1
    m3 = (d_in[:, None] > d_h[None, :]).astype(np.float32)    # output x hidden2
    return m1, m2, m3


def bf16(a):
    """Round-to-nearest-even to bfloat16, returned as float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


class MADE:

    def __init__(self, params, n, hidden, bf16_weights=True, dtype=np.float32):
        """bf16_weights=False and dtype=float64 give the smooth function the finite-difference check
        of the gradients needs."""
        self.n, self.hidden = n, hidden
        self.dtype = dtype
        self.round = bf16 if bf16_weights else (lambda a: np.asarray(a, dtype=dtype))
        self.p = {k: np.asarray(v, dtype=dtype).copy() for k, v in params.items()}
        self.m1, self.m2, self.m3 = (m.astype(dtype) for m in masks(n, hidden))

    def forward(self, x):
        x = np.asarray(x, dtype=self.dtype)
        W1 = self.round(self.p["W1"]) * self.m1
        W2 = self.round(self.p["W2"]) * self.m2
        W3 = self.round(self.p["W3"]) * self.m3
        a1 = x @ W1.T + self.p["b1"]
        h1 = np.maximum(a1, 0)
        a2 = h1 @ W2.T + self.p["b2"]
        h2 = np.maximum(a2, 0)
        o = h2 @ W3.T + self.p["b3"]
        return o, (x, a1, h1, a2, h2)

    def logq(self, x):
        o, _ = self.forward(x)
        x = np.asarray(x, dtype=np.float64)
        o = o.astype(np.float64)
        # log sigmoid(o) = -log(1 + e^-o)
        return -(x * np.logaddexp(0, -o) + (1 - x) * np.logaddexp(0, o)).sum(axis=1)

    def loss_and_grads(self, x):
        """Mean negative log-likelihood and its gradients (masked, through the bfloat16 weights)."""
        o, (xx, a1, h1, a2, h2) = self.forward(x)
        B = xx.shape[0]
        loss = -self.logq(x).mean()
        s = 1.0 / (1.0 + np.exp(-o.astype(np.float64)))
        do = ((s - xx) / B).astype(self.dtype)
        W2 = self.round(self.p["W2"]) * self.m2
        W3 = self.round(self.p["W3"]) * self.m3
        g = {"W3": (do.T @ h2) * self.m3, "b3": do.sum(axis=0)}
        dh2 = (do @ W3) * (a2 > 0)
        g["W2"] = (dh2.T @ h1) * self.m2
        g["b2"] = dh2.sum(axis=0)
        dh1 = (dh2 @ W2) * (a1 > 0)
        g["W1"] = (dh1.T @ xx) * self.m1
        g["b1"] = dh1.sum(axis=0)
        return loss, g


def adam_step(p, g, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update of the float32 parameters (bias-corrected moments, step t >= 1)."""
    for k in p:
        m[k] = beta1 * m[k] + (1 - beta1) * g[k]
        v[k] = beta2 * v[k] + (1 - beta2) * g[k] * g[k]
        mh = m[k] / (1 - beta1**t)
        vh = v[k] / (1 - beta2**t)
        p[k] = (p[k] - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32)
