"""CPU oracle of the learned initialiser's network (test infrastructure).

Restates, in numpy, what libcdm_mlp computes on the tensor cores:
forward n_in -> H -> H -> H -> n_out with GELU (tanh form), the Gaussian
negative log-likelihood head and the backward pass, with the library's
rounding points when `bf16=True`:
  * GEMM operands (inputs, weights, activations, output gradients) are
    bf16, products accumulate in FP32;
  * z = bf16(acc + b); a = bf16(gelu(z));
  * d(loss)/d(out) = bf16(...); dz = bf16(dact * gelu'(z)).
With `bf16=False` and float64 arrays it is the exact network, which the
tests check against finite differences (pinning the oracle itself).
"""
import numpy as np


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(x.shape)


_C0 = np.sqrt(2.0 / np.pi)
_C1 = _C0 * 0.044715


def gelu(z):
    """GELU in its tanh form, as the library defines the network."""
    return 0.5 * z * (1.0 + np.tanh(z * (_C0 + _C1 * z * z)))


def gelu_grad(z):
    t = np.tanh(z * (_C0 + _C1 * z * z))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * (_C0 + 3.0 * _C1 * z * z)


class MlpOracle:
    def __init__(self, weights, biases, n_mu, n_sig, group, logstd_min=-7.0, logstd_max=3.0,
                 bf16_rounding=True):
        self.W = [np.asarray(w) for w in weights]
        self.b = [np.asarray(b) for b in biases]
        self.n_mu, self.n_sig = n_mu, n_sig
        self.group = np.asarray(group[:n_mu])
        self.smin, self.smax = logstd_min, logstd_max
        self.round = bf16_rounding

    def _r(self, x):
        return bf16(x) if self.round else x

    def forward(self, x):
        dt = np.float32 if self.round else np.float64
        a = self._r(np.asarray(x, dtype=dt))
        zs, acts = [], [a]
        for l in range(3):
            z = self._r(a @ self._r(self.W[l].astype(dt)).T + self.b[l].astype(dt))
            a = self._r(gelu(z).astype(dt))
            zs.append(z)
            acts.append(a)
        out = a @ self._r(self.W[3].astype(dt)).T + self.b[3].astype(dt)
        return out, zs, acts

    def loss_and_grad_out(self, out, t):
        n_mu, B = self.n_mu, out.shape[0]
        mu = out[:, :n_mu]
        s_raw = out[:, n_mu:n_mu + self.n_sig]
        s = np.clip(s_raw, self.smin, self.smax)
        sg = s[:, self.group]
        w = np.exp(-2.0 * sg)
        r = mu - t
        loss = np.sum(0.5 * r * r * w + sg) / B
        g = np.zeros_like(out)
        g[:, :n_mu] = r * w / B
        ds = np.zeros_like(s)
        for j in range(n_mu):
            ds[:, self.group[j]] += 1.0 - r[:, j] ** 2 * w[:, j]
        inside = (s_raw > self.smin) & (s_raw < self.smax)
        g[:, n_mu:n_mu + self.n_sig] = np.where(inside, ds / B, 0.0)
        return loss, g

    def gradients(self, x, t):
        """-> loss, [dW0..dW3], [db0..db3]"""
        dt = np.float32 if self.round else np.float64
        out, zs, acts = self.forward(x)
        loss, g = self.loss_and_grad_out(out, np.asarray(t, dtype=dt))
        g = self._r(g)
        dW, db = [None] * 4, [None] * 4
        for l in range(3, -1, -1):
            dW[l] = g.T @ acts[l]
            db[l] = g.sum(axis=0)
            if l > 0:
                da = g @ self._r(self.W[l].astype(dt))
                g = self._r(da * gelu_grad(zs[l - 1]))
        return loss, dW, db


def init_params(n_in, hidden, n_out, seed=0):
    """He-style initial weights (fp32), zero biases; small output layer."""
    rng = np.random.default_rng(seed)
    dims = [n_in, hidden, hidden, hidden, n_out]
    W, b = [], []
    for l in range(4):
        scale = np.sqrt(2.0 / dims[l]) * (0.1 if l == 3 else 1.0)
        W.append((rng.standard_normal((dims[l + 1], dims[l])) * scale).astype(np.float32))
        b.append(np.zeros(dims[l + 1], dtype=np.float32))
    return W, b
