"""The MLP oracle (oracle/mlp_oracle.py) pinned on its own: exact float64
gradients against central finite differences of the loss, and the bf16
rounding helper against known bit patterns. The library's export list is
checked without a GPU."""
import ctypes as C
import os
import re

import numpy as np

from oracle.mlp_oracle import MlpOracle, bf16, init_params

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "cdm_mlp.h")


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3, 65504.0], dtype=np.float32)
    y = bf16(x)
    # 1 + 2^-8 is a tie -> even (1.0); 1 + 1.5 * 2^-8 rounds up to 1 + 2^-7
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == np.float32(1.0078125)
    assert y[3] == -2.5
    assert (y.view(np.uint32) & 0xFFFF == 0).all()
    assert abs(y[4] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(4)
    n_in, H, n_mu, n_sig = 24, 16, 5, 3
    group = [0, 1, 2, 2, 2]
    W, b = init_params(n_in, H, n_mu + n_sig, seed=2)
    W = [w.astype(np.float64) for w in W]
    W[3] *= 10.0
    b = [rng.standard_normal(x.shape) * 0.1 for x in b]
    o = MlpOracle(W, b, n_mu, n_sig, group, bf16_rounding=False)
    x = rng.standard_normal((7, n_in))
    t = rng.standard_normal((7, n_mu))
    loss, dW, db = o.gradients(x, t)
    eps = 1e-6
    for l in range(4):
        for _ in range(6):
            i, j = rng.integers(W[l].shape[0]), rng.integers(W[l].shape[1])
            W[l][i, j] += eps
            lp, _ = o.loss_and_grad_out(o.forward(x)[0], t)
            W[l][i, j] -= 2 * eps
            lm, _ = o.loss_and_grad_out(o.forward(x)[0], t)
            W[l][i, j] += eps
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - dW[l][i, j]) <= 1e-6 * max(1.0, abs(fd)), (l, i, j, fd, dW[l][i, j])
        k = rng.integers(b[l].shape[0])
        b[l][k] += eps
        lp, _ = o.loss_and_grad_out(o.forward(x)[0], t)
        b[l][k] -= 2 * eps
        lm, _ = o.loss_and_grad_out(o.forward(x)[0], t)
        b[l][k] += eps
        assert abs((lp - lm) / (2 * eps) - db[l][k]) <= 1e-6 * max(1.0, abs(db[l][k]))


def test_mlp_library_exports(built):
    from cudimot_gb300 import capi
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    names = sorted(set(re.findall(r"\b(cdm_mlp_[a-z_0-9]+)\s*\(", text)))
    lib = C.CDLL(os.path.join(capi.LIBDIR, "libcdm_mlp.so"))
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
