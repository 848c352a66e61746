"""The learned initialiser end to end on NODDI-Watson:
  * synthetic signals (cdm_synth_signals): at very high SNR they equal the
    FP64 oracle's Predicted_Signal within the FP32 model tolerance, and the
    S0 estimate is the true S0;
  * the plugin head: decode(encode(P)) returns P (orientation as an axis);
  * a network trained on the GPU by the library's own kernels beats the
    method without it: LM started from its predictions ends at or below the
    plain grid-search + LM cost (within 1 %) on >= 90 % of voxels, far more
    than LM from CUDIMOT's default start, and its parameter errors are no
    worse than the plain path's;
  * MCMC with network-seeded proposal widths samples the same posterior as
    MCMC started from CUDIMOT's |P|/10 widths (posterior-mean z-scores)."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import capi, synth
from tests.helpers import angle_deg, oracle

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def protocol():
    rng = np.random.default_rng(8219)
    return synth.protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], rng)


def test_synth_signals_match_oracle(built, cuda):
    cfp = protocol()
    lib = capi.Cudimot("NODDI_Watson", capi.model_cfg("NODDI_Watson"))
    rng = np.random.default_rng(1)
    P, S0 = synth.watson_truth(512, rng)
    meas = torch.zeros(512, cfp.shape[0], dtype=torch.float64, device=cuda)
    s0 = torch.zeros(512, 1, dtype=torch.float64, device=cuda)
    x = torch.zeros(512, 288, dtype=torch.bfloat16, device=cuda)
    lib.synth(T(cfp, cuda), T(P, cuda), T(S0[:, None], cuda), snr=(1e7, 1e7), seed=3, meas=meas,
              s0=s0, x=x)
    torch.cuda.synchronize()
    ref = oracle("NODDI_Watson").signal(P, cfp, S0[:, None])
    got = meas.cpu().numpy()
    assert np.all(np.abs(got - ref) <= 2e-5 * np.abs(ref) + 2e-6 * S0[:, None] + 1e-3)
    np.testing.assert_allclose(s0.cpu().numpy()[:, 0], S0, rtol=1e-5)
    xr = (ref / S0[:, None]).astype(np.float32)
    assert np.max(np.abs(x.float().cpu().numpy() - xr)) <= 2 ** -8


def test_head_round_trip(built, cuda):
    lib = capi.Cudimot("NODDI_Watson", capi.model_cfg("NODDI_Watson"))
    rng = np.random.default_rng(2)
    P, _ = synth.watson_truth(1000, rng)
    t = torch.zeros(1000, 8, dtype=torch.float32, device=cuda)
    lib.mlp_targets(T(P, cuda), t)
    out = torch.zeros(1000, 16, dtype=torch.float32, device=cuda)
    out[:, :8] = t
    out[:, 8:12] = -3.0
    Q = torch.zeros(1000, 5, dtype=torch.float64, device=cuda)
    sd = torch.zeros_like(Q)
    lib.mlp_decode(out, Q, sd)
    torch.cuda.synchronize()
    q = Q.cpu().numpy()
    np.testing.assert_allclose(q[:, :2], np.clip(P[:, :2], 1e-3, 1 - 1e-3), atol=1e-6)
    np.testing.assert_allclose(q[:, 2], P[:, 2], rtol=1e-5)
    assert np.max(angle_deg(q[:, 3], q[:, 4], P[:, 3], P[:, 4])) < 0.05
    assert np.all(sd.cpu().numpy() > 0)


@pytest.fixture(scope="module")
def trained(built):
    from cudimot_gb300.learned import LearnedInit
    dev = torch.device("cuda:0")
    li = LearnedInit("NODDI_Watson", protocol(), grid=synth.WATSON_GRID, seed=77, device=dev)
    x, t = li.make_training_set(n_prior=1 << 20, n_lm=1 << 15)
    li.train(x, t, epochs=3, batch=4096)
    return li


def test_trained_network_beats_the_method_without_it(trained, cuda):
    li = trained
    assert li.history[-1][1] < li.history[0][1] - 1.0, li.history
    d = li.synth(4096, seed=999, snr=(20.0, 20.0), meas=True)
    meas, s0, truth = d["meas"], d["s0"], d["params"].cpu().numpy()
    # plain path: grid search + LM from CUDIMOT's default start with the true axis
    init = li._default_init(4096)
    init[:, 3:5] = d["params"][:, 3:5]
    plain = li.plain_fit(meas, s0, init=init)
    c_plain = li.cost(meas, plain, s0)
    # without the network and without grid search: LM from the default start
    cfg = capi.model_cfg("NODDI_Watson")
    lm = capi.Cudimot("NODDI_Watson", cfg)
    p_def = init.clone()
    lm.levmar(meas, p_def, li.cfp, s0)
    c_def = li.cost(meas, p_def, s0)
    # surrogate: network -> LM
    P, sd = li.predict(meas, s0)
    lm.levmar(meas, P, li.cfp, s0)
    c_sur = li.cost(meas, P, s0)
    torch.cuda.synchronize()
    ok_sur = (c_sur <= c_plain * 1.01).float().mean().item()
    ok_def = (c_def <= c_plain * 1.01).float().mean().item()
    assert ok_sur >= 0.90, (ok_sur, ok_def)
    assert ok_sur > ok_def + 0.05, (ok_sur, ok_def)
    p, q = P.cpu().numpy(), plain.cpu().numpy()
    for k in (0, 1):
        e_sur = np.sqrt(np.mean((p[:, k] - truth[:, k]) ** 2))
        e_plain = np.sqrt(np.mean((q[:, k] - truth[:, k]) ** 2))
        assert e_sur <= e_plain * 1.05, (k, e_sur, e_plain)


def test_seeded_mcmc_samples_the_same_posterior(trained, cuda):
    li = trained
    d = li.synth(256, seed=4242, snr=(20.0, 20.0), meas=True)
    meas, s0 = d["meas"], d["s0"]
    P, sd = li.predict(meas, s0)
    cfg = capi.model_cfg("NODDI_Watson", run_mcmc=1, nburn=500, njumps=2000, sampleevery=10)
    lib = capi.Cudimot("NODDI_Watson", cfg)
    lib.levmar(meas, P, li.cfp, s0)
    a = torch.zeros(256, 5, 200, dtype=torch.float64, device=cuda)
    b = torch.zeros_like(a)
    lib.mcmc_seeded(meas, P.clone(), li.cfp, s0, a, sd)
    cfg2 = capi.model_cfg("NODDI_Watson", run_mcmc=1, nburn=500, njumps=2000, sampleevery=10,
                          seed=4321)
    capi.Cudimot("NODDI_Watson", cfg2).mcmc(meas, P.clone(), li.cfp, s0, b)
    torch.cuda.synchronize()
    g, r = a.cpu().numpy(), b.cpu().numpy()
    for p in (0, 1, 2):
        def se(x):
            bm = x.reshape(x.shape[0], 10, -1).mean(2)
            return bm.std(1, ddof=1) / np.sqrt(10)
        z = (g[:, p].mean(1) - r[:, p].mean(1)) / np.sqrt(se(g[:, p]) ** 2 + se(r[:, p]) ** 2 + 1e-30)
        assert abs(np.median(z)) < 0.5, (p, np.median(z))
        assert np.mean(np.abs(z) < 4) > 0.9, (p, np.mean(np.abs(z) < 4))


def test_cost_select_and_rows(built, cuda):
    cfp = protocol()
    o = oracle("NODDI_Watson")
    rng = np.random.default_rng(5)
    P, S0 = synth.watson_truth(2000, rng)
    meas = synth.rician(o.signal(P, cfp, S0[:, None]), S0[:, None] / 20.0, rng)
    lib = capi.Cudimot("NODDI_Watson", capi.model_cfg("NODDI_Watson"))
    c = torch.zeros(2000, dtype=torch.float64, device=cuda)
    lib.cost(T(meas, cuda), T(P, cuda), T(cfp, cuda), T(S0[:, None], cuda), c)
    torch.cuda.synchronize()
    ref = o.cost(meas, P, cfp, S0[:, None])
    np.testing.assert_allclose(c.cpu().numpy(), ref, rtol=1e-5)
    refc = torch.full_like(c, float(np.median(ref)))
    idx = torch.zeros(2000, dtype=torch.int32, device=cuda)
    cnt = torch.zeros(1, dtype=torch.int32, device=cuda)
    lib.select_worse(c, refc, 0.01, idx, cnt)
    k = int(cnt.item())
    sel = np.sort(idx[:k].cpu().numpy())
    assert np.array_equal(sel, np.nonzero(c.cpu().numpy() > np.median(ref) * 1.01)[0])
    src = T(P, cuda)
    sub = torch.zeros(k, 5, dtype=torch.float64, device=cuda)
    lib.rows(k, idx, src, sub, 0)
    dst = torch.zeros_like(src)
    lib.rows(k, idx, sub, dst, 1)
    lib.rows(k, idx, None, src, 2, -1.0)
    torch.cuda.synchronize()
    ii = idx[:k].long()
    assert torch.equal(sub, T(P, cuda)[ii])
    assert torch.equal(dst[ii], T(P, cuda)[ii])
    assert torch.all(src[ii] == -1.0)
