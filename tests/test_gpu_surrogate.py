"""BF16 MLP barrier surrogate:

* gradients of the GPU's tensor-core forward/backward kernels against the
  float64 reference MLP (oracle/mlp.py) on the same (bf16) weights and inputs;
* the training data generator's labels against the oracle's Quartic barrier of
  the same environment (rebuilt on a lattice from the features);
* a trained ensemble on a held-out seed: MAE of the ensemble mean against the
  plain predictor (the FP64-pinned barrier), and the surrogate-with-fallback
  error, which the fallback bounds by the spread threshold."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(native):
    torch = pytest.importorskip("torch")
    from latticemontecarlo_gb300 import api, synthetic as S
    el = ("Al", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 7)
    model = api.Model.from_coefficients(coeffs, list(el))
    ctx = api.Context(model)
    n = 10
    ctx.set_lattices([n], S.make_lattice(n, {"Al": 0.96, "Mg": 0.02, "Zn": 0.02}, 1, 3, el))
    return torch, api, ctx, el, coeffs, api.surrogate_feature_count(ctx)


def _bits(x_bf16):
    import torch
    return x_bf16.contiguous().view(torch.int16).cpu().numpy().view(np.uint16)


@pytest.mark.parametrize("train_path", [0, 1])
def test_gradients_against_float64(setup, train_path):
    """Both training-GEMM paths (0: tcgen05 with TMEM accumulators, 1: mma.sync) against float64."""
    torch, api, ctx, el, coeffs, nin = setup
    from oracle import mlp as R
    hidden, members, batch = 128, 2, 128
    net = api.Surrogate(nin, hidden, members, seed=5)
    net.set_train_path(train_path)
    x, ea, _, _ = api.surrogate_dataset(ctx, 11, batch, 0.0, 0.3, nin)
    ea_h = ea.cpu().numpy()
    net.set_label_scale(float(ea_h.mean()), float(ea_h.std()))
    bits = _bits(x)
    g, loss = net.gradients(bits, ea_h)
    p = net.params()
    t = (ea_h.astype(np.float64) - np.float32(ea_h.mean())) / np.float32(ea_h.std())
    ref_loss, ref = R.forward_backward(p, R.bf16_bits_to_float(bits), t, nin, hidden, members)
    np.testing.assert_allclose(loss, ref_loss, rtol=2e-2)
    W1, b1, W2, b2, w3, b3 = (np.arange(p.size),) * 6
    sizes = [members * hidden * nin, members * hidden, members * hidden * hidden, members * hidden,
             members * hidden, members]
    off = 0
    for name, sz in zip(["W1", "b1", "W2", "b2", "w3", "b3"], sizes):
        a, b = g[off:off + sz].astype(np.float64), ref[off:off + sz]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert rel < 3e-2 and cos > 0.999, (name, rel, cos)
        off += sz


def test_tcgen05_training_gemms_match_mma_sync(setup):
    """The tcgen05 training GEMMs and the mma.sync ones give the same gradients to the rounding of
    their FP32 sums (the BF16 activations they store may differ by one BF16 step), on the
    workload's own shapes (hidden 256, 4 members, a batch of 512), and one training epoch from
    the same start reaches the same loss."""
    torch, api, ctx, el, coeffs, nin = setup
    hidden, members, batch = 256, 4, 512
    x, ea, _, _ = api.surrogate_dataset(ctx, 13, batch, 0.0, 0.3, nin)
    ea_h = ea.cpu().numpy()
    bits = _bits(x)
    grads, losses = [], []
    for path in (0, 1):
        net = api.Surrogate(nin, hidden, members, seed=9)
        net.set_label_scale(float(ea_h.mean()), float(ea_h.std()))
        net.set_train_path(path)
        g, _ = net.gradients(bits, ea_h)
        grads.append(g.astype(np.float64))
        xt, et, _, _ = api.surrogate_dataset(ctx, 21, 8192, 0.0, 0.3, nin)
        losses.append(net.train(xt, et, batch=1024, epochs=1, lr=2e-3, seed=4))
    a, b = grads
    rel = np.linalg.norm(a - b) / np.linalg.norm(b)
    cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
    assert rel < 1e-2 and cos > 0.9999, (rel, cos)
    np.testing.assert_allclose(losses[0], losses[1], rtol=2e-2)


def test_dataset_labels_match_oracle(setup, oracle_mod):
    torch, api, ctx, el, coeffs, nin = setup
    from latticemontecarlo_gb300 import _native as N, synthetic as S
    x, ea, ea64, de64 = api.surrogate_dataset(ctx, 21, 64, 0.0, 0.4, nin, with_de=True)
    feats = x.float().cpu().numpy()
    n = 10
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    alpha = S.alphabet(el)
    ranks = [c for c in range(len(alpha)) if alpha[c] != "X"]  # one-hot rank -> code
    base, x_code = alpha.index("Al"), alpha.index("X")
    vac = 123
    j = int(lat.neighbors(vac)[0])
    st, mmm, mm2 = (np.zeros(60, np.int64), np.zeros(58, np.int64), np.zeros(58, np.int64))
    N.check(N.lib.lmc_geom_pair_lists(n, vac, j, st.ctypes.data_as(C.POINTER(C.c_int64)),
                                      mmm.ctypes.data_as(C.POINTER(C.c_int64)),
                                      mm2.ctypes.data_as(C.POINTER(C.c_int64))))
    eh = len(ranks)
    for i in range(64):
        sp = np.full(4 * n ** 3, base, np.int8)
        f = feats[i]
        for k in range(58):
            sp[mmm[k]] = ranks[int(np.argmax(f[k * eh:(k + 1) * eh]))]
        sp[j] = ranks[int(np.argmax(f[58 * eh:59 * eh]))]
        sp[vac] = x_code
        q = oracle_mod.quartic(m, lat, sp, vac, j)
        np.testing.assert_allclose(float(ea64[i]), q[0], rtol=1e-9)
        np.testing.assert_allclose(float(de64[i]), q[1], rtol=0, atol=1e-12)


def test_trained_ensemble(setup):
    torch, api, ctx, el, coeffs, nin = setup
    x, ea, ea64, _ = api.surrogate_dataset(ctx, 1, 1 << 20, 0.0, 0.3, nin)
    net = api.Surrogate(nin, 256, 4, seed=1)
    net.set_label_scale(float(ea.mean()), float(ea.std()))
    loss = net.train(x, ea, batch=4096, epochs=6, lr=2e-3, seed=2)
    assert np.all(np.isfinite(loss))
    xt, eat, ea64t, _ = api.surrogate_dataset(ctx, 99, 1 << 16, 0.0, 0.3, nin)  # held-out seed
    mean, spread = net.predict(xt)
    err = (mean.double() - ea64t).abs()
    mae = float(err.mean())
    label_std = float(ea64t.std())
    assert mae < 0.25 * label_std, (mae, label_std)
    # fallback: the plain barrier wherever the ensemble disagrees by more than 10 meV
    fb = spread > 0.010
    merged = torch.where(fb, ea64t, mean.double())
    assert float((merged - ea64t).abs().mean()) <= mae


def test_tcgen05_inference(setup):
    """The fused tcgen05 kernel against the mma.sync path and the float64 network,
    on 1000 rows (a partial last tile of 128)."""
    torch, api, ctx, el, coeffs, nin = setup
    from oracle import mlp as R
    net = api.Surrogate(nin, 256, 4, seed=3)
    x, ea, _, _ = api.surrogate_dataset(ctx, 31, 1 << 16, 0.0, 0.3, nin)
    net.set_label_scale(float(ea.mean()), float(ea.std()))
    net.train(x, ea, batch=4096, epochs=2, lr=2e-3, seed=4)
    xs = x[:1000].contiguous()
    net.set_inference_path(1)
    m_tc, s_tc = net.predict(xs)
    net.set_inference_path(2)
    m_ref, s_ref = net.predict(xs)
    net.set_inference_path(0)
    m_tc, s_tc, m_ref, s_ref = (t.double().cpu().numpy() for t in (m_tc, s_tc, m_ref, s_ref))
    assert np.all(np.isfinite(m_tc))
    np.testing.assert_allclose(m_tc, m_ref, rtol=0, atol=2e-3)
    np.testing.assert_allclose(s_tc, s_ref, rtol=0, atol=3e-3)
    y = R.predict(net.params(), R.bf16_bits_to_float(_bits(xs)), nin, 256, 4)
    mu, sd = float(np.float32(float(ea.mean()))), float(np.float32(float(ea.std())))
    np.testing.assert_allclose(m_tc, mu + sd * y.mean(0), rtol=0, atol=3e-3)


@pytest.mark.parametrize("elements,pad", [(("Al", "Mg", "Zn"), 192), (("Al", "Mg", "Zn"), 180),
                                          (("Al", "Cu", "Mg", "Zn"), 256), (("Al", "Cu", "Mg", "Zn"), 244)])
def test_lattice_features_match_host_lists(native, elements, pad):
    """Features of lattice jumps (both the thread-per-pair writer, rows of a
    multiple of 8, and the warp writer) against the one-hot encoding built on the
    host from the reference-pinned MMM site order."""
    torch = pytest.importorskip("torch")
    from latticemontecarlo_gb300 import api, synthetic as S
    N = native
    coeffs = S.make_coefficients(elements, 3)
    n = 9
    fr = {e: 1.0 / len(elements) for e in elements}
    sp = S.make_lattice(n, fr, 5, 8, elements)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(elements)))
    ctx.set_lattices([n], sp)
    rng = np.random.default_rng(1)
    alpha = S.alphabet(elements)
    rank = {c: (i if i < alpha.index("X") else i - 1) for i, c in enumerate(range(len(alpha))) if alpha[c] != "X"}
    eh = len(elements)
    m = 300
    a = rng.integers(0, sp.size, m)
    pairs = np.zeros((m, 2), np.int64)
    for i in range(m):
        nb = np.zeros(42, np.int64)
        N.check(N.lib.lmc_geom_neighbors(n, int(a[i]), nb.ctypes.data_as(C.POINTER(C.c_int64))))
        pairs[i] = (a[i], nb[rng.integers(0, 12)])
    pd = torch.from_numpy(pairs).cuda()
    out = torch.full((m, pad), 7, dtype=torch.int16, device="cuda")
    N.check(N.lib.lmc_surrogate_features(ctx._h, 0, C.c_void_p(pd.data_ptr()), m, pad, C.c_void_p(out.data_ptr())))
    got = out.cpu().numpy().view(np.uint16)
    for i in range(m):
        st, mmm, mm2 = np.zeros(60, np.int64), np.zeros(58, np.int64), np.zeros(58, np.int64)
        N.check(N.lib.lmc_geom_pair_lists(n, int(pairs[i, 0]), int(pairs[i, 1]),
                                          st.ctypes.data_as(C.POINTER(C.c_int64)),
                                          mmm.ctypes.data_as(C.POINTER(C.c_int64)),
                                          mm2.ctypes.data_as(C.POINTER(C.c_int64))))
        want = np.zeros(pad, np.uint16)
        for k, site in enumerate(list(mmm) + [pairs[i, 1]]):
            c = int(sp[site])
            if alpha[c] != "X":
                want[k * eh + rank[c]] = 0x3F80  # bf16 1.0
        assert np.array_equal(got[i], want), i
    bad = torch.tensor([[0, 5]], dtype=torch.int64, device="cuda")  # not a 1NN pair
    with pytest.raises(N.LmcError):
        N.check(N.lib.lmc_surrogate_features(ctx._h, 0, C.c_void_p(bad.data_ptr()), 1, pad,
                                             C.c_void_p(out.data_ptr())))
