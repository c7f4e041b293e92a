"""Solute-channel features and the fused jump kernel of the barrier surrogate:

* lattice-jump features in the solute encoding (both writers) against the
  encoding built on the host from the reference-pinned MMM site order;
* the training data in the solute encoding against the one-hot data of the
  same seed (same environments, same labels);
* the fused kernel (features gathered inside, weights in shared memory, tcgen05)
  against the unfused path (feature rows, then the mma.sync GEMMs) and the
  float64 network, over several tiles per CTA, with the rows it hands to the
  plain predictor (a second vacancy in the environment) and a rejected pair."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EL = ("Al", "Mg", "Zn")
EL4 = ("Al", "Cu", "Mg", "Zn")


def _pair_sites(N, n, a, b):
    st, mmm, mm2 = np.zeros(60, np.int64), np.zeros(58, np.int64), np.zeros(58, np.int64)
    N.check(N.lib.lmc_geom_pair_lists(n, int(a), int(b), st.ctypes.data_as(C.POINTER(C.c_int64)),
                                      mmm.ctypes.data_as(C.POINTER(C.c_int64)),
                                      mm2.ctypes.data_as(C.POINTER(C.c_int64))))
    return list(mmm) + [int(b)]


def _jumps_of(N, n, sites):
    pairs = []
    for v in sites:
        nb = np.zeros(42, np.int64)
        N.check(N.lib.lmc_geom_neighbors(n, int(v), nb.ctypes.data_as(C.POINTER(C.c_int64))))
        pairs += [(int(v), int(j)) for j in nb[:12]]
    return np.array(pairs, np.int64)


def _solute_row(sp, sites, alpha, el, pad):
    """Solute channels of one jump: per site one channel per element other than the base (Al),
    in element order; Al and X sites all zero."""
    ch = {alpha.index(e): i for i, e in enumerate(el[1:])}
    w = len(el) - 1
    row = np.zeros(pad, np.uint16)
    for k, s in enumerate(sites):
        c = int(sp[s])
        if c in ch:
            row[w * k + ch[c]] = 0x3F80  # bf16 1.0
    return row


@pytest.mark.parametrize("el,pad", [(EL, 128), (EL, 122), (EL4, 192), (EL4, 180)])
def test_solute_features_match_host_lists(native, el, pad):
    torch = pytest.importorskip("torch")
    from latticemontecarlo_gb300 import api, synthetic as S
    N = native
    n = 9
    sp = S.make_lattice(n, {e: 1.0 / len(el) for e in el}, 5, 8, el)
    ctx = api.Context(api.Model.from_coefficients(S.make_coefficients(el, 3), list(el)))
    ctx.set_lattices([n], sp)
    ctx.set_surrogate_encoding(N.LMC_FEATURES_SOLUTE)
    assert api.surrogate_feature_count(ctx) == (128 if len(el) == 3 else 192)
    alpha = S.alphabet(el)
    rng = np.random.default_rng(2)
    pairs = _jumps_of(N, n, rng.integers(0, sp.size, 25))
    got = api.surrogate_features(ctx, torch.from_numpy(pairs).cuda(), pad)
    got = got.contiguous().view(torch.int16).cpu().numpy().view(np.uint16)
    for i, (a, b) in enumerate(pairs):
        assert np.array_equal(got[i], _solute_row(sp, _pair_sites(N, n, a, b), alpha, el, pad)), i


def test_solute_dataset_is_the_onehot_dataset(native):
    """Same seed, same environments and labels; the solute rows are the one-hot rows without
    the base (Al) channel."""
    pytest.importorskip("torch")
    from latticemontecarlo_gb300 import api, synthetic as S
    N = native
    n = 10
    ctx = api.Context(api.Model.from_coefficients(S.make_coefficients(EL, 7), list(EL)))
    ctx.set_lattices([n], S.make_lattice(n, {"Al": 0.96, "Mg": 0.02, "Zn": 0.02}, 1, 3, EL))
    x1, ea1, e64_1, _ = api.surrogate_dataset(ctx, 17, 4096, 0.0, 0.5, 192)
    ctx.set_surrogate_encoding(N.LMC_FEATURES_SOLUTE)
    x2, ea2, e64_2, _ = api.surrogate_dataset(ctx, 17, 4096, 0.0, 0.5, 128)
    ctx.set_surrogate_encoding(N.LMC_FEATURES_ONEHOT)
    assert np.array_equal(e64_1.cpu().numpy(), e64_2.cpu().numpy())
    oh = x1.float().cpu().numpy()[:, :177].reshape(-1, 59, 3)   # ranks Al, Mg, Zn
    so = x2.float().cpu().numpy()
    assert np.array_equal(so[:, :118].reshape(-1, 59, 2), oh[:, :, 1:])
    assert not so[:, 118:].any()


@pytest.fixture(scope="module", params=[EL, EL4], ids=["ternary", "quaternary"])
def trained(native, request):
    """A compact ensemble (2 members, in -> 128 -> 128, in = 128 / 192 for three / four
    species) trained briefly on solute features."""
    torch = pytest.importorskip("torch")
    from latticemontecarlo_gb300 import api, synthetic as S
    N = native
    el = request.param
    n = 12
    el_frac = {e: (0.7 if e == "Al" else 0.3 / (len(el) - 1)) for e in el}
    sp = S.make_lattice(n, el_frac, 9, 0, el)
    alpha = S.alphabet(el)
    x_code = alpha.index("X")
    rng = np.random.default_rng(4)
    vac = rng.choice(sp.size, 40, replace=False)
    sp[vac] = x_code
    ctx = api.Context(api.Model.from_coefficients(S.make_coefficients(el, 1234), list(el)))
    ctx.set_lattices([n], sp)
    ctx.set_surrogate_encoding(N.LMC_FEATURES_SOLUTE)
    nin = api.surrogate_feature_count(ctx)
    x, ea, _, _ = api.surrogate_dataset(ctx, 1, 1 << 17, 0.1, 0.4, nin)
    net = api.Surrogate(nin, 128, 2, seed=3)
    net.set_label_scale(float(ea.mean()), float(ea.std()))
    net.train(x, ea, batch=4096, epochs=3, lr=2e-3, seed=4)
    return torch, api, N, ctx, net, sp, n, vac, alpha


def test_fused_kernel_matches_unfused_and_float64(trained):
    torch, api, N, ctx, net, sp, n, vac, alpha = trained
    from oracle import mlp as R
    pairs = _jumps_of(N, n, vac)                      # 480 jumps, several with a second vacancy nearby
    x_code = alpha.index("X")
    has_x = np.array([any(int(sp[s]) == x_code for s in _pair_sites(N, n, a, b)) for a, b in pairs])
    assert has_x.any() and not has_x.all()
    reps = 100                                        # 48 000 rows: several tiles per CTA, a partial last tile
    pd = torch.from_numpy(np.tile(pairs, (reps, 1))).cuda()
    net.set_inference_path(0)
    m_f, s_f = api.surrogate_predict(ctx, net, pd)
    net.set_inference_path(2)
    m_r, s_r = api.surrogate_predict(ctx, net, pd)
    net.set_inference_path(0)
    m_f, s_f, m_r, s_r = (t.double().cpu().numpy() for t in (m_f, s_f, m_r, s_r))
    flag = np.tile(has_x, reps)
    assert np.all(np.isinf(s_f[flag])) and np.all(np.isfinite(s_f[~flag]))
    assert np.all(np.isfinite(m_f))
    np.testing.assert_allclose(m_f[~flag], m_r[~flag], rtol=0, atol=2e-3)
    np.testing.assert_allclose(s_f[~flag], s_r[~flag], rtol=0, atol=3e-3)
    # every repetition of a jump gives the same bits
    assert np.array_equal(m_f.reshape(reps, -1), np.broadcast_to(m_f[:len(pairs)], (reps, len(pairs))))
    # the float64 network on the same feature rows
    nin = net.in_features
    xs = api.surrogate_features(ctx, pd[:len(pairs)], nin)
    bits = xs.contiguous().view(torch.int16).cpu().numpy().view(np.uint16)
    y = R.predict(net.params(), R.bf16_bits_to_float(bits), nin, 128, 2)
    mu, sd = (float(np.float32(v)) for v in net.label_scale)
    ok = ~has_x
    np.testing.assert_allclose(m_f[:len(pairs)][ok], (mu + sd * y.mean(0))[ok], rtol=0, atol=3e-3)


def test_fused_kernel_rejects_non_jumps(trained):
    torch, api, N, ctx, net, sp, n, vac, alpha = trained
    bad = torch.tensor([[0, 5]], dtype=torch.int64, device="cuda")
    with pytest.raises(N.LmcError):
        api.surrogate_predict(ctx, net, bad)
    # the context stays usable
    pd = torch.from_numpy(_jumps_of(N, n, vac[:2])).cuda()
    m, s = api.surrogate_predict(ctx, net, pd)
    assert torch.isfinite(m).all()


def _vacancy_grid(S, n, spacing, frac, seed, el):
    """Vacancies on every site whose half-lattice coordinates are multiples of `spacing` (no jump
    environment holds a second vacancy), the rest i.i.d. from `frac`; with each vacancy's 12 jumps."""
    alpha = S.alphabet(el)
    rng = np.random.default_rng(seed)
    names = list(frac)
    p = np.array([frac[k] for k in names], float)
    sp = np.array([alpha.index(k) for k in names], np.int8)[rng.choice(len(names), size=4 * n ** 3, p=p / p.sum())]
    m = 2 * n
    g = np.arange(0, m, spacing)
    hx, hy, hz = (a.ravel() for a in np.meshgrid(g, g, g, indexing="ij"))
    vac = hx * 2 * n * n + hy * n + hz // 2
    sp[vac] = alpha.index("X")
    dirs = [(a, b, 0) for a in (-1, 1) for b in (-1, 1)] + [(a, 0, b) for a in (-1, 1) for b in (-1, 1)] + \
        [(0, a, b) for a in (-1, 1) for b in (-1, 1)]
    pairs = [np.stack([vac, ((hx + d[0]) % m) * 2 * n * n + ((hy + d[1]) % m) * n + ((hz + d[2]) % m) // 2], 1)
             for d in dirs]
    return sp, np.stack(pairs, 1).reshape(-1, 2).astype(np.int64)


def test_trained_network_gain(native):
    """What the trained network gains over the method without it. On a solute-rich lattice (Al .70,
    Mg .15, Zn .15: the plain predictor's sparse lists overflow and every jump takes the dense
    cluster sums) the compact ensemble, trained on 2e6 plain barriers of random environments with
    20-40 % solutes, gives the barriers of the lattice's jumps (fallback to the plain predictor where
    its two members differ by more than 10 meV) at least twice as fast as the best plain evaluation,
    within 5 meV mean absolute error of the plain FP64 barriers."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    import time
    from latticemontecarlo_gb300 import api, synthetic as S
    N = native
    ctx = api.Context(api.Model.from_coefficients(S.make_coefficients(EL, 1234), list(EL)))
    n = 128
    sp, pairs = _vacancy_grid(S, n, 8, {"Al": 0.70, "Mg": 0.15, "Zn": 0.15}, 77, EL)
    ctx.set_lattices([n], sp)
    ctx.set_surrogate_encoding(N.LMC_FEATURES_SOLUTE)
    x, ea, _, _ = api.surrogate_dataset(ctx, 1, 2_000_000, 0.2, 0.4, 128)
    net = api.Surrogate(128, 128, 2, seed=1)
    net.set_label_scale(float(ea.mean()), float(ea.std()))
    net.train(x, ea, batch=2048, epochs=80, lr=3e-3, seed=2)
    del x, ea
    pd = torch.from_numpy(pairs).cuda()
    m = pd.shape[0]
    ea_p = torch.empty(m, dtype=torch.float64, device="cuda")
    de_p = torch.empty_like(ea_p)

    def plain():
        N.check(N.lib.lmc_barrier_batch_device(ctx._h, 0, 0, C.c_void_p(pd.data_ptr()), m,
                                               C.c_void_p(ea_p.data_ptr()), C.c_void_p(de_p.data_ptr())))
        N.check(N.lib.lmc_ctx_synchronize(ctx._h))

    out = {}

    def surrogate():
        out["s"] = api.surrogate_barriers(ctx, net, pd, 0.010)

    def median_time(fn):
        for _ in range(3):
            fn()
        ts = []
        for _ in range(9):
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t)
        return float(np.median(ts))

    t_plain = []
    for ev in (N.LMC_EVAL_SPARSE, N.LMC_EVAL_DENSE):
        ctx.set_barrier_evaluation(ev)
        t_plain.append(median_time(plain))
    t_sur = median_time(surrogate)
    ea_s, _, nfb = out["s"]
    mae = float((ea_s - ea_p).abs().mean())
    gain = min(t_plain) / t_sur
    info = dict(gain=gain, mae_mev=1e3 * mae, fallback=nfb / m, plain_per_s=m / min(t_plain), surrogate_per_s=m / t_sur)
    assert mae <= 0.005, info
    assert gain >= 2.0, info
