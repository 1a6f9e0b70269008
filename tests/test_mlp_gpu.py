"""The learned troubled-cell indicator: tensor-core forward (tcgen05) and
backward (mma.sync) kernels against the FP64 oracle, training, the feature
kernel, and the indicator + filter against the plain modal-decay test.

Tolerances: the kernels take BF16 inputs and weights and round the hidden
activations to BF16 between layers, with FP32 accumulation; the oracle runs
in FP64 on the same BF16-rounded inputs and weights.  Probabilities agree to
2e-2, the loss to 2e-2 relative and the gradient vector to 6e-2 relative
(2-norm).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def rounded_params(p):
    """The oracle sees the weights the kernels see: W1, W2 in BF16, biases and W3 in FP32."""
    q = np.asarray(p, dtype=np.float64).copy()
    q[:2048] = bf16(p[:2048])
    q[2112:2112 + 4096] = bf16(p[2112:2112 + 4096])
    return q


def test_forward_matches_oracle(frgpu, oracle):
    from frgpu.learned import MLPIndicator

    m = MLPIndicator(seed=3)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (1000, 32)).astype(np.float32)
    y = m.forward(x)
    ref = oracle.mlp_forward(rounded_params(m.params), bf16(x))
    assert y.shape == (1000,)
    err = np.abs(y - ref)
    print(f"tcgen05 forward vs FP64 oracle: max {err.max():.2e}, mean {err.mean():.2e}")
    assert err.max() < 2e-2
    # every row is computed on its own: ragged groups (n not a multiple of the
    # 64-row group) and single samples give the same values
    for k in (1, 7, 63, 64, 65, 129):
        np.testing.assert_allclose(m.forward(x[:k]), y[:k], rtol=0, atol=1e-6)


def test_gradient_matches_oracle(frgpu, oracle):
    from frgpu.learned import MLPIndicator

    m = MLPIndicator(seed=5)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (517, 32)).astype(np.float32)
    t = (rng.random(517) < 0.3).astype(np.float32)
    loss, g = m.loss_grad(x, t)
    lref, gref = oracle.mlp_loss_grad(rounded_params(m.params), bf16(x), t)
    assert abs(loss - lref) < 2e-2 * abs(lref)
    assert np.linalg.norm(g - gref) < 6e-2 * np.linalg.norm(gref)
    # every block of parameters receives its gradient
    for a, b in ((0, 2048), (2048, 2112), (2112, 6208), (6208, 6272), (6272, 6336), (6336, 6337)):
        assert np.linalg.norm(g[a:b] - gref[a:b]) < 0.1 * np.linalg.norm(gref[a:b]) + 1e-6


def test_training_learns_a_separable_rule(frgpu):
    from frgpu.learned import MLPIndicator

    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, (20000, 32)).astype(np.float32)
    t = ((x[:, 15] + 0.5 * x[:, 31]) > 0.2).astype(np.float32)
    m = MLPIndicator(seed=1)
    losses = m.train(x, t, epochs=8, batch=1024, lr=3e-3, seed=0)
    assert losses[-1] < 0.5 * losses[0]
    acc = np.mean((m.forward(x) > 0.5) == (t > 0.5))
    assert acc > 0.97, acc


def test_features_match_oracle(frgpu, oracle):
    from frgpu import learned

    ps = frgpu.FRPSpace2D(0, 2, 40, 0, 1, 20, 3)
    u, _ = learned.shock_vortex_state(ps.xpg, 0.3)
    prob = frgpu.FREuler2DProblem(u, (0, 1), ps, 1.4, flux="hll", bc="copy")
    frgpu.init(prob, dt=1e-4)
    feat = np.zeros(40 * 20 * 32, dtype=np.float32)
    frgpu._lib.check(frgpu.lib().frgpu_modal_features(prob._h, frgpu._lib.fptr(feat), feat.size))
    feat = feat.reshape(-1, 32)
    po = oracle.Space2D(0, 2, 40, 0, 1, 20, 3)
    ref = oracle.Problem(oracle.EULER2D, po, gamma=1.4).features2d(u)
    # compare where the mode carries energy well above FP32 rounding noise
    sel = ref > 1 - 8 / 8.0  # log10 energy fraction above -8
    assert sel.sum() > 1000
    assert np.max(np.abs(feat[sel] - ref[sel])) < 2e-3


def test_indicator_with_full_fallback_equals_plain_filter(frgpu):
    """band = 0.5 sends every element to the plain test: the learned path then
    reproduces the plain indicator + filter exactly (FP64 state)."""
    from frgpu import learned

    ps = frgpu.FRPSpace2D(0, 2, 80, 0, 1, 40, 3)
    m = learned.MLPIndicator(seed=0)
    S0 = learned.filter_S0(3)
    res = []
    for mode in ("plain", "mlp"):
        # the vortex reaches the grid-aligned shock and bends it: the last
        # flattened mode, which the modal-decay test reads, then carries energy
        u, up = learned.shock_vortex_state(ps.xpg, 0.3)
        prob = frgpu.FREuler2DProblem(u, (0, 1), ps, 1.4, flux="hll", bc=("fix", "copy", "copy", "copy"),
                                      fixed_states=[up, None, None, None])
        itg = frgpu.init(prob, dt=5e-4)
        itg.set_filter("plain", learned.FILTER_LAMBDA, S0, learned.FILTER_KAPPA)
        itg.step(396)
        itg.set_filter("none")  # a few unfiltered steps, so the test below has troubled cells to find
        itg.step(4)
        if mode == "mlp":
            frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, m._h, 0.5, 0.4999))
        n = itg.modal_filter(mode, learned.FILTER_LAMBDA, S0, learned.FILTER_KAPPA)
        res.append((n, itg.troubled(), itg.u))
    assert res[0][0] == res[1][0] and res[0][0] > 0
    assert np.array_equal(res[0][1], res[1][1])
    # the plain path evaluates the test in FP64, the learned path's fallback in FP32
    np.testing.assert_allclose(res[1][2], res[0][2], rtol=0, atol=1e-12)


def test_learned_indicator_trains_and_judges_misfires(frgpu):
    """Small end-to-end run: labels from plain-indicator shock-vortex runs at
    100 x 50 (4 vortex strengths), training on the GPU, then the learned
    indicator inside the step graph on a held-out strength.  The network must
    agree with the plain test on at least 95% of the elements it sees
    (misfires judged by the plain test), and the run must stay finite."""
    from frgpu import learned

    ps = frgpu.FRPSpace2D(0, 2, 100, 0, 1, 50, 3)
    x, t = learned.build_dataset(ps, seeds=range(4), nsteps=600, every=50, keep_neg=0.2)
    assert t.sum() > 50
    xb, tb = learned.balance(x, t, seed=0)
    m = learned.MLPIndicator(seed=0)
    losses = m.train(xb, tb, epochs=30, batch=512, lr=3e-3)
    assert losses[-1] < losses[0]
    prob = learned.shock_vortex_problem(ps, 0.27)
    frgpu._lib.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, m._h, 0.5, 0.0))
    itg = frgpu.init(prob, dt=1.0)
    itg.dt = itg.cfl_dt(0.1)
    itg.set_filter("mlp", learned.FILTER_LAMBDA, learned.filter_S0(3), learned.FILTER_KAPPA)
    itg.step(200)
    stats = np.zeros(3, dtype=np.int32)
    frgpu._lib.check(frgpu.lib().frgpu_indicator_stats(prob._h, stats.ctypes.data_as(frgpu._lib._I)))
    ne = 100 * 50
    assert stats[1] <= 0.05 * ne, stats
    assert np.all(np.isfinite(itg.u))


def test_fused_indicator_agrees_with_separate_kernel(frgpu):
    """The learned indicator inside the third SSPRK3 stage (FP32K, deg 3; the
    network as warp-level mma.sync) and the stand-alone indicator kernel after
    the step (the network on the tcgen05 tensor cores with TMEM accumulators)
    see the same features and weights; their FP32 accumulations differ in
    order only.  After 400 steps of the shock-vortex problem: the troubled
    counts within 1 %, the last step's flags equal on at least 99.9 % of the
    elements, the states within 1e-3 RMS of max |u| (an element whose network
    output sits at the threshold can be filtered by one and not the other), and
    one launch fewer per step when fused."""
    from frgpu import _lib as L
    from frgpu import learned

    ps = frgpu.FRPSpace2D(0, 2, 100, 0, 1, 50, 3)
    net = learned.load_trained()
    out = []
    for fuse in (1, 0):
        prob = learned.shock_vortex_problem(ps, 0.3)
        prob.set_option(L.OPT_FUSED_INDICATOR, fuse)
        itg = frgpu.init(prob, dt=1.0)
        itg.dt = itg.cfl_dt(0.1)
        L.check(frgpu.lib().frgpu_problem_set_mlp(prob._h, net._h, 0.5, 0.02))
        itg.set_filter("mlp", learned.FILTER_LAMBDA, learned.filter_S0(3), learned.FILTER_KAPPA)
        l0 = itg.launches()
        total = 0
        st = np.zeros(3, dtype=np.int32)
        for _ in range(400):
            itg.step(1)
            L.check(frgpu.lib().frgpu_indicator_stats(prob._h, st.ctypes.data_as(L._I)))
            total += int(st[0])
        launches = itg.launches() - l0
        out.append((itg.u, itg.troubled(), total, launches))
    (u1, f1, t1, n1), (u0, f0, t0, n0) = out
    rms = float(np.sqrt(np.mean((u1 - u0) ** 2)) / np.max(np.abs(u0)))
    agree = float(np.mean(f1 == f0))
    print(f"fused (mma.sync) vs separate (tcgen05): troubled {t1} vs {t0}, flag agreement {agree:.5f}, rms {rms:.2e}")
    assert f1.sum() > 0 and t0 > 0  # the vortex has met the shock: something was filtered
    assert abs(t1 - t0) <= 0.01 * t0
    assert agree >= 0.999
    assert rms < 1e-3
    assert n1 < n0  # one launch fewer per step