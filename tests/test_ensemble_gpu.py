"""The batched 1D Burgers ensemble (one persistent launch for all instances).

FP64: every instance is checked bit for bit against the oracle run with the
same time step (dt_i = cfl dx_i / ((2 deg_i + 1) max|u_i|), the last step
shortened to land on t_end) and the same post-step indicator + :l2 filter
(example/euler_highlevel.jl:37-52).  The tile shape (warp or CTA per
instance) must not change the results.  FP32 is held to 2e-4 relative.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_run(oracle, frgpu, ne, deg, u0, t_end, cfl, filt):
    ps = frgpu.FRPSpace1D(0, 2 * math.pi, ne, deg)
    po = oracle.Space1D(0, 2 * math.pi, ne, deg)
    for f in ("ll", "lr", "dl", "dhl", "dhr", "V", "iV", "wp", "J"):
        setattr(po, f, np.array(getattr(ps, f)))
    P = oracle.Problem(oracle.BURGERS, po)
    dx = (2 * math.pi) / ne
    umax = float(np.max(np.abs(u0)))
    dt = (cfl * dx) / ((2.0 * deg + 1.0) * umax)
    nfull = math.floor(t_end / dt)
    last = t_end - nfull * dt
    u = np.asfortranarray(u0)
    steps = [dt] * nfull + ([last] if last > 0 else [])
    for h in steps:
        u = P.ssprk3(u, h, 1)
        if filt:
            u, _, _ = P.filter1d(u, 1, h * math.exp(0.875 * deg) * 0.15)
    return u, dt, len(steps)


def small_ensemble(frgpu, precision):
    from frgpu.ensemble import Ensemble

    ne = [17, 40, 64, 100, 130, 256, 300, 700, 33, 512, 90, 2048, 48, 200, 999, 61]
    deg = [1, 2, 3, 4, 5, 1, 2, 3, 4, 5, 3, 2, 5, 4, 1, 3]
    e = Ensemble(ne, deg, precision=precision)
    e.init_fourier(0.3, seed=7)
    return e


def test_ensemble_fp64_matches_oracle_bitwise(frgpu, oracle):
    e = small_ensemble(frgpu, "fp64")
    u0 = [e.get_state(i) for i in range(e.n)]
    e.tiles = [64, 128, 128, 256, 64]
    e.run(0.02, cfl=0.4, filter=True)
    st = e.stats()
    for i in range(e.n):
        if e.ne[i] > 300:  # the oracle's Python stepping loop is slow for the largest instances
            continue
        ref, dt, n = oracle_run(oracle, frgpu, int(e.ne[i]), int(e.deg[i]), u0[i], 0.02, 0.4, True)
        assert st["dt"][i] == dt and st["steps"][i] == n, i
        assert np.array_equal(e.get_state(i), ref), i
    assert st["dof_stage_updates"] == sum(3 * e.ne[i] * (e.deg[i] + 1) * st["steps"][i] for i in range(e.n))


def test_tile_shape_does_not_change_results(frgpu):
    outs = []
    for thr in ([0, 0, 0, 0, 0], [512, 512, 512, 512, 512], [64, 256, 0, 128, 512]):
        e = small_ensemble(frgpu, "fp64")
        e.tiles = thr
        e.run(0.01)
        outs.append([e.get_state(i) for i in range(e.n)])
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)


def test_ensemble_fp32_close_to_fp64(frgpu):
    e64 = small_ensemble(frgpu, "fp64")
    e32 = small_ensemble(frgpu, "fp32")
    e64.run(0.01, filter=False)
    e32.run(0.01, filter=False)
    for i in range(e64.n):
        a, b = e32.get_state(i), e64.get_state(i)
        assert np.max(np.abs(a - b)) < 2e-4 * np.max(np.abs(b)) + 1e-6, i


def test_config4_sizes_and_autotuner(frgpu):
    from frgpu.ensemble import Ensemble, config4_sizes

    ne, deg = config4_sizes(4096, 0)
    ne2, deg2 = config4_sizes(4096, 0)
    assert np.array_equal(ne, ne2) and np.array_equal(deg, deg2)
    assert ne.min() >= 32 and ne.max() <= 2048 and set(np.unique(deg)) == {1, 2, 3, 4, 5}
    # log-uniform: about half of the instances below sqrt(32 * 2048) = 256
    assert 0.4 < np.mean(ne < 256) < 0.6
    e = Ensemble(ne[:256], deg[:256], precision="fp32")
    e.init_fourier(0.3, 0)
    before = [e.get_state(i) for i in range(0, 256, 37)]
    thr = e.tune(t_probe=0.002)
    assert all(t in (0, 64, 128, 256, 512) for t in thr)
    # tuning restores the state it probes with
    after = [e.get_state(i) for i in range(0, 256, 37)]
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    e.run(0.01)
    assert np.all(np.isfinite(e.get_state(0)))


# ---------------------------------------------------------------- learned 1D indicator
def test_ensemble_features_and_labels_match_oracle(frgpu, oracle):
    """Features (BF16-rounded, as the network sees them) and plain labels of
    every element against the oracle's features1d and filter1d flags."""
    e = small_ensemble(frgpu, "fp64")
    e.run(0.1, filter=True)  # steepening fronts: some elements are troubled
    feat, lab = e.features()
    assert feat.shape == (e.nelem, 32) and lab.sum() > 0
    row = 0
    for i in range(e.n):
        ne, deg = int(e.ne[i]), int(e.deg[i])
        u = e.get_state(i)
        ps = frgpu.FRPSpace1D(0, 2 * math.pi, ne, deg)
        po = oracle.Space1D(0, 2 * math.pi, ne, deg)
        for f in ("ll", "lr", "dl", "dhl", "dhr", "V", "iV", "wp", "J"):
            setattr(po, f, np.array(getattr(ps, f)))
        P = oracle.Problem(oracle.BURGERS, po)
        ref = P.features1d(u)
        _, flags, _ = P.filter1d(u, 1, 0.0)
        got = feat[row:row + ne]
        assert np.array_equal(lab[row:row + ne], flags), i
        # BF16 keeps 8 significant bits; compare modes carrying energy above 1e-8 of the total
        sel = np.zeros_like(ref, dtype=bool)
        sel[:, :deg + 1] = ref[:, :deg + 1] > 0
        sel[:, 8:17] = True
        assert np.max(np.abs(got[sel] - ref[sel])) < 1e-2, i
        row += ne
    assert row == e.nelem


def test_learned_full_fallback_equals_plain(frgpu):
    """band = 0.5 sends every element the network is consulted for to the
    plain test, and the elements in the plain test's sigma = 1 region are smooth
    without the network: the learned path must then reproduce the plain
    indicator + filter bit for bit (FP64)."""
    from frgpu import learned

    outs = []
    for mode in ("plain", "mlp"):
        e = small_ensemble(frgpu, "fp64")
        if mode == "mlp":
            e.set_mlp(learned.MLPIndicator(seed=3), 0.5, 0.5)
        e.run(0.2, filter=True)
        outs.append([e.get_state(i) for i in range(e.n)])
        if mode == "mlp":
            st = e.indicator_stats()
            # floor elements are network decisions that agree with the plain test
            assert 0 < st["fallbacks"] < st["judged"] and st["troubled"] > 0
            assert st["misfires"] <= st["fallbacks"]
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_trained_burgers1d_indicator_agrees_with_plain(frgpu):
    """The shipped 1D network on held-out config-4 instances (seed 0, which
    training never saw): misfires below 5% of the elements judged, finite run."""
    import os

    from frgpu import learned
    from frgpu.ensemble import Ensemble

    if not os.path.exists(learned.BURGERS_WEIGHTS):
        pytest.skip("no trained 1D network shipped yet")
    e = Ensemble.config4(512, seed=0, precision="fp32")
    e.set_mlp(learned.load_trained_burgers1d(), 0.5, 0.0)
    e.run(0.5)
    st = e.indicator_stats()
    assert st["judged"] > 0 and st["troubled"] > 0
    assert st["misfires"] < 0.05 * st["judged"]
    assert all(np.all(np.isfinite(e.get_state(i))) for i in range(0, 512, 51))


def test_non_finite_instance_stops_alone(frgpu, oracle):
    """An instance whose state turns non-finite (here: one value of the
    2048-element p = 2 instance set to NaN on the host before the run) stops
    after its first step; the other 15 instances finish and still match the
    oracle bit for bit, and setting its state again revives it."""
    e = small_ensemble(frgpu, "fp64")
    u0 = [e.get_state(i) for i in range(e.n)]
    bad = u0[11].copy()
    bad.flat[1000] = np.nan
    e.set_state(11, bad)
    e.run(0.3, filter=True)
    f = e.failed()
    assert np.flatnonzero(f).tolist() == [11] and f[11] == 1
    for i in (0, 4, 12, 15):
        ref, _, _ = oracle_run(oracle, frgpu, int(e.ne[i]), int(e.deg[i]), u0[i], 0.3, 0.4, True)
        assert np.array_equal(e.get_state(i), ref), i
    e.set_state(11, u0[11])
    assert e.failed()[11] == 0
    # a state of huge magnitude would need more than 2e9 CFL steps: not started
    big = u0[3].copy()
    big.flat[7] = 1e200
    e.set_state(3, big)
    e.run(0.01, filter=True)
    f = e.failed()
    assert f[3] == -1 and np.flatnonzero(f).tolist() == [3]
    assert e.stats()["steps"][3] == 0
