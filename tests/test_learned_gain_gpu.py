"""What the trained network gains over the method without it.

The method without it is the plain modal-decay indicator (shock_detector,
src/dissipation.jl:13-23) with the :l2 filter after every step
(example/shock-vortex.jl:308-321).  Both run fused into the third SSPRK3 stage
of the FP32K kernel on the same features, so the comparison isolates the
decision.  Workload: the shock-vortex problem (400 x 200, p = 3, HLL) at two
vortex strengths, 600 steps from the initial state (the vortex meets the shock
near step 150), with the ghosts refreshed once per step as the script does.
Accuracy: the L2 error of the density against a converged FP64 solution (the
FP64 form, plain indicator, on the 2x refined mesh with half the step,
evaluated at the coarse solution points).

Measured, and asserted here:
* the indicator matters: without it the run loses positivity before step 600;
* at the shipped decision threshold (0.97) the network filters fewer elements
  than the plain test over the run, with an L2 error within 0.5 % of the plain
  test's.
It costs time: the fused network adds a few per cent to the step on this
workload (bench.py reports both forms).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 600


def _run(frgpu, ps, mach, dt, indicator, net=None, thr=None):
    from frgpu import _lib as L
    from frgpu import learned

    prob = learned.shock_vortex_problem(ps, mach, precision="fp32k")
    itg = frgpu.init(prob, dt=dt)
    if indicator == "mlp":
        L.check(L.lib().frgpu_problem_set_mlp(prob._h, net._h, thr, 0.0))
    itg.set_filter(indicator, learned.FILTER_LAMBDA, learned.filter_S0(3), learned.FILTER_KAPPA)
    st = np.zeros(3, dtype=np.int32)
    total = 0
    for _ in range(STEPS):
        itg.step(1)
        if indicator != "none":
            L.check(L.lib().frgpu_indicator_stats(prob._h, st.ctypes.data_as(L._I)))
            total += int(st[0])
    return itg.u[..., 0], total


@pytest.mark.parametrize("mach", [0.25, 0.4])
def test_learned_indicator_filters_less_at_equal_accuracy(frgpu, mach):
    from frgpu import learned

    ps = learned.config3_space()
    u0, _ = learned.shock_vortex_state(ps.xpg, mach)
    U = u0[..., 1] / u0[..., 0]
    V = u0[..., 2] / u0[..., 0]
    p = 0.4 * (u0[..., 3] - 0.5 * (u0[..., 1] * U + u0[..., 2] * V))
    c = np.sqrt(1.4 * p / u0[..., 0])
    dt = 0.1 / float(np.max((np.abs(U) + c) / ps.dx + (np.abs(V) + c) / ps.dy))
    # converged solution
    psf = frgpu.FRPSpace2D(ps.x0, ps.x1, 2 * ps.nx, ps.y0, ps.y1, 2 * ps.ny, 3)
    itf = frgpu.init(learned.shock_vortex_problem(psf, mach, precision="fp64"), dt=dt / 2)
    itf.set_filter("plain", learned.FILTER_LAMBDA, learned.filter_S0(3), learned.FILTER_KAPPA)
    itf.step(2 * STEPS)
    truth = frgpu.refined_at_coarse_points(itf.u, ps.xpl)[..., 0]
    del itf
    w1 = np.polynomial.legendre.leggauss(4)[1]

    def err(rho):
        return frgpu.quadrature_L2_error(rho, truth, ps.dx, ps.dy, w1)

    net = learned.load_trained()
    rp, np_ = _run(frgpu, ps, mach, dt, "plain")
    rl, nl = _run(frgpu, ps, mach, dt, "mlp", net, learned.DECISION_THRESHOLD)
    ep, el = err(rp), err(rl)
    print(f"Mach {mach}: plain {np_} filterings, L2 {ep:.4e}; learned {nl} filterings ({nl / np_ - 1:+.2%}), "
          f"L2 {el:.4e} ({el / ep - 1:+.3%})")
    with pytest.raises(frgpu.FRGPUError):
        _run(frgpu, ps, mach, dt, "none")
    assert nl < np_
    assert el <= 1.005 * ep
