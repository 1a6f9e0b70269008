"""The FP32 BGK 1D1V path with its transport on the tensor cores
(example/bgk_wave.jl:69-129; TF32-split m16n8k8 products, bgk_tc.cu).

Tolerances (relative to max |oracle|, FP64 oracle): 2e-3 for one residual
evaluation (the relaxation term (M - u)/tau multiplies the FP32 rounding of the
Maxwellian and of the stored state by 1/tau = 100, and the derivative operator
grows with the degree), 2e-5 for the state after 25 SSPRK3 steps on small
cases, 1e-5 for the moments (rho, rho U, E) of the 256-element, 512-velocity,
p = 3 workload, and 1e-5 for its mass drift (the FP32 Maxwellian's density
differs from the moment it was built from by a rounding error in every stage,
times dt/tau).  Tile edge cases: element counts
that are not a multiple of the tile's element count, velocity counts that are
not a multiple of 8, and an 8-velocity tile that straddles v = 0.
"""
import math

import numpy as np
import pytest

from test_parity_gpu import oracle_space1d, rel

pytestmark = pytest.mark.gpu


def maxwellian_ic(xpg, v, ne, deg, amp=0.1):
    rho = 1 + amp * np.sin(2 * np.pi * xpg)
    f = np.zeros((ne, len(v), deg + 1), order="F")
    for k in range(deg + 1):
        # Maxwellian with U = 1, T = 1 (lambda = 1/2 ... prim [rho, 1, 1]) as at bgk_wave.jl:34-40
        f[:, :, k] = rho[:, k, None] * np.sqrt(1 / np.pi) * np.exp(-(v[None, :] - 1) ** 2)
    return f


def moments(f, v, w):
    """rho, rho U, E per (element, point) of u[i, v, k]."""
    m0 = np.einsum("ivk,v->ik", f, w)
    m1 = np.einsum("ivk,v->ik", f, w * v)
    m2 = np.einsum("ivk,v->ik", f, 0.5 * w * v * v)
    return np.stack([m0, m1, m2])


def bgk_pair(frgpu, oracle, ne, deg, v, w, tau, precision="fp32k"):
    ps = frgpu.FRPSpace1D(0, 1, ne, deg)
    po = oracle_space1d(ps, 0, 1, ne, deg)
    f = maxwellian_ic(ps.xpg, v, ne, deg)
    prob = frgpu.FRBGKProblem(f, (0, 1), ps, v, w, tau, precision=precision)
    P = oracle.Problem(oracle.BGK1D, po, tau=tau, velo=v, weights=w)
    return ps, f, prob, P


@pytest.mark.parametrize("deg", [1, 2, 3, 4, 5])
def test_bgk_tensor_core_matches_oracle(frgpu, oracle, deg):
    ne, nv = 61, 100
    # asymmetric grid: v = 0 falls inside the velocity tile 40..47
    dv = 0.16
    v = -7 + (np.arange(nv) + 0.5) * dv
    w = np.full(nv, dv)
    ps, f, prob, P = bgk_pair(frgpu, oracle, ne, deg, v, w, 1e-2)
    assert rel(prob.rhs(f), P.rhs(f)) < 2e-3
    dt = 0.1 * (1 / ne) / 9
    itg = frgpu.init(prob, dt=dt)
    itg.step(25)
    assert rel(itg.u, P.ssprk3(f, dt, 25)) < 2e-5


def test_bgk_tensor_and_cuda_core_forms_agree(frgpu, oracle):
    from frgpu import _lib as L

    ne, nv, deg = 64, 96, 3
    dv = 16 / nv
    v = -8 + (np.arange(nv) + 0.5) * dv
    w = np.full(nv, dv)
    outs = []
    for on in (1, 0):
        ps, f, prob, _ = bgk_pair(frgpu, oracle, ne, deg, v, w, 1e-2)
        prob.set_option(L.OPT_BGK_TENSOR, on)
        itg = frgpu.init(prob, dt=0.1 / ne / 8)
        l0 = itg.launches()
        itg.step(20)
        # tensor-core form: a moments kernel and a transport kernel per stage
        assert itg.launches() - l0 == (120 if on else 60)
        outs.append(itg.u)
    assert rel(outs[0], outs[1]) < 1e-5


@pytest.mark.parametrize("deg", [1, 2, 3, 4, 5])
def test_bgk_tcgen05_form_matches_mma_sync_form(frgpu, oracle, deg):
    """The transport product on tcgen05 (FRGPU_OPT_BGK_TENSOR = 2: 128
    velocities per CTA, TF32 operands in shared memory, FP32 accumulators in
    tensor memory) accumulates the same split terms in the same order as the
    mma.sync form: the same bits for one residual and after 25 steps, on a grid
    whose 100 velocities fill one 128-velocity tile with both signs."""
    from frgpu import _lib as L

    ne, nv = 61, 100
    dv = 0.16
    v = -7 + (np.arange(nv) + 0.5) * dv
    w = np.full(nv, dv)
    dt = 0.1 * (1 / ne) / 9
    outs = []
    for form in (1, 2):
        ps, f, prob, P = bgk_pair(frgpu, oracle, ne, deg, v, w, 1e-2)
        prob.set_option(L.OPT_BGK_TENSOR, form)
        r = prob.rhs(f)
        itg = frgpu.init(prob, dt=dt)
        l0 = itg.launches()
        itg.step(25)
        assert itg.launches() - l0 == 150  # a moments and a transport kernel per stage
        outs.append((r, itg.u))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    assert rel(outs[1][1], P.ssprk3(f, dt, 25)) < 2e-5


@pytest.mark.parametrize("kn", [1e-4, 1e-2])
def test_bgk_workload_moments_match_oracle(frgpu, oracle, kn):
    """256 elements on periodic [0,1], p = 3, 512 velocity midpoints on [-8,8],
    tau = Kn, Maxwellian IC rho = 1 + 0.1 sin(2 pi x), U = 1, T = 1,
    SSPRK3 at dt = 0.1 dx / 8 for 200 steps; moments vs the FP64 oracle, and
    mass conserved to FP32 round-off."""
    ne, nv, deg = 256, 512, 3
    dv = 16 / nv
    v = -8 + (np.arange(nv) + 0.5) * dv
    w = np.full(nv, dv)
    ps, f, prob, P = bgk_pair(frgpu, oracle, ne, deg, v, w, kn)
    dt = 0.1 * (1 / ne) / 8
    itg = frgpu.init(prob, dt=dt)
    itg.step(200)
    got = itg.u
    ref = P.ssprk3(f, dt, 200)
    mg, mr = moments(got, v, w), moments(ref, v, w)
    for q in range(3):
        assert rel(mg[q], mr[q]) < 1e-5, q
    wq = np.asarray(ps.wp) * (1 / ne) / 2
    mass0 = np.sum(moments(f, v, w)[0] * wq[None, :])
    mass_gpu, mass_ref = np.sum(mg[0] * wq[None, :]), np.sum(mr[0] * wq[None, :])
    assert abs(mass_gpu - mass0) < 1e-5 * mass0
    assert abs(mass_ref - mass0) < 1e-10 * mass0  # FP64: conserved to round-off
