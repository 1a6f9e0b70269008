"""C-ABI checks that need no GPU: libfrgpu.so loads, exports every function
include/frgpu.h declares, its host-side setup math matches the golden vectors
and the oracle, and its compute entry points fail loudly without a device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "frgpu.h")
GOLD = os.path.join(ROOT, "tests", "golden", "setup_math.npz")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"FRGPU_API\s+[\w\s\*]+?\b(frgpu_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) >= 30
    assert "frgpu_rhs" in names and "frgpu_step_ssprk3" in names and "frgpu_interp_face" in names


def test_library_exports_every_declared_symbol(frgpu):
    from frgpu import _lib

    L = C.CDLL(_lib._build.LIB)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding covers exactly the declared entry points
    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_no_unexported_internal_symbols(frgpu):
    """Only the C ABI is visible (the build hides everything else)."""
    import subprocess

    from frgpu import _lib

    out = subprocess.run(["nm", "-D", "--defined-only", _lib._build.LIB], capture_output=True, text=True).stdout
    ours = [ln.split()[-1] for ln in out.splitlines() if " T " in ln and ln.split()[-1].startswith("fr")]
    assert set(ours) <= set(declared_functions()), set(ours) - set(declared_functions())


@pytest.mark.parametrize("deg", [1, 2, 3, 4, 5])
def test_host_setup_math_matches_golden(frgpu, deg):
    g = np.load(GOLD)
    x = frgpu.legendre_point(deg)
    np.testing.assert_allclose(x, g[f"x{deg}"], atol=2e-16)
    np.testing.assert_allclose(frgpu.gauss_weights(deg), g[f"w{deg}"], atol=5e-16)
    ll, lr, dl = frgpu.standard_lagrange(x)
    np.testing.assert_allclose(ll, g[f"ll{deg}"], atol=5e-15)
    np.testing.assert_allclose(lr, g[f"lr{deg}"], atol=5e-15)
    np.testing.assert_allclose(dl, g[f"dl{deg}"], atol=5e-14)
    for name, fn in (("radau", frgpu.dradau), ("sd", frgpu.dsd), ("huynh", frgpu.dhuynh)):
        gl, gr = fn(deg, x)
        np.testing.assert_allclose(gl, g[f"{name}_l{deg}"], atol=5e-14)
        np.testing.assert_allclose(gr, g[f"{name}_r{deg}"], atol=5e-14)
    np.testing.assert_allclose(frgpu.vandermonde_matrix(deg, x), g[f"V{deg}"], atol=5e-15)


def test_spaces_match_oracle(frgpu, oracle):
    ps = frgpu.FRPSpace1D(0, 1, 100, 2)
    po = oracle.Space1D(0, 1, 100, 2)
    for f in ("xpl", "wp", "ll", "lr", "dl", "dhl", "dhr", "J", "V"):
        np.testing.assert_allclose(getattr(ps, f), getattr(po, f), atol=1e-13, err_msg=f)
    np.testing.assert_allclose(ps.iV, po.iV, atol=1e-12)
    np.testing.assert_allclose(ps.xpg, po.xpg, atol=1e-15)
    p2 = frgpu.FRPSpace2D(0, 2, 40, 0, 1, 20, 3)
    o2 = oracle.Space2D(0, 2, 40, 0, 1, 20, 3)
    for f in ("xpl", "wp", "ll", "lr", "dl", "dhl", "dhr", "V"):
        np.testing.assert_allclose(getattr(p2, f), getattr(o2, f), atol=1e-13, err_msg=f)
    np.testing.assert_allclose(p2.iV, o2.iV, atol=1e-12)
    np.testing.assert_allclose(p2.xpg, o2.xpg, atol=1e-15)
    assert p2.np == 16  # (deg+1)^2 as in src/struct.jl:221


def test_sd_and_huynh_spaces(frgpu, oracle):
    for corr in ("sd", "huynh"):
        ps = frgpu.FRPSpace1D(0, 1, 10, 3, 0, corr)
        po = oracle.Space1D(0, 1, 10, 3, corr)
        np.testing.assert_allclose(ps.dhl, po.dhl, atol=1e-13)
        np.testing.assert_allclose(ps.dhr, po.dhr, atol=1e-13)


def test_shock_detector_host(frgpu, oracle):
    for Se in (-np.inf, np.log10(0.1), np.log10(1e5), -5.3, -1.2, -8.0):
        for deg in (2, 3, 5):
            assert frgpu.shock_detector(Se, deg) == oracle.shock_detector(Se, deg)


def test_bad_arguments_are_rejected(frgpu):
    from frgpu import _lib

    L = _lib.lib()
    h = C.c_void_p()
    assert L.frgpu_space_create_1d(0.0, 1.0, 0, 2, 0, C.byref(h)) == _lib.ERR_ARG
    assert "nx" in _lib.last_error()
    assert L.frgpu_space_create_1d(1.0, 0.0, 4, 2, 0, C.byref(h)) == _lib.ERR_ARG
    assert L.frgpu_space_create_2d(0.0, 1.0, 4, 0.0, 1.0, 4, 9, C.byref(h)) == _lib.ERR_ARG
    assert L.frgpu_step_ssprk3(None, 0.1, 1) == _lib.ERR_ARG
    with pytest.raises(frgpu.FRGPUError):
        frgpu.FRPSpace1D(0, 1, 10, 0)


def test_compute_fails_loudly_without_gpu(frgpu, has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present: the compute path is exercised by the gpu tests")
    ps = frgpu.FRPSpace1D(0, 1, 10, 2)
    with pytest.raises(frgpu.FRGPUError) as e:
        frgpu.FRAdvectionProblem(np.zeros((10, 3)), (0, 1), ps, 1.0, "period")
    assert e.value.code == -2
    with pytest.raises(frgpu.FRGPUError):
        fd = np.zeros((4, 2))
        frgpu.interp_face_(fd, np.ones((4, 3)), ps.ll, ps.lr)


def test_new_entry_points_reject_bad_arguments(frgpu):
    """Argument checks of the limiter, tableau and metric entry points run
    before any device work."""
    from frgpu import _lib

    L = _lib.lib()
    n = C.c_int(0)
    A = np.array([[0.0, 0.0], [0.5, 0.0]])
    b = np.array([0.0, 1.0])
    assert L.frgpu_positive_limiter(None, None, 1.0, C.byref(n)) == _lib.ERR_ARG
    assert L.frgpu_set_limiter(None, 1, None, 1.0) == _lib.ERR_ARG
    assert L.frgpu_step_erk(None, 2, _lib.dptr(A), _lib.dptr(b), 0.1, 1) == _lib.ERR_ARG
    assert L.frgpu_problem_set_metric(None, None, None, None) == _lib.ERR_ARG
    assert "null" in _lib.last_error()
    with pytest.raises(ValueError):
        frgpu.ExplicitRK([[0.0, 0.5], [0.0, 0.0]], [0.5, 0.5])   # implicit entry above the diagonal
    assert frgpu.Midpoint().A[1, 0] == 0.5 and frgpu.Tsit5().b[-1] == 0.0


def test_allocation_free_reduction_calls_no_allocator():
    """frgpu_reduce2d_noalloc and its helpers (the end of csrc/euler2d.cu, from
    the scratch array's declaration on) name no device or host allocator."""
    src = open(os.path.join(ROOT, "fluxreconstruction.jl_gb300", "csrc", "euler2d.cu")).read()
    body = src[src.index("constexpr int NOALLOC_MAX_BLOCKS"):]
    assert "frgpu_reduce2d_noalloc" in body
    for call in ("cudaMalloc", "cudaFree", "malloc(", "calloc(", "new ", "std::vector", "cudaHostAlloc"):
        assert call not in body, call


def _c_param_counts():
    """{name: number of parameters} of every FRGPU_API declaration."""
    text = re.sub(r"/\*.*?\*/", " ", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"FRGPU_API\s+[\w\s\*]+?\b(frgpu_\w+)\s*\(([^)]*)\)", text):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = len(params)
    return out


@pytest.mark.parametrize("path", [("fluxreconstruction.jl_gb300", "julia", "FRGPU.jl"), ("INTEGRATION.md",)])
def test_julia_binding_calls_declared_entry_points(path):
    """Every ccall of the Julia shim (julia/FRGPU.jl) and of the integration
    notes names an entry point that include/frgpu.h declares, with as many
    argument types as the C function has parameters."""
    jl = open(os.path.join(ROOT, *path)).read()
    counts = _c_param_counts()
    calls = re.findall(r"ccall\(\(:(frgpu_\w+),\s*libfrgpu\),\s*[\w{}]+,\s*\(([^()]*(?:\([^()]*\)[^()]*)*)\)", jl)
    assert len(calls) >= 20 and len(calls) == len(re.findall(r"ccall\(\(:frgpu_", jl))
    for name, types in calls:
        assert name in counts, name
        n = len([t for t in types.split(",") if t.strip()])
        assert n == counts[name], (name, n, counts[name])
