"""Generate tests/golden/setup_math.npz: high-precision values of the
flux-reconstruction setup math for degrees 1..5, computed symbolically with
sympy independently of both the oracle and libfrgpu.

What is pinned (FluxReconstruction.jl definitions):
  * Gauss-Legendre nodes/weights  -- legendre_point (src/Polynomial/poly_legendre.jl:6),
                                     gausslegendre weights (src/struct.jl:47)
  * ll, lr, dl                   -- lagrange_point / dlagrange (src/Polynomial/poly_lagrange.jl:6-59)
  * dradau, dsd, dhuynh          -- src/Polynomial/poly_legendre.jl:29-71
  * V (orthonormal Legendre)     -- vandermonde_matrix (src/Transform/transform.jl:18-26)

Run:  python tests/golden/make_golden.py   (needs sympy; writes setup_math.npz)
"""
import os

import numpy as np

try:
    import sympy as sp
except ImportError as e:  # pragma: no cover
    raise SystemExit("sympy is required to regenerate the golden vectors") from e

DIGITS = 40
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    x = sp.Symbol("x")
    out = {}
    for deg in range(1, 6):
        n = deg + 1
        Pn = sp.legendre(n, x)
        roots = sorted(sp.Poly(Pn, x).nroots(n=DIGITS, maxsteps=200))
        dPn = sp.diff(Pn, x)
        nodes = [sp.Float(r, DIGITS) for r in roots]
        weights = [2 / ((1 - r ** 2) * dPn.subs(x, r) ** 2) for r in nodes]
        # Lagrange basis through the nodes
        ell = []
        for k in range(n):
            lk = sp.Integer(1)
            for j in range(n):
                if j != k:
                    lk *= (x - nodes[j]) / (nodes[k] - nodes[j])
            ell.append(sp.expand(lk))
        ll = [lk.subs(x, -1) for lk in ell]
        lr = [lk.subs(x, 1) for lk in ell]
        dl = [[sp.diff(ell[k], x).subs(x, nodes[m]) for k in range(n)] for m in range(n)]
        dP = {q: sp.diff(sp.legendre(q, x), x) if q > 0 else sp.Integer(0) for q in (deg - 1, deg, deg + 1)}
        sgn = (-1) ** deg
        corr = {}
        for name in ("radau", "sd", "huynh"):
            gl, gr = [], []
            for r in nodes:
                d = dP[deg].subs(x, r)
                dp = dP[deg + 1].subs(x, r)
                dm = dP[deg - 1].subs(x, r) if deg - 1 > 0 else 0
                if name == "radau":
                    y = dp
                elif name == "sd":
                    y = (deg * dm + (deg + 1) * dp) / (2 * deg + 1)
                else:
                    y = ((deg + 1) * dm + deg * dp) / (2 * deg + 1)
                gl.append(sgn * (d - y) / 2)
                gr.append((d + y) / 2)
            corr[name] = (gl, gr)
        V = [[sp.sqrt(sp.Rational(2 * j + 1, 2)) * sp.legendre(j, r) for j in range(n)] for r in nodes]

        def f(a):
            return np.array(sp.Matrix(a).evalf(30).tolist(), dtype=np.float64).reshape(np.shape(a))

        out[f"x{deg}"] = f(nodes)
        out[f"w{deg}"] = f(weights)
        out[f"ll{deg}"] = f(ll)
        out[f"lr{deg}"] = f(lr)
        out[f"dl{deg}"] = f(dl)
        for name, (gl, gr) in corr.items():
            out[f"{name}_l{deg}"] = f(gl)
            out[f"{name}_r{deg}"] = f(gr)
        out[f"V{deg}"] = f(V)
    np.savez(os.path.join(HERE, "setup_math.npz"), **out)
    print("wrote", os.path.join(HERE, "setup_math.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
