"""Generate tests/golden/tri_quadrature.npz: the triangle solution points and
weights of FluxReconstruction.jl's tri_quadrature(deg) (src/Quadrature/
quadrature.jl:14-71) for deg = 1, 2, 3.

The Williams-Shunn-Jameson schemes come from the reference's own Python module
src/Quadrature/qpmin.py (imported from a checkout of the reference, with its
JSON tables); the trilinear -> Cartesian step on the default equilateral
vertices and the equilateral -> right-triangle map xy_rs
(src/Geometry/geo_transform.jl:65-73) are restated here in numpy.  Run from
the repository root with the reference checkout path as the argument:

    python tests/golden/make_tri_quadrature.py <reference checkout>
"""
import os
import sys

import numpy as np


def main(ref):
    sys.path.insert(0, os.path.join(ref, "src", "Quadrature"))
    import qpmin  # noqa: E402  (the reference's module)

    p1 = np.array([-1.0, -1.0 / np.sqrt(3.0)])
    p2 = np.array([1.0, -1.0 / np.sqrt(3.0)])
    p3 = np.array([0.0, 2.0 / np.sqrt(3.0)])
    a, b, c = np.linalg.norm(p2 - p3), np.linalg.norm(p3 - p1), np.linalg.norm(p2 - p1)
    out = {}
    for deg in (1, 2, 3):
        scheme = getattr(qpmin, f"williams_shunn_jameson_{deg + 1}")()
        pts0 = np.asarray(scheme.points, dtype=np.float64)
        w = np.asarray(scheme.weights, dtype=np.float64)
        xy = np.zeros((pts0.shape[1], 2))
        for i in range(pts0.shape[1]):
            x, y, z = pts0[:, i]
            xy[i] = (a * x * p1 + b * y * p2 + c * z * p3) / (a * x + b * y + c * z)
        L1 = (np.sqrt(3.0) * xy[:, 1] + 1.0) / 3.0
        L2 = (-3.0 * xy[:, 0] - np.sqrt(3.0) * xy[:, 1] + 2.0) / 6.0
        L3 = (3.0 * xy[:, 0] - np.sqrt(3.0) * xy[:, 1] + 2.0) / 6.0
        out[f"r{deg}"] = -L2 + L3 - L1
        out[f"s{deg}"] = -L2 - L3 + L1
        out[f"w{deg}"] = w
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tri_quadrature.npz")
    np.savez(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FR_REFERENCE")
    if not ref:
        sys.exit("usage: make_tri_quadrature.py <reference checkout> (or set FR_REFERENCE)")
    main(ref)
