"""Generates tests/golden/fd_nan_element.json: one element of the 40,000-quad
cylinder mesh (element 20478, downstream of the cylinder) with its nine nodes'
coordinates and the fully developed Giesekus state (alpha = 0.1, beta = 0.59,
Wi = 0.1, SQRT form) at them, as hexadecimal floats (exact bits).  On this
element the forward-difference Jacobian of the reference algorithm has
non-finite entries (tests/test_oracle_physics.py::
test_fd_jacobian_nan_at_exact_parallel_flow).

Run:  python tests/golden/make_fd_nan_element.py   (about a minute: it builds
the 40,000-quad mesh and its fully developed state)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ve_flow_around_cylinder_fortran_gb300 import mesh as M  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import newton as N  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import state as S  # noqa: E402

ELEMENT = 20478


def main():
    mesh = M.build_cylinder_mesh(40000)
    phys = S.giesekus(0.1, 0.1, 0.59, "SQRT", nex=0)
    TL, _ = N.initial_state(mesh, phys)
    nodes = mesh.conn[:, ELEMENT].astype(np.int64) - 1        # 1-based, reference node order
    out = {
        "element": ELEMENT, "mesh": "build_cylinder_mesh(40000)",
        "physics": "giesekus(alpha=0.1, Wi=0.1, beta=0.59, SQRT, nex=0)",
        "xyz": [[float(v).hex() for v in row] for row in mesh.xyz[:, nodes]],
        "TL": [[float(v).hex() for v in row] for row in TL[:, nodes]],
    }
    with open(os.path.join(HERE, "fd_nan_element.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
