"""Generates tests/golden/golden.json: SHA-256 digests (and a few sampled
values) of the oracle's element residuals, FD Jacobians and arclength columns
for small seeded cases.  The inputs come from ``state.portable_state``
(uniform draws and elementwise IEEE arithmetic only) so they are the same
bits on every machine.  The digests pin the exact bits: the oracle must keep
producing them (CPU test), and the CUDA library must produce the same bits
(GPU test).  Models that call exp() are left out (libm's last bit is not
portable across machines).

Run:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import mesh as M  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import state as S  # noqa: E402

CASES = []
for model, ve in (("L-PTT", 0.0), ("L-PTT", 0.05), ("m-L-PTT", 0.05), ("GIESEKUS", 0.1),
                  ("FENE-CR", 40.0), ("FENE-P", 40.0)):
    for form in ("T", "SQRT"):
        CASES.append(dict(model=model, VeN=ve, form=form, Wi=0.4, beta=0.59, nex=1, seed=3,
                          nx=2, ny=2, distort=0.3))


def case_mesh(c):
    mesh = M.rect_mesh(c["nx"], c["ny"], 0.0, 1.2, -0.5, 0.7, distort=c["distort"], seed=c["seed"])
    mesh.xyz[0] += 2.0
    return mesh


def case_phys(c):
    return S.Physics(model=c["model"], form=c["form"], WiN=c["Wi"], Wi0=c["Wi"], BvN=c["beta"],
                     VeN=c["VeN"], nex=c["nex"])


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def run_case(c):
    mesh = case_mesh(c)
    phys = case_phys(c)
    TL, EU = S.portable_state(mesh.xyz, phys, c["seed"])
    res, jac, ac = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, EU)
    return mesh, phys, TL, EU, res, jac, ac


def main():
    out = []
    for c in CASES:
        _, _, _, _, res, jac, ac = run_case(c)
        out.append(dict(case=c, res_sha256=digest(res), jac_sha256=digest(jac),
                        ac_sha256=digest(ac), res_sample=[float(res[0, 4, 0]), float(res[-1, 8, 5])],
                        jac_sample=[float(jac[0, 0, 0, 0, 0]), float(jac[-1, 8, 5, 8, 5])]))
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(out)} cases")


if __name__ == "__main__":
    main()
