"""The complex-step exact Jacobian of the oracle (oracle/vefem_oracle.c built
with -DORA_COMPLEX_STEP), the reference point for the library's exact
Jacobian kernels.

It is pinned three ways on CPU: its residual (real part) equals the plain
oracle's residual bit for bit, its columns agree with a
Richardson-extrapolated central difference of the plain oracle residual
(truncation O(h^4)), and with the oracle's forward-difference Jacobian (the
reference algorithm, storeBulk Equations_mod.F90:226-313) within that
difference's truncation error.  Tolerances are relative to the largest
entry.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S

MODELS = [("L-PTT", 0.0), ("L-PTT", 0.05), ("m-L-PTT", 0.05), ("e-PTT", 0.05),
          ("m-e-PTT", 0.05), ("FENE-CR", 40.0), ("FENE-P", 40.0), ("GIESEKUS", 0.1)]


def _two_elements():
    mesh = M.rect_mesh(2, 1, 0.0, 1.0, -0.3, 0.4, distort=0.3, seed=4)
    mesh.xyz[0] += 2.0
    return mesh


def _richardson_columns(phys, mesh, TL, EU, h=2e-4):
    """d Res_e / d TL(inod, ieq) and d Res_e / d EU by central differences
    extrapolated (4 D(h/2) - D(h)) / 3, layout of the element Jacobian."""
    en = mesh.element_nodes()

    def res(tl, eu):
        return O.element_outputs(phys, mesh.conn, mesh.xyz, tl, eu, jacobian=False)[0]

    J = np.zeros((mesh.nel, 9, 6, 9, 6))
    Ac = np.zeros((mesh.nel, 9, 6))
    for e in range(mesh.nel):
        for inod in range(9):
            for ieq in range(6):
                def cd(hh):
                    tp, tm = TL.copy(), TL.copy()
                    tp[ieq, en[e, inod]] += hh
                    tm[ieq, en[e, inod]] -= hh
                    return (res(tp, EU)[e] - res(tm, EU)[e]) / (2 * hh)
                J[e, inod, ieq] = (4 * cd(h / 2) - cd(h)) / 3

    def cde(hh):
        return (res(TL, EU + hh) - res(TL, EU - hh)) / (2 * hh)
    Ac[:] = (4 * cde(h / 2) - cde(h)) / 3
    return J, Ac


@pytest.mark.parametrize("form", ["T", "SQRT"])
@pytest.mark.parametrize("model,ve", MODELS)
def test_complex_step_matches_richardson_and_fd(model, ve, form):
    mesh = _two_elements()
    phys = S.Physics(model=model, form=form, WiN=0.4, Wi0=0.4, BvN=0.59, VeN=ve, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 12)
    r, jfd, acfd = O.element_outputs(phys, mesh.conn, mesh.xyz, TL, EU)
    rc, jc, acc = O.exact_element_outputs(phys, mesh.conn, mesh.xyz, TL, EU)
    assert np.array_equal(rc, r)               # the real part is the oracle residual
    Jr, Acr = _richardson_columns(phys, mesh, TL, EU)
    sc = np.max(np.abs(jc))
    assert np.max(np.abs(jc - Jr)) < 1e-9 * sc
    assert np.max(np.abs(acc[..., 0] - Acr)) < 1e-9 * max(np.max(np.abs(acc)), 1e-300)
    # the reference's forward difference (eps = 1e-8) differs by its truncation
    assert np.max(np.abs(jc - jfd)) < 1e-6 * sc


def test_complex_step_assembly_on_cylinder():
    """Assembled into the AIJ pattern: residual bit-identical to the oracle's
    assembly, Jacobian within the forward difference's truncation."""
    mesh = M.build_cylinder_mesh(500)
    phys = S.giesekus(0.1, 0.5, 0.59, "SQRT", nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 3)
    rp, ci = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    b, v = O.exact_assemble(phys, mesh.conn, mesh.xyz, TL, EU, rp, ci)
    bf, vf = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rp, ci)
    assert np.array_equal(b, bf)
    assert np.max(np.abs(v - vf)) < 1e-6 * np.max(np.abs(vf))
