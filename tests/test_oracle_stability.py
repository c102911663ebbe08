"""CPU pins of the stability oracle (oracle/vefem_stability_oracle.c).

The reference's stability path cannot be run here and ships no data, so the
restatement is pinned by the structure the equations must have: the
perturbation residual is linear in the perturbation (so the forward-difference
blocks equal the operator applied to unit vectors), A is a quadratic
polynomial in the spanwise wavenumber, B does not depend on it, and with the
z-derivative terms off only momentumStability3D sees the wavenumber.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import state as S


def _case(model="oldroyd_b", seed=1, L2=40.0):
    mesh = M.build_cylinder_mesh(60, exact=False)
    if model == "oldroyd_b":
        phys = S.oldroyd_b(0.5, 0.59, "T", nex=0)
    elif model == "giesekus":
        phys = S.giesekus(0.2, 0.5, 0.59, "T", nex=0)
    else:
        phys = S.Physics(model={"fene_cr": "FENE-CR", "fene_p": "FENE-P"}[model], form="T",
                         WiN=0.5, Wi0=0.5, BvN=0.59, VeN=L2, nex=0)
    TL, _ = S.seeded_state(mesh.xyz, phys, seed=seed)
    nn = mesh.nnodes
    TLb = np.zeros((10, nn))
    TLb[0:2] = TL[0:2]      # Ux, Uy; Uz = 0
    TLb[3:7] = TL[2:6]      # P, Txx, Txy, Tyy; Txz = Tyz = Tzz = 0
    return mesh, phys, TLb


@pytest.mark.parametrize("model", ["oldroyd_b", "giesekus", "fene_cr", "fene_p"])
def test_linear_in_the_perturbation(model):
    mesh, phys, TLb = _case(model)
    rng = np.random.default_rng(0)
    x, y = rng.standard_normal((2, 10, mesh.nnodes))
    r = [O.stability_elements(phys, mesh.conn, mesh.xyz, TLb, v, 1.5, jacobian=False)
         for v in (x, y, 2 * x - 3 * y, np.zeros_like(x))]
    for q in (0, 1):
        comb = 2 * r[0][q] - 3 * r[1][q]
        assert np.max(np.abs(r[2][q] - comb)) <= 1e-14 * np.max(np.abs(r[2][q]))
        assert np.max(np.abs(r[3][q])) == 0.0


@pytest.mark.parametrize("model", ["oldroyd_b", "fene_cr", "fene_p"])
def test_fd_blocks_are_the_operator(model):
    mesh, phys, TLb = _case(model)
    _, _, A, B = O.stability_elements(phys, mesh.conn, mesh.xyz, TLb, np.zeros((10, mesh.nnodes)),
                                      1.5)
    x = np.random.default_rng(1).standard_normal((10, mesh.nnodes))
    ra, rb, _, _ = O.stability_elements(phys, mesh.conn, mesh.xyz, TLb, x, 1.5, jacobian=False)
    xe = x[:, mesh.element_nodes()].transpose(1, 2, 0)
    assert np.max(np.abs(np.einsum("eiqjr,eiq->ejr", A, xe) - ra)) <= 1e-14 * np.max(np.abs(ra))
    assert np.max(np.abs(np.einsum("eiqjr,eiq->ejr", B, xe) - rb)) <= 1e-14 * np.max(np.abs(rb))


def test_wavenumber_dependence():
    mesh, phys, TLb = _case()
    z = np.zeros((10, mesh.nnodes))

    def AB(k, kz=True):
        return O.stability_elements(phys, mesh.conn, mesh.xyz, TLb, z, k, kz=kz)[2:]
    (A0, B0), (Ap, Bp), (Am, _), (Ak, Bk) = AB(0.0), AB(1.0), AB(-1.0), AB(2.5)
    a1, a2 = (Ap - Am) / 2, (Ap + Am) / 2 - A0
    assert np.max(np.abs(A0 + 2.5 * a1 + 6.25 * a2 - Ak)) <= 1e-13 * np.max(np.abs(Ak))
    assert np.array_equal(B0, Bk) and np.array_equal(B0, Bp)
    assert np.max(np.abs(a2)) > 1e-3 * np.max(np.abs(A0))
    # as written (no z-derivatives): only the momentum equations' 3-D term sees k
    (W0, _), (W1, _) = AB(0.0, kz=False), AB(2.0, kz=False)
    d = W1 - W0
    assert np.max(np.abs(d[..., 3:])) == 0.0
    assert np.max(np.abs(d[..., :3])) > 0.0


def test_spanwise_velocity_decouples_at_k0():
    """At k = 0 the out-of-plane unknowns (Uz, Txz, Tyz) and the in-plane ones
    do not couple: the 2-D base has no z-dependence and no z-velocity."""
    mesh, phys, TLb = _case()
    _, _, A, B = O.stability_elements(phys, mesh.conn, mesh.xyz, TLb, np.zeros((10, mesh.nnodes)),
                                      0.0)
    out = [2, 7, 8]
    inn = [0, 1, 3, 4, 5, 6, 9]
    for M_ in (A, B):
        assert np.max(np.abs(M_[:, :, out][:, :, :, :, inn])) == 0.0
        assert np.max(np.abs(M_[:, :, inn][:, :, :, :, out])) == 0.0


@pytest.mark.parametrize("model", ["fene_cr", "fene_p"])
def test_fene_tends_to_oldroyd_b(model):
    """FENE-CR and FENE-P with extensibility L^2 -> infinity are Oldroyd-B
    (f_T -> 1, its material derivative -> 0): their stability blocks approach
    the Oldroyd-B ones; at L^2 = 40 they differ."""
    mesh, ob, TLb = _case("oldroyd_b")
    _, _, Ao, Bo = O.stability_elements(ob, mesh.conn, mesh.xyz, TLb, np.zeros_like(TLb), 1.5)
    for L2, close in ((1e12, True), (40.0, False)):
        _, fene, _ = _case(model, L2=L2)
        _, _, Af, Bf = O.stability_elements(fene, mesh.conn, mesh.xyz, TLb, np.zeros_like(TLb), 1.5)
        dA = np.max(np.abs(Af - Ao)) / np.max(np.abs(Ao))
        dB = np.max(np.abs(Bf - Bo)) / np.max(np.abs(Bo))
        if close:
            assert dA < 1e-8 and dB < 1e-8
        else:
            assert dA > 1e-4


def test_sqrt_is_rejected():
    mesh, phys, TLb = _case()
    import dataclasses
    with pytest.raises(ValueError):
        O.stability_elements(dataclasses.replace(phys, form="SQRT"), mesh.conn, mesh.xyz, TLb,
                             TLb, 1.0, jacobian=False)
