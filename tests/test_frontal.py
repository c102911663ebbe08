"""Panel-frontal LU (frontal.py) on the CPU device of torch: solves against
scipy's, the symbolic phase's invariants, the border (arclength) unknown,
device tensors in and out, and the host fallback on a zero pivot."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from ve_flow_around_cylinder_fortran_gb300 import frontal as FR
from test_linsolve import _jacobian

torch = pytest.importorskip("torch")


def _bordered(nel, nex, seed=0):
    mesh, rp, ci, v, b = _jacobian(nel, nex)
    N = len(rp) - 1
    if nex:
        # a dense lambda row, as the arclength equation t . (x - x_o) - dS
        r0, r1 = rp[N - 1], rp[N]
        v[r0:r1] = np.random.default_rng(seed).standard_normal(r1 - r0)
    return mesh, rp, ci, v, b, sp.csr_matrix((v, ci, rp), shape=(N, N))


@pytest.mark.parametrize("nex", [0, 1])
@pytest.mark.parametrize("panel", [None, 3, 11, 60])
def test_frontal_matches_scipy(nex, panel):
    mesh, rp, ci, v, b, A = _bordered(200, nex)
    x_ref = spla.spsolve(A.tocsc(), b)
    lu = FR.FrontalLU(rp, ci, mesh, panel=panel, device="cpu").factor(v)
    x = lu.solve(b)
    assert lu.fallbacks == 0
    assert np.linalg.norm(x - x_ref) <= 1e-9 * np.linalg.norm(x_ref)
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(b)
    # a second right-hand side with the same factorisation, within the
    # solver's own residual check
    b2 = np.random.default_rng(1).standard_normal(len(b))
    assert np.linalg.norm(A @ lu.solve(b2) - b2) <= lu.check_tol * np.linalg.norm(b2)


@pytest.mark.parametrize("nex", [0, 1])
def test_delayed_pressures_match_scipy(nex):
    """The fallback ordering (every pressure eliminated with the last panel
    that touches one of its element-mates) solves the same system."""
    mesh, rp, ci, v, b, A = _bordered(200, nex)
    x_ref = spla.spsolve(A.tocsc(), b)
    plain = FR.FrontalLU(rp, ci, mesh, panel=5, device="cpu")
    lu = FR.FrontalLU(rp, ci, mesh, panel=5, device="cpu", delay_pressure=True).factor(v)
    assert lu.f_sz.mean() > plain.f_sz.mean()          # the pressures stay in the fronts longer
    x = lu.solve(b)
    assert np.linalg.norm(x - x_ref) <= 1e-9 * np.linalg.norm(x_ref)
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(b)


@pytest.mark.parametrize("delay", [False, True])
def test_symbolic_phase_invariants(delay):
    mesh, rp, ci, v, b, A = _bordered(120, 1)
    lu = FR.FrontalLU(rp, ci, mesh, panel=4, device="cpu", delay_pressure=delay)
    N = len(rp) - 1
    piv = np.concatenate([p.numpy() for p in lu.idxP])
    # every unknown is eliminated exactly once; the border with the last panel
    assert np.array_equal(np.sort(piv), np.arange(N))
    assert N - 1 in lu.idxP[-1].numpy()
    for q in range(lu.npan - 1):
        assert lu.idxF[q].numpy()[-1] == N - 1
    # every CSR entry has its own place in one frontal matrix
    dest = lu.dest.numpy()
    assert len(np.unique(dest)) == len(dest) == len(ci)
    assert dest.min() >= 0 and dest.max() < lu.off[-1]
    # the front after panel q reaches panel q + 1 only through its pivots or front
    for q in range(lu.npan - 1):
        nxt = set(lu.idxP[q + 1].numpy()) | set(lu.idxF[q + 1].numpy())
        assert set(lu.idxF[q].numpy()) <= nxt


def test_device_tensors_in_and_out():
    mesh, rp, ci, v, b, A = _bordered(100, 1)
    lu = FR.FrontalLU(rp, ci, mesh, device="cpu").factor(torch.from_numpy(v).float())
    x = lu.solve(torch.from_numpy(b))
    assert isinstance(x, torch.Tensor)
    A32 = sp.csr_matrix((v.astype(np.float32).astype(np.float64), ci, rp), shape=A.shape)
    assert np.linalg.norm(A32 @ x.numpy() - b) <= 1e-12 * np.linalg.norm(b)


def test_zero_pivot_falls_back_to_host():
    """A row that is zero except in the border column makes one panel's pivot
    block exactly singular while the bordered matrix is not: the factorisation
    is handed to the host SuperLU and the solve stays exact."""
    mesh, rp, ci, v, b, A = _bordered(80, 1)
    N = len(rp) - 1
    k = int(mesh.boundary_nodes["Wall"][3]) * 6      # a unit (Dirichlet-like) row
    s0, s1 = rp[k], rp[k + 1]
    v[s0:s1] = (ci[s0:s1] == N - 1).astype(float)
    A = sp.csr_matrix((v, ci, rp), shape=(N, N))
    lu = FR.FrontalLU(rp, ci, mesh, panel=4, device="cpu").factor(v)
    x = lu.solve(b)
    assert lu.fallbacks == 1
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)


def test_krylov_correction_with_device_tensors():
    """The Newton-Krylov correction of the continuation driver on device
    tensors (torch's CPU device here): GMRES with the Jacobian as a torch CSR
    matrix, preconditioned by the frontal factorisation of a perturbed
    matrix (an older Jacobian), solves to its tolerance; the preconditioner
    alone does not."""
    import types

    from ve_flow_around_cylinder_fortran_gb300 import continuation as C
    mesh, rp, ci, v, b, A = _bordered(200, 1)
    old = v * (1.0 + 0.02 * np.random.default_rng(3).standard_normal(len(v)))
    lu = FR.FrontalLU(rp, ci, mesh, device="cpu").factor(old)
    cont = types.SimpleNamespace(cfg=C.ArclengthSettings(krylov=20, krylov_rtol=1e-8),
                                 lrow=types.SimpleNamespace(rowptr=rp, colind=ci),
                                 N=len(rp) - 1, krylov_iterations=0, krylov_failures=0,
                                 last_krylov_its=0)
    s = C.ArclengthContinuation._krylov_solve(cont, lu, torch.from_numpy(v), b)
    assert s is not None and cont.krylov_iterations > 1
    assert np.linalg.norm(A @ s - b) <= 1e-7 * np.linalg.norm(b)
    assert np.linalg.norm(A @ lu.solve(b) - b) > 1e-4 * np.linalg.norm(b)
    # a tolerance GMRES cannot reach in the iterations allowed: no correction
    cont.cfg = C.ArclengthSettings(krylov=1, krylov_rtol=1e-14)
    assert C.ArclengthContinuation._krylov_solve(cont, lu, torch.from_numpy(v), b) is None
    assert cont.krylov_failures == 1
