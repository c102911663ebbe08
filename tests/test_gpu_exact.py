"""Exact (linearised) Jacobian kernels: FP64 and the FP32 precision form.

The exact Jacobian is the derivative the reference's forward difference
approximates, so it is pinned against a Richardson-extrapolated central
difference of the oracle's residual (truncation O(h^4)), compared with the
FD Jacobian (which differs by the FD truncation error, ~1e-8 relative), and
the FP32 kernel against the FP64 one.  The residual returned with an exact
Jacobian is the FP64 residual, bit-identical to the oracle.
Tolerances are relative to the largest Jacobian entry.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    V.load()


def _dense(rowptr, colind, vals):
    return P.dense_from_csr(rowptr, colind, vals.astype(np.float64), len(rowptr) - 1)


def _richardson(phys, mesh, TL, EU, rowptr, colind):
    """Central-difference Jacobian of the oracle residual, Richardson-extrapolated."""
    N = len(rowptr) - 1
    n_dof = mesh.nnodes * 6

    def res(tl, eu):
        b, _ = O.assemble(phys, mesh.conn, mesh.xyz, tl, eu, rowptr, colind, jacobian=False)
        return b

    def cd(h):
        J = np.zeros((N, N))
        for c in range(N):
            tp, tm = TL.copy(), TL.copy()
            ep, em = EU.copy(), EU.copy()
            if c < n_dof:
                tp[c % 6, c // 6] += h
                tm[c % 6, c // 6] -= h
            else:
                ep[0] += h
                em[0] -= h
            J[:, c] = (res(tp, ep) - res(tm, em)) / (2 * h)
        return J
    h = 2e-4
    return (4.0 * cd(h / 2) - cd(h)) / 3.0


CASES = [("L-PTT", 0.0, "T"), ("L-PTT", 0.05, "SQRT"), ("GIESEKUS", 0.1, "T"),
         ("GIESEKUS", 0.1, "SQRT"), ("FENE-P", 40.0, "T"), ("m-e-PTT", 0.05, "SQRT")]


@pytest.mark.parametrize("model,ve,form", CASES)
def test_exact64_matches_richardson_central_difference(model, ve, form):
    mesh = M.rect_mesh(2, 1, 0.0, 1.0, -0.3, 0.4, distort=0.3, seed=4)
    mesh.xyz[0] += 2.0
    phys = S.Physics(model=model, form=form, WiN=0.4, Wi0=0.4, BvN=0.59, VeN=ve, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 12)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    b, v64 = asm.set_equations_bulk(TL, EU, "NRP", jacobian="exact64")
    asm.close()
    bo, _ = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind, jacobian=False)
    assert np.array_equal(b, bo)          # FP64 residual alongside the exact Jacobian
    J = _dense(rowptr, colind, v64)
    Jr = _richardson(phys, mesh, TL, EU, rowptr, colind)
    n_dof = mesh.nnodes * 6
    Jr[n_dof:, :] = 0.0                   # the arclength row is the host's, not the bulk's
    scale = np.max(np.abs(Jr))
    assert np.max(np.abs(J - Jr)) < 1e-7 * scale


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_exact_vs_fd_and_fp32_on_cylinder(form):
    mesh = M.build_cylinder_mesh(2000)
    phys = S.giesekus(0.1, 0.5, 0.59, form, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 3)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    _, vfd = asm.set_equations_bulk(TL, EU, "NRP", jacobian="fd64")
    b64, v64 = asm.set_equations_bulk(TL, EU, "NRP", jacobian="exact64")
    b32, v32 = asm.set_equations_bulk(TL, EU, "NRP", jacobian="exact32")
    asm.close()
    assert v32.dtype == np.float32
    assert np.array_equal(b64, b32)       # the residual stays FP64 in the precision form
    scale = np.max(np.abs(v64))
    assert np.max(np.abs(v64 - vfd)) < 1e-5 * scale     # FD truncation (eps = 1e-8)
    assert np.max(np.abs(v32.astype(np.float64) - v64)) < 2e-5 * scale
    # entries far from the diagonal scale: relative agreement of the bulk of the values
    big = np.abs(v64) > 1e-6 * scale
    rel = np.abs(v32[big] - v64[big]) / np.abs(v64[big])
    assert np.median(rel) < 1e-5


@pytest.mark.parametrize("nel", [2000, 5000])
def test_fp32_jacobian_finite_on_parallel_flow_start(nel):
    """The continuation's starting state (fully developed channel flow with the
    cylinder masked to rest) makes the constitutive residual C vanish up to
    round-off over most of the channel; in FP32 the DCS magnitude
    sqrt(0.5 C:C^T) then sees a negative argument at some Gauss points.  The
    FP32 Jacobian stays finite there and within the FP32 tolerance of the
    FD64 Jacobian."""
    from ve_flow_around_cylinder_fortran_gb300 import newton as N
    mesh = M.build_cylinder_mesh(nel)
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    TL, EU = N.initial_state(mesh, phys)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True)
    _, vfd = asm.set_equations_bulk(TL, EU, "NRP", jacobian="fd64", outlet_edges=True)
    _, v32 = asm.set_equations_bulk(TL, EU, "NRP", jacobian="exact32", outlet_edges=True)
    _, v64 = asm.set_equations_bulk(TL, EU, "NRP", jacobian="exact64", outlet_edges=True)
    asm.close()
    assert np.isfinite(v32).all() and np.isfinite(v64).all()
    scale = np.max(np.abs(vfd))
    # sqrt(0.5 C:C^T) has a kink at C = 0, where the forward difference and the
    # derivative differ by O(|dC/dx|): a looser bound than on generic states
    assert np.max(np.abs(v64 - vfd)) < 1e-4 * scale
    assert np.max(np.abs(v32.astype(np.float64) - vfd)) < 1e-4 * scale
