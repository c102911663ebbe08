"""Exact (linearised) Jacobian kernels: FP64 and the FP32 precision form.

The exact Jacobian is the derivative the reference's forward difference
approximates.  It is pinned against the oracle's complex-step Jacobian
(oracle/vefem_oracle.c on complex numbers: exact to rounding) at <= 1e-12
relative in FP64 on the 2,000-quad mesh for every model and form, in FP32
within its rounding, and for the batched kernel instance by instance; also
against a Richardson-extrapolated central difference of the oracle's
residual, the FD Jacobian (which differs by the FD truncation error, ~1e-8
relative), and the FP32 kernel against the FP64 one.  The residual returned with an exact
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


MODELS7 = [("L-PTT", 0.05), ("m-L-PTT", 0.05), ("e-PTT", 0.05), ("m-e-PTT", 0.05),
           ("FENE-CR", 40.0), ("FENE-P", 40.0), ("GIESEKUS", 0.1)]


@pytest.mark.parametrize("form", ["T", "SQRT"])
@pytest.mark.parametrize("model,ve", MODELS7)
def test_exact64_matches_complex_step_oracle_2000(model, ve, form):
    """FP64 exact Jacobian on the 2,000-quad cylinder mesh against the
    oracle's complex-step Jacobian: <= 1e-12 relative (max-norm of the
    difference over max-norm of the matrix), every model and both forms.
    The residual is bit-identical, except for the exponential-PTT models
    (1e-12 relative: exp() of the host and of CUDA may differ in the last
    bit)."""
    mesh = M.build_cylinder_mesh(2000)
    phys = S.Physics(model=model, form=form, WiN=0.3, Wi0=0.3, BvN=0.59, VeN=ve, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 5)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    b, v64 = asm.set_equations_bulk(TL, EU, "NRP", jacobian="exact64")
    asm.close()
    bo, vo = O.exact_assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind)
    if model in ("e-PTT", "m-e-PTT"):
        # host libm and CUDA exp() may differ in the last bit
        assert np.max(np.abs(b - bo)) <= 1e-12 * np.max(np.abs(bo))
    else:
        assert np.array_equal(b, bo)
    assert np.max(np.abs(v64 - vo)) <= 1e-12 * np.max(np.abs(vo))


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_exact32_matches_complex_step_oracle_2000(form):
    """FP32 exact Jacobian (the precision form) against the complex-step
    oracle: max-norm error <= 1e-5 relative to the largest entry, and the
    median relative error of the entries above 1e-6 of it <= 2e-6 (FP32
    unit roundoff 6e-8 times the depth of the Gauss and element sums)."""
    mesh = M.build_cylinder_mesh(2000)
    phys = S.giesekus(0.1, 0.5, 0.59, form, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 3)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    b32, v32 = asm.set_equations_bulk(TL, EU, "NRP", jacobian="exact32")
    asm.close()
    bo, vo = O.exact_assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind)
    assert np.array_equal(b32, bo)
    scale = np.max(np.abs(vo))
    err = np.max(np.abs(v32.astype(np.float64) - vo)) / scale
    big = np.abs(vo) > 1e-6 * scale
    med = np.median(np.abs(v32[big] - vo[big]) / np.abs(vo[big]))
    print(f"exact32 vs complex step ({form}): max {err:.3e}, median {med:.3e}")
    assert err <= 1e-5
    assert med <= 2e-6


@pytest.mark.parametrize("jac", ["exact64", "exact32"])
def test_batched_exact_matches_complex_step_oracle(jac):
    """Three instances of uneven size in one batched launch, each against the
    complex-step oracle directly (not against the single-mesh kernel)."""
    import torch
    f32 = jac == "exact32"
    insts = []
    for k, (n, wi) in enumerate(zip([300, 1200, 700], [0.2, 0.6, 0.9])):
        mesh = M.build_cylinder_mesh(n, exact=False)
        phys = S.giesekus(0.1, wi, 0.59, "SQRT", nex=1)
        TL, EU = S.seeded_state(mesh.xyz, phys, seed=20 + k)
        rp, ci = V.build_pattern(mesh.conn, mesh.nnodes, 1)
        insts.append((mesh, phys, (rp, ci), TL, EU))
    bt = V.BatchAssembler([i[0] for i in insts], [i[1] for i in insts], [i[2] for i in insts])
    d = torch.device("cuda:0")
    bs = [torch.zeros(len(i[2][0]) - 1, dtype=torch.float64, device=d) for i in insts]
    vs = [torch.zeros(len(i[2][1]), dtype=torch.float32 if f32 else torch.float64, device=d)
          for i in insts]
    bt.assemble([torch.from_numpy(i[3]).to(d) for i in insts],
                [torch.from_numpy(i[4]).to(d) for i in insts],
                V.VEFEM_RESIDUAL | V.JACOBIANS[jac] | V.VEFEM_ZERO_FIRST, bs, vs, on_device=True)
    bt.close()
    tol = 1e-5 if f32 else 1e-12
    for k, (mesh, phys, (rp, ci), TL, EU) in enumerate(insts):
        bo, vo = O.exact_assemble(phys, mesh.conn, mesh.xyz, TL, EU, rp, ci)
        assert np.array_equal(bs[k].cpu().numpy(), bo), k
        v = vs[k].cpu().numpy().astype(np.float64)
        assert np.max(np.abs(v - vo)) <= tol * np.max(np.abs(vo)), k
