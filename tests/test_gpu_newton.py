"""Newton-Raphson on the GPU assembly (host driver restating loopNewtonRaphson,
host SuperLU standing in for MUMPS), Dirichlet rows applied on the device.

* FD64 Jacobian: every iterate equals the oracle-driven Newton's bit for bit
  (same residual and Jacobian bits, same deterministic factorisation);
* exact FP64 and the FP32 precision form (FP64 residual, FP32 Jacobian,
  inexact Newton) reach ||R|| < 1e-10 and the same solution within 1e-8
  relative.
"""
import numpy as np
import pytest

from oracle_assembly import OracleAssembly
from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import newton as N
from ve_flow_around_cylinder_fortran_gb300 import pattern as P
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    V.load()


def _setup(nel, phys):
    mesh = M.build_cylinder_mesh(nel)
    TL, EU = N.initial_state(mesh, phys)
    rows, values = N.boundary_conditions(mesh, phys)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    return mesh, TL, EU, rows, values, rowptr, colind


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_gpu_newton_equals_oracle_newton(form):
    phys = S.oldroyd_b(0.1, 0.59, form, nex=0)
    mesh, TL, EU, rows, values, rowptr, colind = _setup(500, phys)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True)
    gpu = N.NewtonRaphson(N.DeviceAssembly(asm, rows, values, "fd64"), rowptr, colind, 0)
    r1 = gpu.solve(TL, EU, tol=1e-10)
    asm.close()
    cpu = N.NewtonRaphson(OracleAssembly(phys, mesh, rowptr, colind, rows, values), rowptr,
                          colind, 0)
    r2 = cpu.solve(TL, EU, tol=1e-10)
    assert r1.converged and r2.converged
    assert r1.iterations == r2.iterations
    assert [h["res_norm"] for h in r1.history] == [h["res_norm"] for h in r2.history]
    assert np.array_equal(r1.TL, r2.TL)


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_precision_form_converges_to_fp64_solution(form):
    """Giesekus alpha = 0.1, beta = 0.59 up to Wi = 0.5 by natural continuation
    (Wi = 0.1, 0.3, 0.5), with each Jacobian."""
    phys = S.giesekus(0.1, 0.1, 0.59, form, nex=0)
    mesh, TL, EU, rows, values, rowptr, colind = _setup(500, phys)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True)
    out = {}
    for jac in ("fd64", "exact64", "exact32"):
        res = N.natural_continuation(asm, mesh, phys, [0.1, 0.3, 0.5], jacobian=jac, tol=1e-10)
        out[jac] = res[-1]
        assert all(r.converged for r in res), jac
        assert out[jac].history[-1]["res_norm"] < 1e-10
    asm.close()
    ref = out["fd64"].TL
    for jac in ("exact64", "exact32"):
        err = np.linalg.norm(out[jac].TL - ref) / np.linalg.norm(ref)
        assert err < 1e-8, (jac, err)


def test_device_and_host_dirichlet_agree():
    torch = pytest.importorskip("torch")
    phys = S.oldroyd_b(0.1, 0.59, "T", nex=1)
    mesh, TL, EU, rows, values, rowptr, colind = _setup(500, phys)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    b, vals = asm.set_equations_bulk(TL, EU, "NRP")
    bh, vh = b.copy(), vals.copy()
    asm.apply_dirichlet(rows, values, TL, bh, vh, V.VEFEM_RESIDUAL | V.VEFEM_JAC_FD64)
    d = torch.device("cuda:0")
    tb, tv = torch.from_numpy(b).to(d), torch.from_numpy(vals).to(d)
    asm.apply_dirichlet(torch.from_numpy(rows).to(d), torch.from_numpy(values).to(d),
                        torch.from_numpy(TL).to(d), tb, tv, V.VEFEM_RESIDUAL | V.VEFEM_JAC_FD64,
                        on_device=True, nrows=len(rows))
    torch.cuda.synchronize()
    assert np.array_equal(tb.cpu().numpy(), bh)
    assert np.array_equal(tv.cpu().numpy(), vh)
    # the Dirichlet rows: b = TL - g, a unit row
    r = rows[5]
    assert bh[r] == TL[r % 6, r // 6] - values[5]
    row = vh[rowptr[r]:rowptr[r + 1]]
    assert row.sum() == 1.0 and row[np.searchsorted(colind[rowptr[r]:rowptr[r + 1]], r)] == 1.0
    asm.close()
