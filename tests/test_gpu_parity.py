"""GPU parity: the CUDA assembly (through the C ABI) against the CPU oracle.

The FP64 path evaluates the reference's arithmetic in the same order with no
FMA contraction, so the bar is bit-for-bit equality of the element residuals,
the forward-difference Jacobian (differences of residuals divided by 1e-8)
and the element-ordered global sums.  The exponential-PTT models call exp(),
whose last bit may differ between the host libm and CUDA; they are held to
1e-12 relative on the residual and 1e-6 relative on the FD Jacobian instead.
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

EXP_MODELS = ("e-PTT", "m-e-PTT")


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    V.load()


def _compare(model, got, want, what, rel_exp=1e-12):
    if model in EXP_MODELS:
        scale = max(np.max(np.abs(want)), 1e-300)
        assert np.max(np.abs(got - want)) <= rel_exp * scale, what
    else:
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, f"{what}: {bad.size} entries differ, first {bad[:5]}, " \
                              f"max |d| = {np.max(np.abs(got - want)):.3e}"


def _phys(model, form, nex, Wi=0.4, beta=0.59, DfN=0.0):
    ve = {"L-PTT": 0.05, "m-L-PTT": 0.05, "e-PTT": 0.05, "m-e-PTT": 0.05, "FENE-CR": 40.0,
          "FENE-P": 40.0, "GIESEKUS": 0.1}[model]
    return S.Physics(model=model, form=form, WiN=Wi, Wi0=Wi, BvN=beta, VeN=ve, nex=nex, DfN=DfN)


def _case(mesh, phys, seed, flag_nr="NRP", edges=False):
    TL, EU = S.seeded_state(mesh.xyz, phys, seed)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=edges)
    b, vals = asm.set_equations_bulk(TL, EU, flag_nr, outlet_edges=edges)
    bo, vo = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind,
                        jacobian=(flag_nr == "NRP"))
    asm.close()
    return TL, EU, rowptr, colind, b, vals, bo, vo


MODELS = ["L-PTT", "m-L-PTT", "e-PTT", "m-e-PTT", "FENE-CR", "FENE-P", "GIESEKUS"]


@pytest.mark.parametrize("form", ["T", "SQRT"])
@pytest.mark.parametrize("model", MODELS)
def test_small_mesh_all_models_bitwise(model, form):
    mesh = M.rect_mesh(3, 2, 0.0, 1.5, -0.4, 0.6, distort=0.25, seed=7)
    mesh.xyz[0] += 2.0      # keep the mask away from zero velocity
    phys = _phys(model, form, nex=1)
    _, _, _, _, b, vals, bo, vo = _case(mesh, phys, seed=11)
    _compare(model, b, bo, "residual")
    _compare(model, vals, vo, "jacobian", rel_exp=1e-6)


@pytest.mark.parametrize("nex", [0, 1])
@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_cylinder_2000_oldroyd_b_bitwise(form, nex):
    """2,000-element Oldroyd-B case (beta = 0.59, Wi = 0.1) in both forms."""
    mesh = M.build_cylinder_mesh(2000)
    phys = S.oldroyd_b(0.1, 0.59, form, nex=nex)
    _, _, _, _, b, vals, bo, vo = _case(mesh, phys, seed=0)
    _compare("L-PTT", b, bo, "residual")
    _compare("L-PTT", vals, vo, "jacobian")


def test_residual_only_matches():
    """'MNR' (residual only) uses the per-Gauss-point kernel; same bits."""
    mesh = M.build_cylinder_mesh(2000)
    for form in ("T", "SQRT"):
        phys = S.giesekus(0.1, 0.5, 0.59, form, nex=1)
        _, _, _, _, b, _, bo, _ = _case(mesh, phys, seed=2, flag_nr="MNR")
        _compare("GIESEKUS", b, bo, f"residual {form}")


def test_dfn_positive_disables_dcs():
    mesh = M.build_cylinder_mesh(2000)
    phys = S.oldroyd_b(0.1, 0.59, "T", nex=1, DfN=1.0e-3)
    _, _, _, _, b, vals, bo, vo = _case(mesh, phys, seed=3)
    _compare("L-PTT", b, bo, "residual")
    _compare("L-PTT", vals, vo, "jacobian")


def test_restore_residue_state():
    """States whose (x+eps)-eps is not x (tiny values, values just below powers
    of two) exercise the restore-residue staging of later FD columns."""
    mesh = M.rect_mesh(2, 2, 0.0, 1.0, 0.0, 1.0, distort=0.3, seed=1)
    mesh.xyz[0] += 2.0
    phys = S.giesekus(0.1, 0.5, 0.59, "T", nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 5)
    TL[2, ::3] = 3.0e-13
    TL[4, ::4] = 0.5 - 4.0e-9
    TL[0, 1::5] = -1.0 + 3.0e-9
    assert np.count_nonzero(((TL + 1e-8) - 1e-8) != TL) > 5
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    b, vals = asm.set_equations_bulk(TL, EU, "NRP")
    bo, vo = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind)
    _compare("GIESEKUS", b, bo, "residual")
    _compare("GIESEKUS", vals, vo, "jacobian")


def test_add_semantics_and_determinism():
    """ADD_VALUES onto existing values, and two runs are bit-identical."""
    mesh = M.build_cylinder_mesh(2000)
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 9)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    rng = np.random.default_rng(0)
    b0 = rng.normal(size=len(rowptr) - 1)
    v0 = rng.normal(size=len(colind))
    b1, v1 = asm.set_equations_bulk(TL, EU, "NRP", b=b0.copy(), vals=v0.copy())
    b2, v2 = asm.set_equations_bulk(TL, EU, "NRP", b=b0.copy(), vals=v0.copy())
    assert np.array_equal(b1, b2) and np.array_equal(v1, v2)
    bo, vo = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind, b=b0.copy(),
                        vals=v0.copy())
    _compare("L-PTT", b1, bo, "residual (add)")
    _compare("L-PTT", v1, vo, "jacobian (add)")
    # zero-first equals a fresh assembly
    b3, v3 = asm.set_equations_bulk(TL, EU, "NRP", b=b0.copy(), vals=v0.copy(), zero_first=True)
    bz, vz = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind)
    _compare("L-PTT", b3, bz, "residual (zero first)")
    _compare("L-PTT", v3, vz, "jacobian (zero first)")
    asm.close()


@pytest.mark.parametrize("jac", ["fd64", "exact32"])
def test_zero_first_with_entries_outside_element_blocks(jac):
    """A caller's pattern may hold node-row entries no element block covers
    (here: the six columns of a distant node in the rows of node 0).  With
    VEFEM_ZERO_FIRST they come back zero and every other entry equals the
    assembly on the plain pattern, whatever the arrays held before."""
    mesh = M.build_cylinder_mesh(2000)
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 4)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    far = mesh.nnodes - 1
    assert far * 6 not in set(colind[rowptr[0]:rowptr[1]])
    rows = [list(colind[rowptr[r]:rowptr[r + 1]]) for r in range(len(rowptr) - 1)]
    for r in range(6):
        rows[r] = sorted(rows[r] + [far * 6 + q for q in range(6)])
    rp2 = np.concatenate([[0], np.cumsum([len(c) for c in rows])]).astype(rowptr.dtype)
    ci2 = np.concatenate(rows).astype(colind.dtype)
    rng = np.random.default_rng(1)
    out = {}
    for name, (rp, ci) in (("plain", (rowptr, colind)), ("extra", (rp2, ci2))):
        asm = V.BulkAssembler(mesh, phys, rp, ci)
        b0 = rng.normal(size=len(rp) - 1)
        v0 = rng.normal(size=len(ci)).astype(np.float64 if jac == "fd64" else np.float32)
        b, v = asm.set_equations_bulk(TL, EU, "NRP", b=b0, vals=v0, zero_first=True, jacobian=jac)
        asm.close()
        out[name] = (rp, ci, b, v)
    _, _, bp, vp = out["plain"]
    _, _, be, ve = out["extra"]
    assert np.array_equal(bp, be)
    extra = np.zeros(len(ci2), dtype=bool)
    for r in range(6):
        cols = ci2[rp2[r]:rp2[r + 1]]
        extra[rp2[r]:rp2[r + 1]] = (cols >= far * 6) & (cols < far * 6 + 6)
    assert np.all(ve[extra] == 0)
    assert np.array_equal(ve[~extra], vp)


@pytest.mark.parametrize("form", ["T", "SQRT"])
def test_outlet_edges_after_bulk(form):
    """Outlet open-BC edges (setEquationsEdge) added after the bulk, in edge order."""
    mesh = M.build_cylinder_mesh(2000)
    phys = S.giesekus(0.1, 0.5, 0.59, form, nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 6)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True)
    b, vals = asm.set_equations_bulk(TL, EU, "NRP", outlet_edges=True)
    bo, vo = O.assemble(phys, mesh.conn, mesh.xyz, TL, EU, rowptr, colind)
    en = mesh.element_nodes()
    N = len(rowptr) - 1
    for e, ied in mesh.outlet_edges:
        r, jac, ac = O.edge_open(phys, mesh.conn, mesh.xyz, TL, EU, e, ied)
        g = en[e]
        for jnod in range(9):
            for jeq in range(6):
                row = g[jnod] * 6 + jeq
                bo[row] = bo[row] + r[jnod, jeq]
        for jnod in range(9):
            for jeq in range(6):
                row = g[jnod] * 6 + jeq
                cols = colind[rowptr[row]:rowptr[row + 1]]
                for inod in range(9):
                    for ieq in range(6):
                        s = rowptr[row] + np.searchsorted(cols, g[inod] * 6 + ieq)
                        vo[s] = vo[s] + jac[inod, ieq, jnod, jeq]
                s = rowptr[row + 1] - 1
                assert colind[s] == N - 1
                vo[s] = vo[s] + ac[jnod, jeq, 0]
    _compare("GIESEKUS", b, bo, "residual with edges")
    _compare("GIESEKUS", vals, vo, "jacobian with edges")
    asm.close()


def test_device_pointers_match_host_path():
    torch = pytest.importorskip("torch")
    mesh = M.build_cylinder_mesh(2000)
    phys = S.giesekus(0.1, 0.5, 0.59, "SQRT", nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, 1)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind)
    bh, vh = asm.set_equations_bulk(TL, EU, "NRP")
    dev = torch.device("cuda:0")
    tTL = torch.from_numpy(TL).to(dev)
    tEU = torch.from_numpy(EU).to(dev)
    tb = torch.zeros(len(rowptr) - 1, dtype=torch.float64, device=dev)
    tv = torch.zeros(len(colind), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    asm.assemble(tTL, tEU, V.VEFEM_RESIDUAL | V.VEFEM_JAC_FD64, tb, tv, on_device=True)
    assert np.array_equal(tb.cpu().numpy(), bh)
    assert np.array_equal(tv.cpu().numpy(), vh)
    assert asm.last_launch_count() == 4
    asm.close()


@pytest.mark.slow
def test_cylinder_40000_giesekus_sqrt_bitwise():
    """40,000 elements, Giesekus alpha = 0.1, beta = 0.59, Wi = 0.5, SQRT form."""
    mesh = M.build_cylinder_mesh(40000)
    phys = S.giesekus(0.1, 0.5, 0.59, "SQRT", nex=1)
    _, _, _, _, b, vals, bo, vo = _case(mesh, phys, seed=0)
    _compare("GIESEKUS", b, bo, "residual")
    _compare("GIESEKUS", vals, vo, "jacobian")


@pytest.mark.parametrize("form", ["T", "SQRT"])
@pytest.mark.parametrize("DfN", [0.0, 1.0e-3])
def test_reynolds_nonzero(form, DfN):
    """Re > 0 and DfN > 0 take the kernel variants that keep the convection,
    LSME-momentum and diffusion terms (the Re = 0 / DfN = 0 variants drop them)."""
    mesh = M.build_cylinder_mesh(2000)
    phys = S.Physics(model="GIESEKUS", form=form, ReN=0.7, WiN=0.5, Wi0=0.5, BvN=0.59, VeN=0.1,
                     nex=1, DfN=DfN)
    _, _, _, _, b, vals, bo, vo = _case(mesh, phys, seed=8)
    _compare("GIESEKUS", b, bo, "residual")
    _compare("GIESEKUS", vals, vo, "jacobian")
