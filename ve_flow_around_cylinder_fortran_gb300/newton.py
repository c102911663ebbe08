"""Newton-Raphson host driver over the GPU assembly.

Restates the reference's nonlinear loop for the Cylinder_2D problem so the
assembly can be exercised the way the Fortran host uses it:

* loopNewtonRaphson (Newton_Raphson_mod.F90:21-172): iterate while the last
  correction norm or the last residual norm is above tolerance, assemble
  ('NRP' with a Jacobian, 'MNR' reusing the last factorisation), solve,
  update; every 10th iteration is a full 'NRP';
* checkNewtonConvergence (:453-529): NaN stop, 'NRP' -> 'MNR' when the
  correction norm drops below MNR_eps = 0.1, 'MNR' -> 'NRP' when it grows;
  divergence above Cor_Norm_div = 1e8 or more than Niter = 50 iterations;
* updateNewton (:619-680): TL -= xF s, EU -= xF s;
* boundary rows after assembly, applyDirichletBC and
  applyDirichletBCFullyDeveloped (Dirichlet_mod.F90:104-192), through
  vefem_apply_dirichlet on the device; boundary equations per
  setBoundaryEQs (Boundary_mod.F90:202-317): inlet fully developed
  (u, v and the stresses), outlet p = 0, walls and cylinder u = v = 0.

The linear solve is the host stand-in for PETSc/MUMPS: SuperLU (scipy) on
the AIJ matrix in FP64 (an FP32 Jacobian is widened before factorisation,
the inexact-Newton precision form), in a nested-dissection order of the
mesh when the mesh is given (linsolve.py).

Fully developed inflow: u = 1.5 (1 - (y/H)^2), v = 0, and the stresses of
steady homogeneous shear at the local shear rate, which is the exact
fully developed state for Oldroyd-B; for the other models it is the
pointwise shear solution on the parabolic profile (the reference solves a
separate 1-D inflow problem, out of scope here).
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import linsolve as LS
from . import state as S
from . import vefem as V

NITER = 50
MNR_EPS = 1.0e-1
COR_NORM_DIV = 1.0e8


def _shear_conformation(phys: S.Physics, gdot: np.ndarray) -> np.ndarray:
    """c [n,2,2] of steady homogeneous shear u = gdot*y: solves
    -Wi (L c + c L^T) + F(c) = 0 with L = [[0, gdot], [0, 0]]."""
    Wi = phys.WiN
    n = gdot.shape[0]
    out = np.empty((n, 2, 2))
    for i, g in enumerate(gdot):
        if phys.model == "L-PTT" and phys.VeN == 0.0:
            # Oldroyd-B, closed form
            c = np.array([[1.0 + 2.0 * (Wi * g) ** 2, Wi * g], [Wi * g, 1.0]])
        else:
            c = _solve_shear_point(phys, g)
        out[i] = c
    return out


def _solve_shear_point(phys: S.Physics, g: float) -> np.ndarray:
    Wi, eps = phys.WiN, phys.VeN
    I = np.eye(2)
    L = np.array([[0.0, g], [0.0, 0.0]])

    def F(c):
        tr = c[0, 0] + c[1, 1]
        if phys.model in ("L-PTT", "m-L-PTT"):
            return (1.0 + eps * (tr - 2.0)) * (c - I)
        if phys.model in ("e-PTT", "m-e-PTT"):
            return np.exp(eps * (tr - 2.0)) * (c - I)
        if phys.model == "GIESEKUS":
            return (c - I) + eps * (c - I) @ (c - I)
        if phys.model == "FENE-CR":
            return (eps - 2.0) / (eps - tr) * (c - I)
        return (eps - 2.0) / (eps - tr) * c - I     # FENE-P

    v = np.array([1.0 + 2.0 * (Wi * g) ** 2, Wi * g, 1.0])
    for _ in range(60):
        def res(v):
            c = np.array([[v[0], v[1]], [v[1], v[2]]])
            r = -Wi * (L @ c + c @ L.T) + F(c)
            return np.array([r[0, 0], r[0, 1], r[1, 1]])
        r = res(v)
        if np.max(np.abs(r)) < 1e-15:
            break
        J = np.zeros((3, 3))
        for k in range(3):
            dv = np.zeros(3)
            dv[k] = 1e-7
            J[:, k] = (res(v + dv) - res(v - dv)) / 2e-7
        v = v - np.linalg.solve(J, r)
    return np.array([[v[0], v[1]], [v[1], v[2]]])


def inflow_profile(y: np.ndarray, phys: S.Physics, H: float = 2.0) -> np.ndarray:
    """[6, n] fully developed unknowns at heights y (p left at 0)."""
    u = 1.5 * (1.0 - (y / H) ** 2)
    du = -3.0 * y / H ** 2
    out = np.zeros((6, y.shape[0]))
    out[0] = u
    out[3:] = S.conformation_to_unknowns(_shear_conformation(phys, du), phys)
    return out


def boundary_conditions(mesh, phys: S.Physics):
    """Dirichlet (rows, values): inlet u, v, stresses; outlet p = 0; walls and
    cylinder u = v = 0, applied in the reference's order (inlet first, then
    Outlet, Wall, Cylinder); a row named twice keeps its last value."""
    bn = mesh.boundary_nodes
    rows, vals = [], []
    inlet = bn["Inlet"]
    prof = inflow_profile(mesh.xyz[1][inlet], phys)
    for f in (0, 1, 3, 4, 5):
        rows.append(inlet * 6 + f)
        vals.append(prof[f])
    out = bn["Outlet"]
    rows.append(out * 6 + 2)
    vals.append(np.zeros(out.size))
    for name in ("Wall", "Cylinder"):
        nodes = bn[name]
        for f in (0, 1):
            rows.append(nodes * 6 + f)
            vals.append(np.zeros(nodes.size))
    rows = np.concatenate(rows).astype(np.int64)
    vals = np.concatenate(vals)
    last = {}
    for i, r in enumerate(rows):
        last[int(r)] = i
    keep = np.array(sorted(last.values()))
    return np.ascontiguousarray(rows[keep]), np.ascontiguousarray(vals[keep])


def initial_state(mesh, phys: S.Physics, R: float = 1.0, H: float = 2.0):
    """Fully developed inflow profile over the whole channel, velocity and
    polymer stress masked to rest near the cylinder, and the Poiseuille
    pressure gradient of the total viscosity (the starting point for the
    lowest Wi of a continuation)."""
    x, y = mesh.xyz[0], mesh.xyz[1]
    r = np.hypot(x, y)
    mask = np.clip((r - R) / 0.5, 0.0, 1.0)
    TL = inflow_profile(y, phys, H)
    TL[0] *= mask
    x_out = float(mesh.params.get("x_out", np.max(x)))
    TL[2] = 3.0 / H ** 2 * (x_out - x)
    rest = S.conformation_to_unknowns(np.repeat(np.eye(2)[None], x.shape[0], axis=0), phys)
    TL[3:] = rest + (TL[3:] - rest) * mask
    EU = np.ones(phys.nex)
    if phys.nex:
        phys.Wi0 = phys.WiN
    return np.ascontiguousarray(TL), EU


@dataclasses.dataclass
class NewtonResult:
    TL: np.ndarray
    EU: np.ndarray
    converged: bool
    iterations: int
    history: list
    assembly_s: float
    solve_s: float


class DeviceAssembly:
    """Residual, Jacobian and Dirichlet rows on the GPU, results on the host."""

    def __init__(self, asm: V.BulkAssembler, rows: np.ndarray, values: np.ndarray,
                 jacobian: str = "fd64", outlet_edges: bool = True):
        import torch
        # True: the AIJ values stay on the device (FP64) for a device solver
        self.device_values = False
        self.torch = torch
        self.asm = asm
        self.jacobian = jacobian
        self.jflag = V.JACOBIANS[jacobian]
        self.edges = outlet_edges
        d = torch.device(f"cuda:{asm.device}")
        self.dev = d
        self.rows = torch.from_numpy(rows).to(d)
        self.values = torch.from_numpy(values).to(d)
        self.nrows = int(rows.shape[0])
        self.b = torch.zeros(asm.N, dtype=torch.float64, device=d)
        vdt = torch.float32 if jacobian == "exact32" else torch.float64
        self.vals = torch.zeros(asm.nnz, dtype=vdt, device=d)

    def set_values(self, values: np.ndarray):
        """New Dirichlet values for the same rows (the inflow profile follows Wi)."""
        self.values = self.torch.from_numpy(np.ascontiguousarray(values)).to(self.dev)

    def __call__(self, TL: np.ndarray, EU: np.ndarray, want_jac: bool):
        torch = self.torch
        tTL = torch.from_numpy(np.ascontiguousarray(TL)).to(self.dev)
        tEU = torch.from_numpy(np.ascontiguousarray(EU if len(EU) else np.zeros(1))).to(self.dev)
        flags = V.VEFEM_RESIDUAL | V.VEFEM_ZERO_FIRST
        if want_jac:
            flags |= self.jflag
        if self.edges:
            flags |= V.VEFEM_OUTLET_EDGES
        torch.cuda.synchronize()
        self.asm.assemble(tTL, tEU, flags, self.b, self.vals if want_jac else None, on_device=True)
        dflags = V.VEFEM_RESIDUAL | (self.jflag if want_jac else 0)
        self.asm.apply_dirichlet(self.rows, self.values, tTL, self.b,
                                 self.vals if want_jac else None, dflags, on_device=True,
                                 nrows=self.nrows)
        b = self.b.cpu().numpy()
        if not want_jac:
            return b, None
        if self.device_values:
            return b, self.vals.to(torch.float64)
        return b, self.vals.cpu().numpy().astype(np.float64)


def emergency_solve(newton, TL, EU, log=None, max_restarts=None, **kw):
    """emergencyNewtonRaphson (Newton_Raphson_mod.F90:533-584): on divergence
    restart from the same state with the relaxation factor halved and
    50 x Niter iterations allowed, until xF < 1e-2 (or after ``max_restarts``
    restarts, when given)."""
    xF = kw.pop("xF", 1.0)
    res = newton.solve(TL, EU, xF=xF, log=log, **kw)
    restarts = 0
    while not res.converged:
        xF = xF / 2.0
        if xF < 1.0e-2 or (max_restarts is not None and restarts >= max_restarts):
            return res
        restarts += 1
        if log:
            log(f"restarting with relaxation xF = {xF}")
        kw["max_iter"] = 50 * NITER
        res = newton.solve(TL, EU, xF=xF, log=log, **kw)
    return res


def extrapolate(wis_done, TLs, wi: float) -> np.ndarray:
    """Start of the next natural-continuation point: the Lagrange polynomial
    in Wi through the last (up to three) converged states, evaluated at
    ``wi`` -- the reference's transient predictor (updateSolutionTransient,
    Continuation_Transient_mod.F90:188-243: TLp = Lb TLb + Lo TLo + L TL)
    with Wi in place of time."""
    w = list(wis_done[-3:])
    X = list(TLs[-3:])
    out = np.zeros_like(X[-1])
    for i in range(len(w)):
        c = 1.0
        for j in range(len(w)):
            if j != i:
                c *= (wi - w[j]) / (w[i] - w[j])
        out += c * X[i]
    return out


def natural_continuation(asm, mesh, phys: S.Physics, wis, jacobian: str = "fd64",
                         tol: float = 1.0e-10, outlet_edges: bool = True, TL=None, log=None,
                         linear_solver="superlu", predictor: bool = True,
                         max_restarts=None, stop_on_failure: bool = False,
                         max_iter: int = NITER):
    """Solve at each Weissenberg number of ``wis`` in turn (the inflow
    Dirichlet data follow Wi), each from the previous solution or, with
    ``predictor``, from the extrapolation through the last converged
    solutions (``extrapolate``).  ``max_iter`` bounds the Newton iterations
    of a first attempt (Niter), ``max_restarts`` the emergency restarts per
    point; a point that does not converge raises, or with
    ``stop_on_failure`` ends the run.  Returns the list of NewtonResult of
    the converged points."""
    out = []
    EU = np.ones(phys.nex)
    done_w, done_TL = [], []
    # one solver for all points (the frontal LU's symbolic phase is per mesh)
    solver = LS.make_solver(linear_solver, asm.rowptr, asm.colind, mesh)
    for wi in wis:
        p = dataclasses.replace(phys, WiN=wi, Wi0=wi)
        asm.set_params(p)
        rows, values = boundary_conditions(mesh, p)
        if TL is None:
            TL, EU = initial_state(mesh, p)
        elif predictor and len(done_w) >= 2:
            TL = extrapolate(done_w, done_TL, wi)
        TL = np.ascontiguousarray(TL)
        nr = NewtonRaphson(DeviceAssembly(asm, rows, values, jacobian, outlet_edges),
                           asm.rowptr, asm.colind, p.nex, mesh, linear_solver=solver)
        try:
            res = emergency_solve(nr, TL, EU, log=log, tol=tol, max_restarts=max_restarts,
                                  max_iter=max_iter)
        except (RuntimeError, FloatingPointError):
            if not stop_on_failure:
                raise
            break
        if not res.converged:
            if stop_on_failure:
                break
            raise RuntimeError(f"Newton did not converge at Wi = {wi}")
        out.append(res)
        TL, EU = res.TL, res.EU
        done_w.append(wi)
        done_TL.append(res.TL)
    return out


class NewtonRaphson:
    """loopNewtonRaphson for one parameter point.  ``assembly(TL, EU, want_jac)``
    returns the host residual and AIJ values with the Dirichlet rows applied."""

    def __init__(self, assembly, rowptr: np.ndarray, colind: np.ndarray, nex: int, mesh=None,
                 linear_solver="superlu"):
        self.assembly = assembly
        self.rowptr = rowptr
        self.colind = colind
        self.nex = nex
        self.N = len(rowptr) - 1
        # host SuperLU (nested-dissection order from the mesh when given, else
        # column AMD) or the GPU frontal LU (linsolve.make_solver)
        self.solver = LS.make_solver(linear_solver, rowptr, colind, mesh)
        if hasattr(assembly, "device_values"):
            assembly.device_values = LS.on_device(self.solver)

    def solve(self, TL: np.ndarray, EU: np.ndarray, tol: float = 1.0e-8,
              res_tol: float | None = None, max_iter: int = NITER, mnr: bool = True,
              xF: float = 1.0, log=None) -> NewtonResult:
        res_tol = tol if res_tol is None else res_tol
        TL = TL.copy()
        EU = EU.copy()
        nn = TL.shape[1]
        it = 0
        res_norm = 1.0
        cor_new = 1.0
        cor_old = 1.0
        flag = "NRP"
        lu = None
        hist = []
        t_asm = t_sol = 0.0
        while True:
            if cor_new < tol and res_norm < res_tol:
                return NewtonResult(TL, EU, True, it, hist, t_asm, t_sol)
            it += 1
            if it % 10 == 0:
                flag = "NRP"
            t0 = time.perf_counter()
            want_jac = flag == "NRP" or lu is None
            b, vals = self.assembly(TL, EU, want_jac)
            t1 = time.perf_counter()
            res_norm = float(np.linalg.norm(b))
            if want_jac:
                lu = self.solver.factor(vals)
            s = lu.solve(b)
            t2 = time.perf_counter()
            t_asm += t1 - t0
            t_sol += t2 - t1
            cor_new = float(np.linalg.norm(s))
            hist.append(dict(it=it, flag="NRP" if want_jac else "MNR",
                             res_norm=res_norm, cor_norm=cor_new))
            if log:
                log(f"{it:4d}. {flag}: RES_NORM = {res_norm:.4e}, COR_NORM = {cor_new:.4e}")
            if cor_new != cor_new:
                raise FloatingPointError("NaN encountered in the Newton correction")
            if flag == "NRP":
                flag = "MNR" if (mnr and cor_new < MNR_EPS) else "NRP"
            else:
                flag = "NRP" if cor_new > cor_old else "MNR"
            if cor_new > COR_NORM_DIV or it > max_iter:
                return NewtonResult(TL, EU, False, it, hist, t_asm, t_sol)
            cor_old = cor_new
            TL -= xF * s[:nn * 6].reshape(nn, 6).T
            if self.nex:
                EU -= xF * s[nn * 6:]
