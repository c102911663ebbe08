"""Pseudo-arclength continuation in the Weissenberg number over the GPU assembly.

Restates the reference's arclength driver for the Cylinder_2D problem with
Nex = 1 (the extra unknown lambda, Wi = Wi0 * lambda at every Gauss point):

* continuationStepArclength (Continuation_Arclength_mod.F90:77-130): Newton
  at the predicted point, then direction, step control and the next
  prediction; each Newton solve starts in the mode checkMNR picks
  (Newton_Raphson_mod.F90:72-78, 425-449), so a solve whose predecessor
  started with a small correction reuses the previous factorisation;
* the lambda equation (arclength, Extra_Equations_mod.F90:698-768): for the
  first two increments lambda is pinned, lambda - (LN0 + (k-1) dArN), with
  the lambda row and column replaced by the unit vector (MatZeroRowsColumns);
  afterwards pseudoArclength (:772-829): t . (x - x_o) - dS with the row
  [dTLodS, dEUodS];
* setDirectionVectors (:151-280): secant (x - x_o)/|x - x_o| at increment 2,
  afterwards the tangent solving J t = e_lambda with the last factorised
  Jacobian, normalised;
* adjustContinuationStep (:282-337): err_pr = max over fields of
  |x - x_p| / |x|, trns = sqrt(Eps_Pr / err_pr) capped at 2,
  dS = min(dS trns, dS_max);
* updateSolutionArclength (:339-379): the plain predictor x_p = x + t dS;
* emergencyNewtonRaphson (Newton_Raphson_mod.F90:533-584) when Newton
  diverges: restart from the prediction with the relaxation halved, 50 x
  Niter iterations and dSo halved.

A predictor object can replace the plain prediction (the learned POD/MLP
predictor in ``learned.py``); Newton stays the corrector.

Factorisation reuse (``ArclengthSettings.reuse``): "reference" follows
checkMNR and checkNewtonConvergence as above (every 10th iteration of a
solve refactorises).  "contraction" is the policy of the learned + mixed
path: the last factorisation is kept across steps for chord iterations as
long as each one contracts the correction by theta_max or better and the
iterations it predicts until the tolerance cost less than a factorisation;
a stale factorisation that stops contracting is replaced at the iterate
the failed chord step started from.  The residual, the tolerance and hence
the converged points are the same; only the Jacobian the corrections are
solved with is older.  Step cutbacks (``ArclengthSettings.cutbacks``, also
the learned + mixed path's) halve dS after a failed solve and predict again
from the last converged point before the reference's relaxation restart, so
the continuation follows the branch through folds instead of relaxing across
them.  The host solves
with SuperLU in a nested-dissection order (linsolve.py, stand-in for
MUMPS) or on the GPU with the panel-frontal LU (frontal.py); the dense lambda
row and the arclength column make the matrix bordered, and the lambda unknown
is ordered last.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import linsolve as LS
from . import newton as NW
from . import state as S

EPS_PR = 1.0e-3
DS_MAX = 50.0


@dataclasses.dataclass
class ArclengthSettings:
    LN0: float = 1.0          # lambda of increment 1 (Wi = Wi0 * LN0)
    dArN: float = 0.1         # lambda step of increment 2
    dS0: float = 1.0          # first arclength step
    dS_max: float = DS_MAX
    eps_pr: float = EPS_PR
    tol: float = 1.0e-10      # Newton tolerance on |s| and |R|
    lam_max: float = 10.0     # stop once lambda >= lam_max
    max_steps: int = 200
    # factorisation reuse: "reference" (checkMNR / checkNewtonConvergence
    # switching) or "contraction" (chord iterations on the last factorisation
    # across steps, refactorised when their observed contraction makes the
    # remaining iterations cost more than a new factorisation)
    reuse: str = "reference"
    # cost of a factorisation in chord iterations for "contraction"; None
    # measures both costs online (host wall time)
    factor_cost: float | None = None
    chord_max: int = 30       # at most this many predicted chord iterations
    theta_max: float = 1.0    # refactorise when a chord step contracts less than this
    # step cutbacks before the reference's emergency (relaxation halving): a
    # failed arclength solve halves dS and predicts again from the last
    # converged point; a solve on a cutback-enabled step fails early once it
    # has taken ``cutback_factorisations`` factorisations without converging
    cutbacks: int = 0
    cutback_factorisations: int = 3
    # Newton-Krylov corrections on an older factorisation ("contraction" reuse
    # only): GMRES iterations allowed per correction (0: chord steps), its
    # relative tolerance, and the iteration count beyond which the next
    # iterate takes a new factorisation
    krylov: int = 0
    krylov_rtol: float = 1.0e-4
    krylov_refactor: int = 8
    # with krylov > 0: the arclength tangent from the Jacobian at the converged
    # point by GMRES (an older factorisation tilts the arclength plane)
    krylov_tangent: bool = True
    # relative residual a linear solve is checked (and refined) against
    # during this run; None keeps the solver's own (1e-10 for the GPU
    # frontal LU).  An inexact Newton (stale factorisations, FP32 Jacobian)
    # needs no 1e-10 solves: its corrections are approximate by design
    solve_check_tol: float | None = None


@dataclasses.dataclass
class StepRecord:
    increment: int
    wi: float
    lam: float
    dS: float
    newton_iterations: int
    factorisations: int
    res_norm: float
    predictor: str
    pred_error: float
    wall_s: float
    assembly_s: float = 0.0     # device assembly + Dirichlet/lambda rows, host copies
    factor_s: float = 0.0       # host LU factorisations
    solve_s: float = 0.0        # host triangular solves (Newton and tangent)
    predictor_s: float = 0.0    # learned predictor: prediction, judging, training
    emergencies: int = 0        # Newton restarts with relaxation (emergencyNewtonRaphson)
    cutbacks: int = 0           # step cutbacks (dS halved, predicted again)


class LambdaRow:
    """Host side of the lambda equation applied after assembly and Dirichlet."""

    def __init__(self, rowptr: np.ndarray, colind: np.ndarray):
        self.rowptr = rowptr
        self.colind = colind
        self.N = len(rowptr) - 1
        self.last_col_slots = rowptr[1:-1] - 1          # last entry of every node row
        assert np.all(colind[self.last_col_slots] == self.N - 1)
        self.mode = "pinned"
        self.target = 0.0
        self.t = None          # direction (N,)
        self.x_o = None        # previous converged point (N,)
        self.dS = 0.0

    def __call__(self, x: np.ndarray, b: np.ndarray, vals):
        """``vals``: host array, device tensor (FP64) or None."""
        N = self.N
        r0, r1 = self.rowptr[N - 1], self.rowptr[N]
        slots = self.last_col_slots
        if vals is not None and not isinstance(vals, np.ndarray):
            slots = self._device_slots(vals.device)
        if self.mode == "pinned":
            b[N - 1] = x[N - 1] - self.target
            if vals is not None:
                vals[slots] = 0.0
                vals[r0:r1] = 0.0
                vals[r1 - 1] = 1.0
        else:
            b[N - 1] = float(np.dot(self.t, x - self.x_o)) - self.dS
            if vals is None:
                pass
            elif isinstance(vals, np.ndarray):
                vals[r0:r1] = self.t
            else:
                import torch
                vals[r0:r1] = torch.from_numpy(self.t).to(vals.device)

    def _device_slots(self, device):
        if getattr(self, "_dslots", None) is None or self._dslots.device != device:
            import torch
            self._dslots = torch.from_numpy(self.last_col_slots.astype(np.int64)).to(device)
        return self._dslots


class SecantPredictor:
    """Secant prediction x_p = x_k + dS (x_k - x_{k-1}) / |x_k - x_{k-1}| in
    place of the reference's tangent (the reference uses the secant only at
    increment 2, setDirectionVectors, Continuation_Arclength_mod.F90:183-206).
    It replaces the tangent step outright (no residual judging)."""

    replaces = True

    def __init__(self):
        self.last = []

    def observe(self, k, x, wi):
        self.last = (self.last + [x.copy()])[-2:]

    def predict(self, k, x_o, t, dS, x_plain):
        if len(self.last) < 2:
            return None
        d = self.last[1] - self.last[0]
        return self.last[1] + d * (dS / np.linalg.norm(d))


class ArclengthContinuation:
    """loopArclength for one mesh and one assembler (nex = 1)."""

    def __init__(self, asm, mesh, phys: S.Physics, jacobian: str = "fd64",
                 settings: ArclengthSettings | None = None, outlet_edges: bool = True,
                 log=None, assembly=None, linear_solver="superlu"):
        if phys.nex != 1:
            raise ValueError("arclength continuation needs nex = 1")
        self.asm, self.mesh, self.phys = asm, mesh, phys
        self.cfg = settings or ArclengthSettings()
        self.jacobian = jacobian
        self.log = log
        rows, values = NW.boundary_conditions(mesh, phys)
        self.rows = rows
        self.dev = assembly if assembly is not None else \
            NW.DeviceAssembly(asm, rows, values, jacobian, outlet_edges)
        self.lrow = LambdaRow(asm.rowptr, asm.colind)
        # host SuperLU or the GPU frontal LU (linsolve.make_solver); a device
        # solver takes the AIJ values where the assembly left them
        self.solver = LS.make_solver(linear_solver, asm.rowptr, asm.colind, mesh)
        if hasattr(self.dev, "device_values"):
            self.dev.device_values = LS.on_device(self.solver)
        self.N = asm.N
        self.nn = asm.nnodes
        self.judge_s = 0.0
        self.cor0 = 1.0          # first correction norm of the last solve (cor_norm0_Main)
        self.have_lu = False     # a factorisation exists (LS%maxit > 0)
        self.failed_factorisations = 0
        if self.cfg.reuse not in ("reference", "contraction"):
            raise ValueError(f"unknown factorisation reuse policy {self.cfg.reuse!r}")
        # running costs (s) of a chord iteration and of a factorisation, for
        # the "contraction" policy
        self.t_iter = None
        self.t_fac = None
        self.reverted = 0        # chord steps undone because they did not contract
        self.krylov_iterations = 0   # GMRES iterations of Newton-Krylov corrections
        self.krylov_failures = 0     # corrections whose GMRES missed its tolerance
        self.last_krylov_its = 0

    # state vector x = [TL in node-major order, lambda]
    def pack(self, TL, EU):
        return np.concatenate([TL.T.reshape(-1), EU])

    def unpack(self, x):
        return np.ascontiguousarray(x[:-1].reshape(self.nn, 6).T), x[-1:].copy()

    def _update_inflow(self, lam: float):
        # the inflow profile follows Wi = Wi0 * lambda (applyDirichletBCFullyDeveloped)
        p = dataclasses.replace(self.phys, WiN=self.phys.Wi0 * lam)
        rows, values = NW.boundary_conditions(self.mesh, p)
        self.dev.set_values(values)

    def _start_flag(self, k: int) -> str:
        """checkMNR (Newton_Raphson_mod.F90:425-449): a solve starts with 'MNR'
        -- the factorisation of the previous solve -- when the first correction
        of the previous solve was below MNR_eps, except at every 100th
        increment (if that correction was above MNR_eps/10) and every 1000th."""
        if self.cfg.reuse == "contraction":
            return "MNR" if self.have_lu else "NRP"
        flag = "MNR" if self.cor0 < NW.MNR_EPS else "NRP"
        if (k % 100 == 0 and self.cor0 > NW.MNR_EPS / 10.0) or k % 1000 == 0:
            flag = "NRP"
        return flag if self.have_lu else "NRP"

    def _factor_cost(self) -> float:
        """A factorisation's cost in chord iterations."""
        if self.cfg.factor_cost is not None:
            return self.cfg.factor_cost
        if self.t_iter is None or self.t_fac is None:
            return 10.0
        return self.t_fac / max(self.t_iter, 1e-9)

    def _newton_chord(self, x0: np.ndarray, xF: float, max_iter: int, flag: str,
                      max_fac: int | None = None):
        """Newton with the lambda row, reusing the last factorisation across
        solves (chord iterations) while it contracts well enough.  With a
        contraction rate theta = |s_k| / |s_(k-1)| observed on one
        factorisation, finishing takes n = log(tol / |s_k|) / log(theta) more
        iterations; a new factorisation is taken at the next iterate when n
        exceeds ``chord_max`` or costs more than a factorisation plus three
        iterations.  A chord step on an older factorisation that does not
        contract (theta >= 1) is undone and the Jacobian assembled at the
        iterate it started from; after a Newton step on a factorisation taken
        at its own starting point the Jacobian is assembled at the new iterate
        (the reference's 'MNR' -> 'NRP' switch).  With ``max_fac`` the solve
        fails once it would take a factorisation beyond that many.

        With ``krylov`` > 0, where this policy would take a new factorisation
        at an iterate that an older one could still serve (chord steps that
        stopped contracting, mostly the stall of chord iterations close to
        the solution), a Newton-Krylov step comes first: the Jacobian is
        assembled at the iterate (cheap next to a factorisation) and J s = R
        is solved by GMRES to ``krylov_rtol``, preconditioned by the older
        factorisation; chord steps resume after it.  The factorisation is
        taken (from the Jacobian just assembled) only when GMRES misses the
        tolerance within ``krylov`` iterations, or at the next iterate after
        a GMRES that needed more than ``krylov_refactor``.  Returns what
        _newton returns."""
        cfg = self.cfg
        x = x0.copy()
        tm = self.timers
        res_norm = cor_new = 1.0
        cor_old = None           # last correction on the current factorisation
        x_prev = None            # the iterate that correction started from
        prev_fresh = False       # the factorisation was taken at x_prev
        lu = self.solver if self.have_lu else None
        want = flag == "NRP" or lu is None
        want_krylov = False
        it = nfac = 0
        while True:
            if cor_new < cfg.tol and res_norm < cfg.tol:
                return x, it, nfac, res_norm, lu, True
            it += 1
            t0 = time.perf_counter()
            TL, EU = self.unpack(x)
            self._update_inflow(float(EU[0]))
            if want and max_fac is not None and nfac >= max_fac:
                return x, it, nfac, res_norm, lu, False
            krylov = want_krylov and not want and lu is not None
            want_krylov = False
            b, vals = self.dev(TL, EU, want or krylov)
            self.lrow(x, b, vals)
            res_norm = float(np.linalg.norm(b))
            t1 = time.perf_counter()
            if not np.isfinite(res_norm):
                return x, it, nfac, res_norm, lu, False
            s = None
            if krylov:
                s = self._krylov_solve(lu, vals, b)
                if s is None:
                    # GMRES did not converge: factorise the Jacobian just assembled
                    if max_fac is not None and nfac >= max_fac:
                        return x, it, nfac, res_norm, lu, False
                    want = True
            t_k = time.perf_counter()
            if want:
                try:
                    lu = self.solver.factor(vals)
                except RuntimeError:
                    self.failed_factorisations += 1
                    self.have_lu = False
                    tm["factor"] += time.perf_counter() - t_k
                    return x, it, nfac, res_norm, None, False
                self.have_lu = True
                nfac += 1
                cor_old = None
            t2 = time.perf_counter()
            if s is None:
                try:
                    s = lu.solve(b)
                except RuntimeError:     # its pivoted re-factorisation was singular
                    self.failed_factorisations += 1
                    self.have_lu = False
                    return x, it, nfac, res_norm, None, False
            t3 = time.perf_counter()
            tm["assembly"] += t1 - t0
            tm["factor"] += t2 - t_k
            tm["solve"] += (t3 - t2) + (t_k - t1)
            if want:
                c = (t1 - t0) + (t2 - t_k)
                self.t_fac = c if self.t_fac is None else 0.5 * (self.t_fac + c)
            else:
                c = (t1 - t0) + (t3 - t2) + (t_k - t1)
                self.t_iter = c if self.t_iter is None else 0.5 * (self.t_iter + c)
            cor_new = float(np.linalg.norm(s))
            if it == 1:
                self.cor0 = cor_new
            if self.log:
                mode = "NRP" if want else ("NK" if krylov else "MNR")
                self.log(f"   {it:3d}. {mode}: RES_NORM = {res_norm:.4e}, "
                         f"COR_NORM = {cor_new:.4e}")
            if cor_new != cor_new or cor_new > NW.COR_NORM_DIV or it > max_iter:
                return x, it, nfac, res_norm, lu, False
            fresh = want
            want = False
            # a Newton-Krylov step in place of the factorisation the rules
            # below ask for (not after a fresh factorisation, nor right after
            # a Newton-Krylov step that needed many GMRES iterations)
            use_krylov = cfg.krylov > 0 and not fresh and \
                not (krylov and self.last_krylov_its > cfg.krylov_refactor)
            if cor_old is not None and cor_new >= cfg.tol:
                theta = cor_new / cor_old
                if theta >= 1.0 and not prev_fresh:
                    # a stale factorisation that does not contract: undo the
                    # chord step, refactorise (or take a Newton-Krylov step)
                    # where it started
                    self.reverted += 1
                    x = x_prev
                    cor_new = cor_old
                    if use_krylov and not krylov:
                        want_krylov = True
                    else:
                        want = True
                    continue
                if theta >= cfg.theta_max:
                    want = True
                else:
                    n = np.log(cfg.tol / cor_new) / np.log(theta)
                    want = n > cfg.chord_max or n > self._factor_cost() + 3.0
            elif fresh and cor_new > NW.MNR_EPS:
                # far from the solution: full Newton steps, as the reference
                # stays in 'NRP' until the correction drops below MNR_eps
                want = True
            if krylov and self.last_krylov_its > cfg.krylov_refactor:
                want = True
            elif want and use_krylov:
                want, want_krylov = False, True
            cor_old = cor_new
            x_prev, prev_fresh = x, fresh
            x = x - xF * s

    def _krylov_solve(self, lu, vals, b):
        """GMRES on J s = b with the Jacobian values ``vals`` (device tensor or
        host array, lambda and Dirichlet rows applied) and the factorisation
        ``lu`` as right preconditioner; the correction as a host array, or
        None when GMRES did not reach ``krylov_rtol``."""
        cfg = self.cfg
        if isinstance(vals, np.ndarray):
            import scipy.sparse as sp
            J = sp.csr_matrix((vals, self.lrow.colind, self.lrow.rowptr), shape=(self.N, self.N))
            rhs = np.asarray(b, dtype=np.float64)
            pre = getattr(lu, "precondition", lu.solve)
            s, its, rel = LS.gmres(lambda v: J @ v, pre, rhs, cfg.krylov_rtol, cfg.krylov)
        else:
            import warnings

            import torch
            dev = vals.device
            if getattr(self, "_csr_dev", None) != dev:
                self._crow = torch.from_numpy(self.lrow.rowptr.astype(np.int64)).to(dev)
                self._col = torch.from_numpy(self.lrow.colind.astype(np.int64)).to(dev)
                self._csr_dev = dev
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                J = torch.sparse_csr_tensor(self._crow, self._col, vals.to(torch.float64),
                                            size=(self.N, self.N), check_invariants=False)
            rhs = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).to(dev)
            pre = lu.precondition if hasattr(lu, "precondition") else \
                (lambda v: torch.from_numpy(lu.solve(v.cpu().numpy())).to(dev))
            s, its, rel = LS.gmres(lambda v: J @ v, pre, rhs, cfg.krylov_rtol, cfg.krylov)
            s = s.cpu().numpy()
        self.last_krylov_its = its
        self.krylov_iterations += its
        if not (rel <= cfg.krylov_rtol) or not np.all(np.isfinite(s)):
            self.krylov_failures += 1
            return None
        return s

    def _newton(self, x0: np.ndarray, xF: float = 1.0, max_iter: int = NW.NITER,
                flag: str = "NRP", max_fac: int | None = None):
        """Newton with the lambda row and relaxation xF, starting in mode
        ``flag``; returns (x, iterations, factorisations, last residual norm,
        the solver holding the last factorisation, converged)."""
        cfg = self.cfg
        if cfg.reuse == "contraction":
            return self._newton_chord(x0, xF, max_iter, flag, max_fac)
        x = x0.copy()
        tm = self.timers
        res_norm = cor_new = cor_old = 1.0
        lu = self.solver if self.have_lu else None
        it = nfac = 0
        while True:
            if cor_new < cfg.tol and res_norm < cfg.tol:
                return x, it, nfac, res_norm, lu, True
            it += 1
            if it % 10 == 0:
                flag = "NRP"
            t0 = time.perf_counter()
            TL, EU = self.unpack(x)
            want = flag == "NRP" or lu is None
            self._update_inflow(float(EU[0]))
            b, vals = self.dev(TL, EU, want)
            self.lrow(x, b, vals)
            res_norm = float(np.linalg.norm(b))
            t1 = time.perf_counter()
            if not np.isfinite(res_norm):
                # a diverged iterate (non-finite residual): a failed solve
                return x, it, nfac, res_norm, lu, False
            if want:
                try:
                    lu = self.solver.factor(vals)
                except RuntimeError:
                    # a singular Jacobian (SuperLU: exactly zero pivot under
                    # partial pivoting too) fails this solve like divergence;
                    # the caller restarts with the relaxation halved
                    self.failed_factorisations += 1
                    self.have_lu = False
                    tm["factor"] += time.perf_counter() - t1
                    return x, it, nfac, res_norm, None, False
                self.have_lu = True
                nfac += 1
            t2 = time.perf_counter()
            try:
                s = lu.solve(b)
            except RuntimeError:     # its pivoted re-factorisation was singular
                self.failed_factorisations += 1
                self.have_lu = False
                return x, it, nfac, res_norm, None, False
            t3 = time.perf_counter()
            tm["assembly"] += t1 - t0
            tm["factor"] += t2 - t1
            tm["solve"] += t3 - t2
            cor_new = float(np.linalg.norm(s))
            if it == 1:
                self.cor0 = cor_new
            if self.log:
                self.log(f"   {it:3d}. {flag}: RES_NORM = {res_norm:.4e}, COR_NORM = {cor_new:.4e}")
            if cor_new != cor_new or cor_new > NW.COR_NORM_DIV or it > max_iter:
                return x, it, nfac, res_norm, lu, False
            if flag == "NRP":
                flag = "MNR" if cor_new < NW.MNR_EPS else "NRP"
            else:
                flag = "NRP" if cor_new > cor_old else "MNR"
            cor_old = cor_new
            x = x - xF * s

    def run(self, TL0: np.ndarray, EU0: np.ndarray, predictor=None):
        """Continue from (TL0, EU0) until lambda >= lam_max; returns the step
        records and the converged states."""
        saved = getattr(self.solver, "check_tol", None)
        if self.cfg.solve_check_tol is not None and saved is not None:
            self.solver.check_tol = self.cfg.solve_check_tol
        try:
            return self._run(TL0, EU0, predictor)
        finally:
            if saved is not None:
                self.solver.check_tol = saved

    def _run(self, TL0: np.ndarray, EU0: np.ndarray, predictor=None):
        cfg = self.cfg
        x_p = self.pack(TL0, EU0)
        x_p[-1] = cfg.LN0
        x_o = None
        t = None
        dS = cfg.dS0
        records, states = [], []
        for k in range(1, cfg.max_steps + 1):
            t0 = time.perf_counter()
            self.timers = dict(assembly=0.0, factor=0.0, solve=0.0, predictor=0.0)
            if k <= 2:
                self.lrow.mode = "pinned"
                self.lrow.target = cfg.LN0 + (k - 1) * cfg.dArN
                x_p[-1] = self.lrow.target
            else:
                self.lrow.mode = "arclength"
                self.lrow.t, self.lrow.x_o, self.lrow.dS = t, x_o, dS
            pred_name = "plain"
            if predictor is not None and k > 2:
                x_p, pred_name = self._predict(predictor, k, x_o, t, dS, x_p)
            # step cutbacks (cfg.cutbacks, the learned + mixed path): halve dS
            # and predict again from the last converged point
            # emergencyNewtonRaphson (Newton_Raphson_mod.F90:533-584): restart
            # from the prediction with the relaxation halved, 50 x Niter
            # iterations allowed and, on the arclength branch, dSo halved
            xF, max_it, its, nfac, emerg, cuts = 1.0, NW.NITER, 0, 0, 0, 0
            flag0 = self._start_flag(k)
            while True:
                can_cut = k > 2 and cuts < cfg.cutbacks
                x, i1, f1, rn, lu, ok = self._newton(
                    x_p, xF, max_it, flag0, cfg.cutback_factorisations if can_cut else None)
                its += i1
                nfac += f1
                if ok:
                    break
                if can_cut:
                    cuts += 1
                    dS *= 0.5
                    self.lrow.dS = dS
                    x_p, pred_name = x_o + t * dS, "plain"
                    if predictor is not None:
                        x_p, pred_name = self._predict(predictor, k, x_o, t, dS, x_p)
                    flag0 = "NRP"
                    if self.log:
                        self.log(f"step {k}: cutback to dS = {dS:.4g}")
                    continue
                xF *= 0.5
                emerg += 1
                if xF < 1.0e-2:
                    raise RuntimeError(f"arclength Newton failed at increment {k} "
                                       f"(lambda = {x_p[-1]:.6g}, dS = {dS:.4g})")
                max_it = 50 * NW.NITER
                flag0 = "NRP"
                if k > 2:
                    dS *= 0.5
                    self.lrow.dS = dS
            err_pr = 0.0
            if k > 1:
                TLc, EUc = self.unpack(x)
                TLp, EUp = self.unpack(x_p)
                e = [np.linalg.norm(TLc[f] - TLp[f]) / max(np.linalg.norm(TLc[f]), 1e-300)
                     for f in range(6)]
                e.append(abs(EUc[0] - EUp[0]) / max(abs(EUc[0]), 1e-300))
                err_pr = max(e)
            lam = float(x[-1])
            if predictor is not None:
                tp = time.perf_counter()
                predictor.observe(k, x, self.phys.Wi0 * lam)
                self.timers["predictor"] += time.perf_counter() - tp
            states.append(x.copy())
            done = lam >= cfg.lam_max
            # direction (setDirectionVectors)
            if k == 1:
                t_new = None
            elif k == 2:
                d = x - x_o
                t_new = d / np.linalg.norm(d)
            elif not done:
                e_l = np.zeros(self.N)
                e_l[-1] = 1.0
                ts = time.perf_counter()
                tv = None
                if cfg.krylov > 0 and cfg.krylov_tangent:
                    # the tangent of the Jacobian at the converged point, by
                    # GMRES preconditioned with the (possibly older) factorisation
                    TLc, EUc = self.unpack(x)
                    self._update_inflow(float(EUc[0]))
                    _, vals_c = self.dev(TLc, EUc, True)
                    self.lrow(x, np.zeros(self.N), vals_c)
                    tv = self._krylov_solve(lu, vals_c, e_l)
                if tv is None:
                    tv = lu.solve(e_l)
                self.timers["solve"] += time.perf_counter() - ts
                t_new = tv / np.linalg.norm(tv)
                if np.dot(t_new, t) < 0.0:
                    t_new = -t_new
            wall = time.perf_counter() - t0
            tm = self.timers
            records.append(StepRecord(k, self.phys.Wi0 * lam, lam, dS, its, nfac, rn, pred_name,
                                      err_pr, wall, tm["assembly"], tm["factor"], tm["solve"],
                                      tm["predictor"], emerg, cuts))
            if self.log:
                self.log(f"step {k}: Wi = {self.phys.Wi0 * lam:.4f}, Newton {its}, "
                         f"pred {pred_name} err {err_pr:.2e}, dS = {dS:.3f}, {wall:.2f} s")
            if done:
                break
            # step size (adjustContinuationStep)
            if k > 1:
                trns = min(np.sqrt(cfg.eps_pr / max(err_pr, 1e-300)), 2.0)
                dS = min(dS * trns, cfg.dS_max)
            # prediction (updateSolutionArclength)
            x_o = x.copy()
            t = t_new
            x_p = x.copy() if t is None else x + t * dS
        return records, states

    def _predict(self, predictor, k, x_o, t, dS, x_plain):
        """The predictor's candidates for step length dS, judged against the
        plain prediction x_plain; returns (x_p, name)."""
        tp = time.perf_counter()
        x_p, name = x_plain, "plain"
        if hasattr(predictor, "candidates"):
            cands = predictor.candidates(k, x_o, t, dS, x_plain)
            if cands:
                x_p, name = self._judge([("plain", x_plain)] + cands)
        else:
            cand = predictor.predict(k, x_o, t, dS, x_plain)
            if cand is not None and getattr(predictor, "replaces", False):
                x_p, name = cand, type(predictor).__name__
            elif cand is not None:
                x_p, name = self._judge([("plain", x_plain), ("learned", cand)])
        self.timers["predictor"] += time.perf_counter() - tp
        return x_p, name

    def _judge(self, cands):
        """Newton judges the predictions by residual norm: of the (name, x)
        candidates, the plain prediction first, the one with the smallest
        residual (Dirichlet and lambda rows included) is taken; ties keep
        the earlier one."""
        t0 = time.perf_counter()
        best, best_r = cands[0], None
        for name, x in cands:
            TL, EU = self.unpack(x)
            self._update_inflow(float(EU[0]))
            b, _ = self.dev(TL, EU, False)
            self.lrow(x, b, None)
            r = float(np.linalg.norm(b))
            if best_r is None or r < best_r:
                best, best_r = (name, x), r
        self.judge_s += time.perf_counter() - t0
        return best[1], best[0]
