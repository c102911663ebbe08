"""Panel-frontal LU of the bordered Newton Jacobian on the GPU (stand-in for
the reference's MUMPS direct solve, ``KSPSolve`` in Petsc_mod.F90:850).

The host SuperLU of ``linsolve.py`` needs ~32 s per factorisation of the
20,000-quad Jacobian; this solver factorises the same matrix on the device in
dense FP64 blocks.

Symbolic phase (once per mesh and AIJ pattern).  Elements are swept
downstream in order of their centroid x and grouped into panels of ``G``
elements (by default about one element column of the channel).  A node is
*fully summed* after the last panel that touches it; the *front* after panel
q is the set of nodes touched by panels <= q and by a later panel.  Panel q's
frontal matrix covers, in this order, its pivots P_q (the unknowns of the
nodes fully summed at q) and the front F_q; the border unknowns (the
arclength lambda: a dense row and column) stay at the end of every front and
are eliminated with the last panel's pivots, so a Jacobian that is singular
at a fold (where the bordered matrix is not) never has to be factorised
without its border.  Each CSR entry (i, j) is added exactly once, to the
frontal matrix of panel min(last(i), last(j)); both ends are in that panel's
pivots or front.

Numeric phase (every factorisation), for q = 0, 1, ...:

    M_q  = original entries of panel q + extend-add of S_(q-1)
    LU_q = lu(M_q[P, P]) with partial pivoting            (cuSOLVER getrf)
    X_q  = M_q[P, P]^-1 M_q[P, F]                         (triangular solves)
    S_q  = M_q[F, F] - M_q[F, P] X_q                      (cuBLAS gemm)

A pivot the unpivoted elimination refuses (below 1e-12 of its 16 x 16 block)
is met by delaying pressures: a pressure row couples to the velocities of
its element-mates, and where those are all still in the front its entries
inside the pivot block can cancel; the symbolic phase is then redone once
with every pressure eliminated with the last panel that touches any of its
element-mates (fronts ~1.3x, work ~1.55x), and the solver stays so.

Solve: forward y_P = LU_q^-1 b_P, b_F -= M_q[F, P] y_P; backward
x_P = y_P - X_q x_F.  Each solve is checked against the CSR matrix (FP64
SpMV) and refined (x += solve(b - A x)) up to ``refine`` times; a zero pivot
or a solve that stays inaccurate hands the matrix to the host SuperLU
(``linsolve.SparseLU``) for that factorisation.

On the cylinder meshes the fronts are one node column of the channel plus the
border (~500 unknowns on average at 20,000 quads, ~1,300 at most around the
cylinder); a factorisation is ~0.9 TFLOP at 20,000 quads, 2.6 TFLOP at 40,000.
Everything is FP64.
"""
from __future__ import annotations

import math
import warnings

import numpy as np


def default_panel(nel: int) -> int:
    """Elements per panel: about a quarter of an element column of the
    cylinder meshes (their channel is m elements high with nel ~ 20 m^2).
    Smaller panels mean smaller pivot blocks, hence less elimination work per
    unknown (the front, one node column, stays the same), but more steps;
    a quarter column measured fastest on GB300 at 20,000 and 40,000 quads."""
    return max(4, int(round(math.sqrt(nel / 20.0) / 4.0)))


class FrontalLU:
    """Factorise and solve A x = b for AIJ values on a fixed CSR pattern whose
    first ``neq * nnodes`` unknowns are node-major mesh unknowns and whose
    remaining ones (if any) are border unknowns with dense rows and columns."""

    def __init__(self, rowptr: np.ndarray, colind: np.ndarray, mesh, neq: int = 6,
                 panel: int | None = None, device=None, check_tol: float = 1.0e-10,
                 refine: int = 3, method: str | None = None, pivot_tol: float = 1.0e-12,
                 p_field: int | None = 2, delay_pressure: bool = False):
        import torch
        self.torch = torch
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device()) \
                if torch.cuda.is_available() else torch.device("cpu")
        self.dev = torch.device(device)
        self.rowptr = np.asarray(rowptr, dtype=np.int64)
        self.colind = np.asarray(colind)
        self.N = len(self.rowptr) - 1
        self.neq = neq
        self.nn = mesh.nnodes
        self.nb = self.N - neq * self.nn
        if self.nb < 0:
            raise ValueError("pattern smaller than neq * nnodes")
        self.mesh = mesh
        self.p_field = p_field        # the pressure's place among a node's unknowns
        # pressures eliminated with their node (fronts ~25% smaller) until a
        # pivot is refused; then the symbolic phase is redone with the
        # pressures delayed (see _symbolic) and kept that way
        self.delay_pressure = delay_pressure
        self.check_tol = check_tol
        self.refine = refine
        en = mesh.element_nodes()
        # "native": the library's unpivoted blocked Gauss-Jordan kernels (CUDA
        # devices), with the pivoted path for a matrix whose pivots fail;
        # "pivoted": partial-pivoting LU per panel through torch (cuSOLVER)
        if method is None:
            method = "native" if self.dev.type == "cuda" else "pivoted"
        if method not in ("native", "pivoted"):
            raise ValueError(f"unknown frontal method {method!r}")
        if method == "native" and self.dev.type != "cuda":
            raise ValueError("the native frontal elimination needs a CUDA device")
        self.method = method
        self.pivot_tol = pivot_tol
        self.G = int(panel) if panel else default_panel(en.shape[0])
        self._handle = None
        self._symbolic(en, mesh.xyz[0][en].mean(axis=1))
        if method == "native":
            self._create_native()
        self.device_values = True   # factor() takes the AIJ values on the device
        self.fallbacks = 0          # factorisations handed to the host SuperLU
        self.pivoted_factorisations = 0   # native elimination refused a pivot
        self.resymbolised = False   # switched to delayed pressures after a refusal
        self.min_pivot = None       # smallest relative pivot of the last native factorisation
        self.mode = None            # path of the last factorisation
        self.refinements = 0        # refinement steps taken by solves
        self.check_every = 8        # solves between residual checks on one factorisation
        self._since_factor = 0
        self._needs_checks = False
        self._hb = self._hx = None  # pinned staging of host right-hand sides
        self.refactorisations = 0
        self.pivoted = True
        self._host = None
        self._factors = None

    # ------------------------------------------------------------------ symbolic
    def _symbolic(self, en: np.ndarray, xcen: np.ndarray):
        torch, dev = self.torch, self.dev
        nel, nbf = en.shape
        nn, neq, N, nb = self.nn, self.neq, self.N, self.nb
        order = np.argsort(xcen, kind="stable")
        pan = np.empty(nel, dtype=np.int64)
        pan[order] = np.arange(nel) // self.G
        npan = int(pan.max()) + 1
        ev = en.reshape(-1)
        ep = np.repeat(pan, nbf)
        last = np.full(nn, -1, dtype=np.int64)
        np.maximum.at(last, ev, ep)
        first = np.full(nn, npan, dtype=np.int64)
        np.minimum.at(first, ev, ep)
        if (last < 0).any():
            raise ValueError("a node belongs to no element")
        # Per unknown: the panel it is eliminated with.  A node's unknowns go
        # with the last panel that touches the node, except its pressure
        # (field ``p_field``), which is delayed to the last panel that touches
        # any node of its elements: a pressure row couples to the velocities
        # of its element-mates (continuity), and on symmetric stretches of the
        # mesh its couplings inside a panel whose other pivots do not include
        # those velocities cancel, leaving a zero pivot row; once they are
        # eliminated their Schur complement gives it a nonzero diagonal.
        last_nb = np.full(nn, -1, dtype=np.int64)
        np.maximum.at(last_nb, ev, np.repeat(last[en].max(axis=1), nbf))
        last_u = np.repeat(last, neq).reshape(nn, neq)
        if self.delay_pressure and self.p_field is not None:
            last_u[:, self.p_field] = last_nb
        last_u = np.concatenate([last_u.reshape(-1), np.full(nb, npan - 1, np.int64)])
        first_u = np.concatenate([np.repeat(first, neq), np.zeros(nb, np.int64)])
        # pivots of each panel, by unknown id (the border unknowns come last)
        piv_u = np.argsort(last_u, kind="stable")
        piv_ptr = np.concatenate([[0], np.cumsum(np.bincount(last_u, minlength=npan))])
        # front after each panel: (q, unknown) for first <= q < last, by (q, unknown)
        span = last_u - first_u
        tot = int(span.sum())
        fq = np.repeat(first_u, span) + (np.arange(tot) - np.repeat(np.cumsum(span) - span, span))
        fv = np.repeat(np.arange(N, dtype=np.int64), span)
        o = np.lexsort((fv, fq))
        fq, fv = fq[o], fv[o]
        fr_ptr = np.concatenate([[0], np.cumsum(np.bincount(fq, minlength=npan))])

        p_sz, f_sz, ids, idxP, idxF = [], [], [], [], []
        for q in range(npan):
            P = piv_u[piv_ptr[q]:piv_ptr[q + 1]].astype(np.int64)
            F = fv[fr_ptr[q]:fr_ptr[q + 1]]
            p_sz.append(len(P))
            f_sz.append(len(F))
            idxP.append(P)
            idxF.append(F)
            ids.append(np.concatenate([P, F]))
        self.npan = npan
        self.p_sz = np.array(p_sz, dtype=np.int64)
        self.f_sz = np.array(f_sz, dtype=np.int64)
        n_sz = self.p_sz + self.f_sz
        self.n_sz = n_sz
        self.off = np.concatenate([[0], np.cumsum(n_sz * n_sz)])
        # (panel, unknown) -> position in the panel's frontal matrix
        all_ids = np.concatenate(ids)
        all_q = np.repeat(np.arange(npan, dtype=np.int64), n_sz)
        all_pos = np.concatenate([np.arange(n, dtype=np.int64) for n in n_sz])
        keys = all_q * N + all_ids
        ko = np.argsort(keys, kind="stable")
        keys_t = torch.from_numpy(keys[ko]).to(dev)
        pos_t = torch.from_numpy(all_pos[ko]).to(dev)

        def lookup(qv, uv):
            k = qv * N + uv
            i = torch.searchsorted(keys_t, k)
            i = torch.clamp(i, max=len(keys_t) - 1)
            if not bool((keys_t[i] == k).all()):
                raise RuntimeError("frontal symbolic phase: an entry outside its panel")
            return pos_t[i]

        # each CSR entry goes to panel min(last(row), last(col))
        last_u = torch.from_numpy(last_u).to(dev)
        rp = torch.from_numpy(self.rowptr).to(dev)
        ci = torch.from_numpy(self.colind.astype(np.int64)).to(dev)
        rows = torch.repeat_interleave(torch.arange(N, device=dev), rp[1:] - rp[:-1])
        qs = torch.minimum(last_u[rows], last_u[ci])
        pr = lookup(qs, rows)
        pc = lookup(qs, ci)
        n_t = torch.from_numpy(n_sz).to(dev)
        off_t = torch.from_numpy(self.off[:-1]).to(dev)
        self.dest = off_t[qs] + pr * n_t[qs] + pc
        del rows, qs, pr, pc
        # extend-add maps: front of q -> positions in panel q + 1
        self.ext = []
        for q in range(npan - 1):
            F = torch.from_numpy(idxF[q]).to(dev)
            self.ext.append(lookup(torch.full_like(F, q + 1), F))
        self.idxP = [torch.from_numpy(a).to(dev) for a in idxP]
        self.idxF = [torch.from_numpy(a).to(dev) for a in idxF]
        # the same, flattened, for the native kernels
        self.ext_cat = torch.cat([e.to(torch.int32) for e in self.ext]) if self.ext else \
            torch.zeros(1, dtype=torch.int32, device=dev)
        self.ext_off = np.concatenate([[0], np.cumsum([len(e) for e in self.ext])]).astype(np.int64)
        if len(self.ext_off) < npan:
            self.ext_off = np.concatenate([self.ext_off, np.zeros(npan - len(self.ext_off), np.int64)])
        self.idx_cat = torch.from_numpy(all_ids).to(dev)
        self.idx_off = np.concatenate([[0], np.cumsum(n_sz)]).astype(np.int64)
        self.buf = torch.zeros(int(self.off[-1]), dtype=torch.float64, device=dev)
        self.crow = rp
        self.col = ci
        pf = self.p_sz.astype(float)
        ff = self.f_sz.astype(float)
        self.flops = float((2.0 / 3.0 * pf ** 3 + 2.0 * pf ** 2 * ff + 2.0 * ff ** 2 * pf).sum())

    def _create_native(self):
        import ctypes
        from . import vefem as V
        L = V.load()
        self._L = L
        h = ctypes.c_void_p()
        n32 = self.n_sz.astype(np.int32)
        p32 = self.p_sz.astype(np.int32)
        off = self.off.astype(np.int64)
        rc = L.vefem_frontal_create(self.dev.index or 0, self.npan, off.ctypes.data,
                                    n32.ctypes.data, p32.ctypes.data, self.ext_cat.data_ptr(),
                                    self.ext_off.ctypes.data, self.idx_cat.data_ptr(),
                                    self.idx_off.ctypes.data, self.N, ctypes.byref(h))
        if rc != 0:
            raise V.VefemError(f"vefem_frontal_create failed ({rc})")
        self._handle = h

    @property
    def solve_path(self):
        """How the last native solve's launches were chained: 1 programmatic
        dependent launch, 2 plain stream order, -1 no solve yet."""
        if self._handle is None:
            return -1
        return int(self._L.vefem_frontal_solve_path(self._handle))

    def close(self):
        if self._handle is not None:
            self._L.vefem_frontal_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ numeric
    def factor(self, vals):
        """Factorise the matrix with AIJ values ``vals`` (host array or device
        tensor, FP32 or FP64; FP32 values are widened)."""
        torch = self.torch
        if isinstance(vals, np.ndarray):
            v = torch.from_numpy(np.ascontiguousarray(vals, dtype=np.float64)).to(self.dev)
        else:
            # a copy: the caller's buffer is overwritten by the next assembly
            # while this factorisation is still in use
            v = vals.to(device=self.dev, dtype=torch.float64, copy=True)
        self.vals = v
        self._since_factor = 0
        self._needs_checks = False
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")        # sparse CSR support is marked beta
            self.A = torch.sparse_csr_tensor(self.crow, self.col, v, size=(self.N, self.N),
                                             check_invariants=False)
        self._host = None
        if self.method == "native":
            if self._factor_native(v):
                return self
            if not self.delay_pressure and self.p_field is not None:
                # a refused pivot: redo the symbolic phase with the pressures
                # delayed to their element-mates' panels, keep it, retry
                self.delay_pressure = True
                self.resymbolised = True
                self.close()
                self.buf = None
                en = self.mesh.element_nodes()
                self._symbolic(en, self.mesh.xyz[0][en].mean(axis=1))
                self._create_native()
                if self._factor_native(v):
                    return self
        return self._factor_pivoted(v)

    def _scatter(self, v):
        self.buf.zero_()
        self.buf[self.dest] = v

    def _factor_native(self, v) -> bool:
        """Unpivoted Gauss-Jordan elimination in the library; False when a
        pivot fails its test (the caller factorises with pivoting instead)."""
        import ctypes
        from . import vefem as V
        torch = self.torch
        self._scatter(v)
        mp = ctypes.c_double(0.0)
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        rc = self._L.vefem_frontal_factor(self._handle, self.buf.data_ptr(), stream,
                                          self.pivot_tol, ctypes.byref(mp))
        self.min_pivot = mp.value
        if rc == V.VEFEM_ERR_SINGULAR:
            self.pivoted_factorisations += 1
            return False
        if rc != 0:
            raise V.VefemError("vefem_frontal_factor: " +
                               self._L.vefem_frontal_last_error(self._handle).decode())
        self.mode = "native"
        return True

    def _factor_pivoted(self, v):
        torch = self.torch
        buf = self.buf
        self._scatter(v)
        self.mode = "pivoted"
        facs, infos = [], []
        S = None
        for q in range(self.npan):
            n, p, f = int(self.n_sz[q]), int(self.p_sz[q]), int(self.f_sz[q])
            o = int(self.off[q])
            M = buf[o:o + n * n].view(n, n)
            if S is not None:
                e = self.ext[q - 1]
                M[e[:, None], e[None, :]] += S
            if p == 0:
                S = M
                facs.append(None)
                continue
            LU, piv, info = torch.linalg.lu_factor_ex(M[:p, :p])
            infos.append(info)
            X = torch.linalg.lu_solve(LU, piv, M[:p, p:]) if f else None
            S = torch.addmm(M[p:, p:], M[p:, :p], X, beta=1.0, alpha=-1.0) if f else None
            facs.append((LU, piv, X, M[p:, :p] if f else None))
        self._factors = facs
        bad = int(torch.stack(infos).max().item()) if infos else 0
        if bad > 0:
            self._to_host()
        return self

    HOST_MAX_UNKNOWNS = 300_000

    def _to_host(self):
        """Factorise on the host instead (a zero pivot, or a solve that stays
        inaccurate after refinement).  Above HOST_MAX_UNKNOWNS the host LU
        runs out of memory (SuperLU's 32-bit indices overflow around a
        million unknowns), so the factorisation fails with RuntimeError at
        once, which the Newton drivers treat as a failed solve."""
        from . import linsolve as LS
        if self.N > self.HOST_MAX_UNKNOWNS:
            raise RuntimeError(f"no pivot-stable factorisation on the device and {self.N} "
                               f"unknowns are beyond the host fallback")
        self.fallbacks += 1
        self._host = LS.SparseLU(self.rowptr, self.colind, self.mesh, neq=self.neq)
        self._host.factor(self.vals.cpu().numpy())

    def _sweep(self, b):
        torch = self.torch
        if self.mode == "native":
            b = b.contiguous()
            x = torch.empty_like(b)
            stream = torch.cuda.current_stream(self.dev).cuda_stream
            rc = self._L.vefem_frontal_solve(self._handle, self.buf.data_ptr(), b.data_ptr(),
                                             x.data_ptr(), stream)
            if rc != 0:
                from . import vefem as V
                raise V.VefemError("vefem_frontal_solve: " +
                                   self._L.vefem_frontal_last_error(self._handle).decode())
            return x
        y = b.clone()
        ys = []
        for q, fac in enumerate(self._factors):
            if fac is None:
                ys.append(None)
                continue
            LU, piv, X, MFP = fac
            yP = torch.linalg.lu_solve(LU, piv, y[self.idxP[q]].unsqueeze(1)).squeeze(1)
            if MFP is not None:
                y.index_add_(0, self.idxF[q], MFP @ yP, alpha=-1.0)
            ys.append(yP)
        x = torch.empty_like(b)
        for q in range(self.npan - 1, -1, -1):
            fac = self._factors[q]
            if fac is None:
                continue
            LU, piv, X, MFP = fac
            xP = ys[q]
            if X is not None:
                xP = xP - X @ x[self.idxF[q]]
            x[self.idxP[q]] = xP
        return x

    def precondition(self, b):
        """The last factorisation's solve as a preconditioner: the sweeps only,
        without the residual check (a device tensor in, a device tensor out;
        a host array goes through solve)."""
        if self._host is not None or isinstance(b, np.ndarray):
            return self.solve(b)
        return self._sweep(b.to(device=self.dev, dtype=self.torch.float64))

    def solve(self, b):
        """Solve with the last factorisation; ``b`` a host array (returns a host
        array) or a device tensor (returns a device tensor).

        The first solve after a factorisation (and every ``check_every``-th
        after it, and every one once a refinement was needed) is checked
        against the CSR matrix and refined up to ``refine`` times; the
        backward error of an unpivoted elimination is a property of its
        factors, so a factorisation that passes on its first right-hand side
        passes on the next ones."""
        torch = self.torch
        host = isinstance(b, np.ndarray)
        if self._host is not None:
            if host:
                return self._host.solve(b)
            return torch.from_numpy(self._host.solve(b.cpu().numpy())).to(b.device)
        if host:
            if self._hb is None or self._hb.numel() != self.N:
                pin = self.dev.type == "cuda"
                self._hb = torch.empty(self.N, dtype=torch.float64, pin_memory=pin)
                self._hx = torch.empty(self.N, dtype=torch.float64, pin_memory=pin)
            self._hb.numpy()[:] = b
            bt = self._hb.to(self.dev, non_blocking=True)
        else:
            bt = b.to(device=self.dev, dtype=torch.float64)
        x = self._sweep(bt)
        check = (self._since_factor % self.check_every == 0) or self._needs_checks
        self._since_factor += 1
        if check:
            nb = float(torch.linalg.vector_norm(bt))
            ok = False
            for k in range(self.refine + 1):
                r = bt - self.A @ x
                rn = float(torch.linalg.vector_norm(r))
                if math.isfinite(rn) and rn <= self.check_tol * max(nb, 1e-300):
                    ok = True
                    break
                if k == self.refine or not math.isfinite(rn):
                    break
                x = x + self._sweep(r)
                self.refinements += 1
                self._needs_checks = True
            if not ok:
                self._to_host()
                xh = self._host.solve(bt.cpu().numpy())
                return xh if host else torch.from_numpy(xh).to(b.device)
        if not host:
            return x
        self._hx.copy_(x, non_blocking=True)
        if self.dev.type == "cuda":
            torch.cuda.current_stream(self.dev).synchronize()
        return self._hx.numpy().copy()
