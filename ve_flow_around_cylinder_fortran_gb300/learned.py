"""Learned predictor for the arclength continuation.

The reference predicts the next continuation point with the tangent step
x_p = x + t dS (updateSolutionArclength, Continuation_Arclength_mod.F90:339-379).
This module adds a learned prediction in a reduced space:

* POD: the converged snapshots x_1..x_m (state vector [TL, lambda]) are
  centred on their mean and decomposed by the method of snapshots (Gram
  matrix on the GPU, its eigenvectors on the host, modes re-orthonormalised
  by Cholesky QR); up to ``n_modes`` modes Phi with coefficients
  a_j = Phi^T (x_j - mean).
* Network: the library's multilayer perceptron (vefem.MLP: 3 GELU layers of
  width 256, BF16 weights, FP32 accumulation, trained by the library's own
  forward, backward and Adam kernels).  Input of the sample for point j:
  Wi_{j-1}, the arclength step ds_j = s_j - s_{j-1}, the last coefficient
  vector a_{j-1} and the two last slopes (a_{j-1} - a_{j-2}) / ds_{j-1},
  (a_{j-2} - a_{j-3}) / ds_{j-2} (the last three coefficient vectors in
  difference form).  Output: the slope (a_j - a_{j-1}) / ds_j minus the
  slope of the polynomial extrapolation in s through the last ``order`` + 1
  points (cubic by default); an output of zero is that extrapolation.  Inputs
  and outputs are standardised over the training set.
* Online training: once ``start`` points have converged (20), the network is
  trained, and retrained (warm start) on all samples after every converged
  point; the basis is rebuilt after every point from ``predict_from`` (4) on.
* Prediction: a = a_m + dS (poly + net(...)) with poly the extrapolated
  slope (the network term only once it is trained), and the candidate
  x = mean + Phi a.  The
  candidate does not use the tangent: the tangent is solved with the last
  factorised Jacobian, taken at the first Newton iterate rather than at the
  converged point, and most of the tangent step's error lies outside the
  span of the converged snapshots.

Newton stays the corrector and the judge: of the tangent prediction, the
extrapolation and the network-corrected extrapolation the continuation
takes the one of the smallest residual norm (ArclengthContinuation._judge),
so an untrained or mistaken network costs one residual evaluation and
never a worse starting point.
"""
from __future__ import annotations

import time

import numpy as np


class LearnedPredictor:
    def __init__(self, n_modes: int = 32, start: int = 20, width: int = 256, hidden: int = 3,
                 iters: int = 400, lr: float = 1.0e-3, seed: int = 0, device: str = "cuda:0",
                 net=None, log=None, use_net: bool = True, order: int = 3,
                 predict_from: int | None = 4):
        import torch
        self.torch = torch
        self.dev = torch.device(device)
        # the network trains once ``start`` points have converged; the
        # reduced-space extrapolation predicts from ``predict_from`` points on
        # (by default from ``start``), with the network's correction added
        # once it is trained
        self.n_modes, self.start = n_modes, start
        self.predict_from = start if predict_from is None else predict_from
        if self.predict_from < 4:
            raise ValueError("the reduced extrapolation needs 4 converged points")
        self.trained = False
        self.iters, self.lr = iters, lr
        self.in_dim = 2 + 3 * n_modes
        if net is None:
            from . import vefem as V
            net = V.MLP(self.in_dim, n_modes, width=width, hidden=hidden, seed=seed,
                        device=self.dev.index or 0)
        self.net = net
        self.log = log
        self.X = []          # snapshots (device tensors)
        self.wi = []
        self.s = [0.0]       # cumulative chord length at each snapshot
        self.basis = None    # (mean, Phi)
        self.norm = None     # (xm, xs, ym, ys)
        self.coef = None     # [m][r] coefficients of the snapshots
        self.last_loss = None
        self.trainings = 0
        self.timers = {"pod": 0.0, "train": 0.0, "predict": 0.0}
        # use_net = False: the ablation without the network (the reduced-space
        # quadratic extrapolation alone)
        self.use_net = use_net
        # degree of the polynomial extrapolation in s the network corrects
        # (3: the cubic through the last four points)
        if order < 1:
            raise ValueError("extrapolation order must be >= 1")
        self.order = order

    def warm_up(self, n: int, m: int = 6):
        """Run the predictor's own code path (observe: snapshot upload, chord
        length, Gram matrix and mode re-orthonormalisation; candidates:
        features, extrapolation and reconstruction) on ``m`` or more synthetic
        snapshots of length ``n``, without the network, so that the
        framework's first-use costs (lazy loading and JIT of its kernels,
        seconds on a fresh process) fall outside a timed continuation.  The
        predictor's state is restored afterwards."""
        torch = self.torch
        keys = ("X", "wi", "s", "basis", "coef", "norm", "trained", "trainings", "last_loss",
                "use_net")
        saved = {k: getattr(self, k) for k in keys}
        saved_timers = dict(self.timers)
        rng = np.random.default_rng(0)
        x0, d1, d2 = (rng.standard_normal(n) for _ in range(3))
        try:
            self.X, self.wi, self.s = [], [], [0.0]
            self.basis = self.coef = self.norm = None
            self.use_net = False
            for j in range(max(m, self.predict_from + 1)):
                self.observe(j + 1, x0 + j * d1 + 0.1 * j * j * d2, 0.1 * (j + 1))
            x1 = x0 + j * d1
            self.candidates(j + 2, x1, d1 / np.linalg.norm(d1), 1.0, x1 + d1)
        finally:
            for k, v in saved.items():
                setattr(self, k, v)
            self.timers = saved_timers
        if self.dev.type == "cuda":
            torch.cuda.synchronize(self.dev)

    # ---- data --------------------------------------------------------------
    def observe(self, k: int, x: np.ndarray, wi: float):
        t = self.torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(self.dev)
        if self.X:
            self.s.append(self.s[-1] + float(self.torch.linalg.vector_norm(t - self.X[-1])))
        self.X.append(t)
        self.wi.append(float(wi))
        if len(self.X) >= min(self.start, self.predict_from):
            self._fit()

    def _pod(self):
        torch = self.torch
        Xm = torch.stack(self.X, dim=1)                       # N x m
        mean = Xm.mean(dim=1)
        Xc = Xm - mean[:, None]
        G = (Xc.T @ Xc).cpu().numpy()
        lam, V = np.linalg.eigh(G)
        order = np.argsort(lam)[::-1]
        lam, V = lam[order], V[:, order]
        keep = lam > lam[0] * 1e-14          # drop round-off directions
        r = min(self.n_modes, int(keep.sum()))
        lam, V = lam[:r], V[:, :r]
        W = torch.from_numpy(V / np.sqrt(lam)).to(self.dev)
        # re-orthonormalised (two passes of Cholesky QR, the r x r factors on
        # the host): the snapshot method loses orthogonality in the weak modes
        # by round-off ~ eps * lam_0 / lam_i
        Phi = Xc @ W                                          # N x r
        for _ in range(2):
            Lc = np.linalg.cholesky((Phi.T @ Phi).cpu().numpy())
            Phi = Phi @ torch.from_numpy(np.linalg.inv(Lc).T.copy()).to(self.dev)
        if self.basis is not None:                            # keep mode signs stable
            old = self.basis[1]
            rr = min(r, old.shape[1])
            sgn = torch.sign((Phi[:, :rr] * old[:, :rr]).sum(dim=0))
            sgn[sgn == 0] = 1.0
            Phi[:, :rr] *= sgn
        coef = (Phi.T @ Xc).T.cpu().numpy()                   # m x r
        if r < self.n_modes:
            coef = np.pad(coef, ((0, 0), (0, self.n_modes - r)))
        return mean, Phi, coef

    def _features(self, j: int, ds_j: float, coef: np.ndarray):
        """Network input of the sample for point j (0-based, j >= 3) and the
        quadratic-extrapolation slope of the step s_{j-1} -> s_j."""
        ds1 = self.s[j - 1] - self.s[j - 2]
        ds2 = self.s[j - 2] - self.s[j - 3]
        sl1 = (coef[j - 1] - coef[j - 2]) / ds1
        sl2 = (coef[j - 2] - coef[j - 3]) / ds2
        q = min(self.order, j - 1)
        if q == 2:
            # slopes are derivatives at interval midpoints: exact for a quadratic a(s)
            quad = sl1 + (sl1 - sl2) * (ds_j + ds1) / (ds1 + ds2)
        else:
            # Lagrange extrapolation through the last q + 1 points
            sn = self.s[j - 1] + ds_j
            nodes = self.s[j - 1 - q:j]
            ext = np.zeros_like(coef[0])
            for i in range(q + 1):
                w = 1.0
                for l in range(q + 1):
                    if l != i:
                        w *= (sn - nodes[l]) / (nodes[i] - nodes[l])
                ext = ext + w * coef[j - 1 - q + i]
            quad = (ext - coef[j - 1]) / ds_j
        return np.concatenate([[self.wi[j - 1], ds_j], coef[j - 1], sl1, sl2]), quad

    def _dataset(self, coef):
        X, Y = [], []
        for j in range(max(3, self.order + 1), len(self.X)):
            ds = self.s[j] - self.s[j - 1]
            f, quad = self._features(j, ds, coef)
            X.append(f)
            Y.append((coef[j] - coef[j - 1]) / ds - quad)
        return np.array(X), np.array(Y)

    def _fit(self):
        t0 = time.perf_counter()
        mean, Phi, coef = self._pod()
        self.basis, self.coef = (mean, Phi), coef
        t1 = time.perf_counter()
        if self.use_net and len(self.X) >= self.start:
            X, Y = self._dataset(coef)
            xm, xs = X.mean(axis=0), X.std(axis=0)
            ym, ys = Y.mean(axis=0), Y.std(axis=0)
            xs = np.where(xs > 1e-12 * max(1.0, np.abs(xm).max()), xs, 1.0)
            ys = np.where(ys > 1e-30, ys, 1.0)
            self.norm = (xm, xs, ym, ys)
            self.net.reset_optimizer()
            self.last_loss = self.net.train((X - xm) / xs, (Y - ym) / ys, self.iters, self.lr)
            self.trained = True
            self.trainings += 1
            if self.log:
                self.log(f"learned predictor: {len(self.X)} snapshots, {Phi.shape[1]} modes, "
                         f"training loss {self.last_loss:.3e}")
        self.timers["pod"] += t1 - t0
        self.timers["train"] += time.perf_counter() - t1

    # ---- prediction --------------------------------------------------------
    def candidates(self, k: int, x_o: np.ndarray, t: np.ndarray, dS: float,
                   x_plain: np.ndarray):
        """The reduced-space candidates for the next point, best first:
        [("learned", extrapolation + network)] once the network is trained,
        then ("extrapolation", the polynomial extrapolation alone); empty
        before ``predict_from`` points have converged."""
        if self.basis is None or len(self.X) < self.predict_from:
            return []
        t0 = time.perf_counter()
        torch = self.torch
        mean, Phi = self.basis
        m = len(self.X)
        coef = self.coef
        r = Phi.shape[1]
        f, poly = self._features(m, dS, coef)
        steps = []
        if self.trained:
            xm, xs, ym, ys = self.norm
            dy = self.net.forward(((f - xm) / xs)[None, :])[0].astype(np.float64) * ys + ym
            steps.append(("learned", poly + dy))
        steps.append(("extrapolation", poly))
        out = []
        for name, slope in steps:
            a = coef[m - 1] + dS * slope
            out.append((name, (mean + Phi @ torch.from_numpy(a[:r]).to(self.dev)).cpu().numpy()))
        self.timers["predict"] += time.perf_counter() - t0
        return out

    def predict(self, k: int, x_o: np.ndarray, t: np.ndarray, dS: float, x_plain: np.ndarray):
        """The first candidate (the network-corrected one once trained), or None."""
        c = self.candidates(k, x_o, t, dS, x_plain)
        return c[0][1] if c else None
