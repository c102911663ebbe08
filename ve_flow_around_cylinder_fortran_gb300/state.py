"""Seeded synthetic nodal states and physical parameters.

The reference has no shipped states or benchmark inputs; its runs start from
continuation.  These seeded states stand in for them, with the distribution
the workloads are quoted on:

* u = 1.5 (1 - (y/H)^2) * mask + N(0, 0.01^2),  mask = clip((r - R) / 0.25, 0, 1)
* v = N(0, 0.01^2),  p = N(0, 0.01^2)
* conformation c = I + 0.1 A A^T with A ~ N(0, 0.1^2) per node (SPD)
* T form unknowns (polymer stress, inverse of setStressTensor,
  Constitutive_Models_mod.F90:346-347 with g = 1): T = (1 - beta)/Wi (c - I)
* SQRT form unknowns: S = c^(1/2) (symmetric square root)

Draw order from ``numpy.random.default_rng(seed)``: u-noise (Nnodes), v
(Nnodes), p (Nnodes), A (Nnodes x 2 x 2).  ``portable_state`` draws uniform
numbers instead (exact across machines) for fixtures whose bits are recorded.

Field order and layout follow the reference: TL(Nnodes, Neq) column-major,
i.e. a C array [6, Nnodes] with rows Ux, Uy, P, Txx, Txy, Tyy
(Tools_mod.F90:622-649).
"""
from __future__ import annotations

import dataclasses

import numpy as np

MODELS = {"L-PTT": 0, "m-L-PTT": 1, "e-PTT": 2, "m-e-PTT": 3, "FENE-CR": 4, "FENE-P": 5,
          "GIESEKUS": 6}
FORMS = {"T": 0, "SQRT": 1}
HUGE = float(np.finfo(np.float64).max)   # dt = huge(1d0) in steady runs (Physical_mod.F90:345)


@dataclasses.dataclass
class Physics:
    """Run-time restatement of the reference's compile-time physics parameters
    (Parameters_mod.F90:98-122).  ``nex`` = 1 means arclength continuation in
    Wi: WiN = Wi0 * EU(Nex) at every Gauss point
    (Element_Calculations_mod.F90:577-601); ``nex`` = 0 uses ``WiN``."""
    model: str = "L-PTT"
    form: str = "T"
    ReN: float = 0.0
    WiN: float = 0.1
    BvN: float = 0.59
    VeN: float = 0.0
    DfN: float = 0.0
    Wi0: float = 0.1
    nex: int = 1
    dt: float = HUGE
    eps: float = 1.0e-8

    def int_params(self) -> np.ndarray:
        return np.array([MODELS[self.model], FORMS[self.form], self.nex], dtype=np.int32)

    def dbl_params(self) -> np.ndarray:
        return np.array([self.ReN, self.WiN, self.BvN, self.VeN, self.DfN, self.Wi0, self.dt,
                         self.eps], dtype=np.float64)

    @property
    def wi_effective(self) -> float:
        return self.WiN


def oldroyd_b(Wi: float = 0.1, beta: float = 0.59, form: str = "T", nex: int = 1,
              DfN: float = 0.0) -> Physics:
    """Oldroyd-B = L-PTT with epsilon (VeN) = 0 (Constitutive_Models_mod.F90:96-117)."""
    return Physics(model="L-PTT", form=form, WiN=Wi, Wi0=Wi, BvN=beta, VeN=0.0, nex=nex, DfN=DfN)


def giesekus(alpha: float = 0.1, Wi: float = 0.5, beta: float = 0.59, form: str = "SQRT",
             nex: int = 1, DfN: float = 0.0) -> Physics:
    return Physics(model="GIESEKUS", form=form, WiN=Wi, Wi0=Wi, BvN=beta, VeN=alpha, nex=nex,
                   DfN=DfN)


def conformation_to_unknowns(c: np.ndarray, phys: Physics) -> np.ndarray:
    """c [n, 2, 2] SPD -> (Txx, Txy, Tyy) or (Sxx, Sxy, Syy) per node, [3, n].

    The square root of a 2x2 SPD matrix is taken in closed form,
    S = (c + sqrt(det c) I) / sqrt(tr c + 2 sqrt(det c)), with elementwise
    IEEE operations only, so the same seed gives the same bits on every
    machine (a LAPACK eigensolver would not)."""
    a, b, d = c[:, 0, 0], c[:, 0, 1], c[:, 1, 1]
    if phys.form == "SQRT":
        sd = np.sqrt(a * d - b * b)
        t = np.sqrt(a + d + 2.0 * sd)
        return np.stack([(a + sd) / t, b / t, (d + sd) / t])
    k = (1.0 - phys.BvN) / phys.WiN
    return np.stack([k * (a - 1.0), k * b, k * (d - 1.0)])


def seeded_state(xyz: np.ndarray, phys: Physics, seed: int = 0, R: float = 1.0, H: float = 2.0,
                 arn: float = 1.0):
    """Return (TL [6, Nnodes] float64, EU [nex] float64)."""
    rng = np.random.default_rng(seed)
    x, y = xyz[0], xyz[1]
    n = x.shape[0]
    r = np.hypot(x, y)
    mask = np.clip((r - R) / 0.25, 0.0, 1.0)
    u = 1.5 * (1.0 - (y / H) ** 2) * mask + rng.normal(0.0, 0.01, n)
    v = rng.normal(0.0, 0.01, n)
    p = rng.normal(0.0, 0.01, n)
    A = rng.normal(0.0, 0.1, (n, 2, 2))
    c = np.empty((n, 2, 2))
    c[:, 0, 0] = 1.0 + 0.1 * (A[:, 0, 0] * A[:, 0, 0] + A[:, 0, 1] * A[:, 0, 1])
    c[:, 0, 1] = 0.1 * (A[:, 0, 0] * A[:, 1, 0] + A[:, 0, 1] * A[:, 1, 1])
    c[:, 1, 0] = c[:, 0, 1]
    c[:, 1, 1] = 1.0 + 0.1 * (A[:, 1, 0] * A[:, 1, 0] + A[:, 1, 1] * A[:, 1, 1])
    TL = np.empty((6, n))
    TL[0], TL[1], TL[2] = u, v, p
    TL[3:] = conformation_to_unknowns(c, phys)
    EU = np.full(phys.nex, arn, dtype=np.float64)
    if phys.nex:
        phys.Wi0 = phys.WiN / arn
    return np.ascontiguousarray(TL), EU


def portable_state(xyz: np.ndarray, phys: Physics, seed: int = 0, arn: float = 1.0):
    """A state built only from uniform draws (53-bit integers scaled by 2^-53)
    and elementwise IEEE operations, so its bits are the same on every
    machine: u in [1, 1.5), v and p in [-0.05, 0.05), conformation
    c = I + 0.1 B with B symmetric, entries in [-0.1, 0.1) (diagonal in [0, 0.1))."""
    rng = np.random.default_rng(seed)
    n = xyz.shape[1]
    r = rng.random((7, n))
    TL = np.empty((6, n))
    TL[0] = 1.0 + 0.5 * r[0]
    TL[1] = 0.1 * (r[1] - 0.5)
    TL[2] = 0.1 * (r[2] - 0.5)
    c = np.empty((n, 2, 2))
    c[:, 0, 0] = 1.0 + 0.1 * (0.1 * r[3])
    c[:, 0, 1] = 0.1 * (0.2 * (r[4] - 0.5))
    c[:, 1, 0] = c[:, 0, 1]
    c[:, 1, 1] = 1.0 + 0.1 * (0.1 * r[5])
    TL[3:] = conformation_to_unknowns(c, phys)
    EU = np.full(phys.nex, arn, dtype=np.float64)
    if phys.nex:
        phys.Wi0 = phys.WiN / arn
    return np.ascontiguousarray(TL), EU
