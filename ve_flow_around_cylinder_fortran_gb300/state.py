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
(Nnodes), p (Nnodes), A (Nnodes x 2 x 2).

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
    """c [n, 2, 2] SPD -> (Txx, Txy, Tyy) or (Sxx, Sxy, Syy) per node, [3, n]."""
    if phys.form == "SQRT":
        w, v = np.linalg.eigh(c)
        s = np.einsum("nij,nj,nkj->nik", v, np.sqrt(w), v)
        return np.stack([s[:, 0, 0], s[:, 0, 1], s[:, 1, 1]])
    t = (1.0 - phys.BvN) / phys.WiN * (c - np.eye(2)[None])
    return np.stack([t[:, 0, 0], t[:, 0, 1], t[:, 1, 1]])


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
    c = np.eye(2)[None] + 0.1 * np.einsum("nij,nkj->nik", A, A)
    TL = np.empty((6, n))
    TL[0], TL[1], TL[2] = u, v, p
    TL[3:] = conformation_to_unknowns(c, phys)
    EU = np.full(phys.nex, arn, dtype=np.float64)
    if phys.nex:
        phys.Wi0 = phys.WiN / arn
    return np.ascontiguousarray(TL), EU
