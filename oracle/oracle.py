"""ctypes wrapper of the C oracle (vefem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, the smoke check and the
CPU-baseline leg of the benchmark, never by the product.  The shared object is
built by ``oracle/build.sh`` into ``oracle/_build/`` (git-ignored).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "libvefem_oracle.so")
SO_CS = os.path.join(HERE, "_build", "libvefem_oracle_cs.so")

_lib = None
_cs = None


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("vefem_oracle.c", "vefem_stability_oracle.c",
                                           "build.sh")]
    if force or not os.path.exists(SO) or not os.path.exists(SO_CS) or any(
            os.path.getmtime(x) < os.path.getmtime(f) for f in srcs for x in (SO, SO_CS)):
        subprocess.check_call(["bash", os.path.join(HERE, "build.sh")])
    return SO


def build_flags() -> str:
    """Compiler and flags the oracle library was built with."""
    path = os.path.join(HERE, "_build", "flags.txt")
    return open(path).read().strip() if os.path.exists(path) else "unknown"


def cpu_model() -> str:
    """Host CPU model name (x86 'model name', or the Arm implementer/part)."""
    try:
        txt = open("/proc/cpuinfo").read()
    except OSError:
        return "unknown"
    for line in txt.splitlines():
        if line.lower().startswith("model name"):
            return line.split(":", 1)[1].strip()
    parts = {}
    for line in txt.splitlines():
        if ":" in line:
            k, v = line.split(":", 1)
            parts.setdefault(k.strip(), v.strip())
    arm_parts = {"0xd4f": "Neoverse-V2", "0xd40": "Neoverse-V1", "0xd0c": "Neoverse-N1"}
    if "CPU part" in parts:
        return "Arm " + arm_parts.get(parts["CPU part"], "part " + parts["CPU part"])
    return "unknown"


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(SO)
        P = ctypes.c_void_p
        I = ctypes.c_int
        L.ora_element_batch.argtypes = [P, P, I, I, P, P, P, P, I, I, P, P, P, I]
        L.ora_assemble.argtypes = [P, P, I, I, P, P, P, P, I, P, P, P, P, I]
        L.ora_edge_open.argtypes = [P, P, I, I, P, P, P, P, I, I, P, P, P]
        L.ora_gp_probe.argtypes = [P, P, I, I, P, P, P, P, I, P]
        L.ora_gauss_tables.argtypes = [P, P]
        D = ctypes.c_double
        L.ora_stability_batch.argtypes = [P, P, D, I, I, I, P, P, P, P, I, I, P, P, P, P, I]
        L.ora_stability_batch.restype = I
        for f in (L.ora_element_batch, L.ora_assemble, L.ora_edge_open, L.ora_gp_probe):
            f.restype = I
        _lib = L
    return _lib


def cs_lib():
    """The oracle built on complex numbers (complex-step exact Jacobian)."""
    global _cs
    if _cs is None:
        build()
        L = ctypes.CDLL(SO_CS)
        P = ctypes.c_void_p
        I = ctypes.c_int
        L.ora_cs_element_batch.argtypes = [P, P, I, I, P, P, P, P, I, I, P, P, P, I]
        L.ora_cs_element_batch.restype = I
        _cs = L
    return _cs


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _prep(phys, conn, xyz, TL, EU):
    ip = np.ascontiguousarray(phys.int_params(), dtype=np.int32)
    dp = np.ascontiguousarray(phys.dbl_params(), dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    TL = np.ascontiguousarray(TL, dtype=np.float64)
    EU = np.ascontiguousarray(EU if EU is not None and len(EU) else np.zeros(1), dtype=np.float64)
    return ip, dp, conn, xyz, TL, EU


def gauss_tables():
    t = np.zeros((6, 9, 9))
    w = np.zeros(9)
    lib().ora_gauss_tables(_p(t), _p(w))
    return t, w


def element_outputs(phys, conn, xyz, TL, EU, e0=0, e1=None, jacobian=True, nthreads=0):
    """Element residuals [n, 9, 6], FD Jacobians [n, 9, 6, 9, 6] (TEMP_A_f(inod,ieq,jnod,jeq))
    and Ac columns [n, 9, 6, nex] for elements [e0, e1)."""
    ip, dp, conn, xyz, TL, EU = _prep(phys, conn, xyz, TL, EU)
    nel = conn.shape[1]
    nn = xyz.shape[1]
    e1 = nel if e1 is None else e1
    n = e1 - e0
    res = np.zeros((n, 9, 6))
    jac = np.zeros((n, 9, 6, 9, 6)) if jacobian else None
    ac = np.zeros((n, 9, 6, max(phys.nex, 1))) if jacobian else None
    rc = lib().ora_element_batch(_p(ip), _p(dp), nel, nn, _p(conn), _p(xyz), _p(TL), _p(EU), e0,
                                 e1, _p(res), _p(jac), _p(ac), nthreads)
    assert rc == 0
    return res, jac, (ac[..., :phys.nex] if ac is not None else None)


def assemble(phys, conn, xyz, TL, EU, rowptr, colind, jacobian=True, nthreads=0, b=None,
             vals=None):
    """Global residual b and CSR values (ADD semantics onto the given arrays)."""
    ip, dp, conn, xyz, TL, EU = _prep(phys, conn, xyz, TL, EU)
    nel = conn.shape[1]
    nn = xyz.shape[1]
    N = rowptr.shape[0] - 1
    b = np.zeros(N) if b is None else b
    vals = np.zeros(colind.shape[0]) if vals is None else vals
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    colind = np.ascontiguousarray(colind, dtype=np.int32)
    rc = lib().ora_assemble(_p(ip), _p(dp), nel, nn, _p(conn), _p(xyz), _p(TL), _p(EU),
                            1 if jacobian else 0, _p(rowptr), _p(colind), _p(b),
                            _p(vals) if jacobian else None, nthreads)
    if rc != 0:
        raise RuntimeError("oracle assembly: element entry missing from the CSR pattern")
    return b, vals


def edge_open(phys, conn, xyz, TL, EU, iel, ied, jacobian=True):
    ip, dp, conn, xyz, TL, EU = _prep(phys, conn, xyz, TL, EU)
    res = np.zeros((9, 6))
    jac = np.zeros((9, 6, 9, 6)) if jacobian else None
    ac = np.zeros((9, 6, max(phys.nex, 1))) if jacobian else None
    lib().ora_edge_open(_p(ip), _p(dp), conn.shape[1], xyz.shape[1], _p(conn), _p(xyz), _p(TL),
                        _p(EU), int(iel), int(ied), _p(res), _p(jac), _p(ac))
    return res, jac, (ac[..., :phys.nex] if ac is not None else None)


def gp_probe(phys, conn, xyz, TL, EU, iel):
    """Per-Gauss-point [Momentum x/y, Continuity, Con_EQ 11/12/22, tlsme, tlsic, tlsce, tdcs, WET]."""
    ip, dp, conn, xyz, TL, EU = _prep(phys, conn, xyz, TL, EU)
    out = np.zeros((9, 11))
    lib().ora_gp_probe(_p(ip), _p(dp), conn.shape[1], xyz.shape[1], _p(conn), _p(xyz), _p(TL),
                       _p(EU), int(iel), _p(out))
    return out


def stability_elements(phys, conn, xyz, TLb, TLd, KwN: float, kz: bool = True, jacobian=True,
                       e0: int = 0, e1: int | None = None, nthreads: int = 0):
    """Stability element outputs (vefem_stability_oracle.c): Res_a, Res_b
    [nel][9][10] and the FD blocks A, B [nel][9][10][9][10] (inod, ieq, jnod, jeq)."""
    L = lib()
    ip = np.ascontiguousarray(phys.int_params(), dtype=np.int32)
    dp = np.ascontiguousarray(phys.dbl_params(), dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    TLb = np.ascontiguousarray(TLb, dtype=np.float64)
    TLd = np.ascontiguousarray(TLd, dtype=np.float64)
    nel = conn.shape[1]
    nnodes = TLb.shape[1]
    e1 = nel if e1 is None else e1
    n = e1 - e0
    ra = np.zeros((n, 9, 10))
    rb = np.zeros((n, 9, 10))
    A = np.zeros((n, 9, 10, 9, 10)) if jacobian else None
    B = np.zeros((n, 9, 10, 9, 10)) if jacobian else None
    rc = L.ora_stability_batch(_p(ip), _p(dp), float(KwN), 1 if kz else 0, nel, nnodes, _p(conn),
                               _p(xyz), _p(TLb), _p(TLd), e0, e1, _p(ra), _p(rb), _p(A), _p(B),
                               nthreads)
    if rc:
        raise ValueError(f"ora_stability_batch: {rc} (T form only)")
    return ra, rb, A, B


def exact_element_outputs(phys, conn, xyz, TL, EU, e0=0, e1=None, nthreads=0):
    """Element residuals [n, 9, 6], exact Jacobians [n, 9, 6, 9, 6] by the
    complex step (layout of element_outputs) and exact Ac columns [n, 9, 6, nex]."""
    ip, dp, conn, xyz, TL, EU = _prep(phys, conn, xyz, TL, EU)
    nel = conn.shape[1]
    nn = xyz.shape[1]
    e1 = nel if e1 is None else e1
    n = e1 - e0
    res = np.zeros((n, 9, 6))
    jac = np.zeros((n, 9, 6, 9, 6))
    ac = np.zeros((n, 9, 6, max(phys.nex, 1)))
    rc = cs_lib().ora_cs_element_batch(_p(ip), _p(dp), nel, nn, _p(conn), _p(xyz), _p(TL),
                                       _p(EU), e0, e1, _p(res), _p(jac), _p(ac), nthreads)
    assert rc == 0
    return res, jac, ac[..., :phys.nex]


def exact_assemble(phys, conn, xyz, TL, EU, rowptr, colind, nthreads=0):
    """Exact (complex-step) Jacobian of the bulk assembly into CSR values:
    row (jnod, jeq) equation, column (inod, ieq) unknown, and the arclength
    column (the last entry of every node row), added in element order
    (storeResidual / storeJacobian / storeJacobian_Ac, Storage_mod.F90:10-115).
    Returns (b, vals)."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    nel = conn.shape[1]
    en = conn.T.astype(np.int64) - 1
    N = len(rowptr) - 1
    rowptr = np.asarray(rowptr, dtype=np.int64)
    colind = np.asarray(colind, dtype=np.int64)
    keys = np.repeat(np.arange(N, dtype=np.int64), np.diff(rowptr)) * N + colind
    b = np.zeros(N)
    vals = np.zeros(len(colind))
    chunk = 2048
    for e0 in range(0, nel, chunk):
        e1 = min(nel, e0 + chunk)
        res, jac, ac = exact_element_outputs(phys, conn, xyz, TL, EU, e0, e1, nthreads)
        dof = (en[e0:e1, :, None] * 6 + np.arange(6)[None, None, :]).reshape(e1 - e0, 54)
        np.add.at(b, dof.reshape(-1), res.reshape(-1))
        # A[row = (jnod, jeq), col = (inod, ieq)] = jac[inod, ieq, jnod, jeq]
        blk = jac.reshape(e1 - e0, 54, 54).transpose(0, 2, 1)
        q = (dof[:, :, None] * N + dof[:, None, :]).reshape(-1)
        slots = np.searchsorted(keys, q)
        if np.any(slots >= len(keys)) or np.any(keys[np.minimum(slots, len(keys) - 1)] != q):
            raise RuntimeError("exact assembly: element entry missing from the pattern")
        np.add.at(vals, slots, blk.reshape(-1))
        if phys.nex:
            np.add.at(vals, rowptr[dof.reshape(-1) + 1] - 1, ac[..., 0].reshape(-1))
    return b, vals
