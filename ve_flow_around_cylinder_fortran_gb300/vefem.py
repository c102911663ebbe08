"""Python binding of the C ABI (include/vefem.h) through ctypes.

The class ``BulkAssembler`` mirrors the reference's call
``setEquationsBulk(Problem, FE, Mesh, Boundary, GaussInt, Sol, basis_p,
Flag_NR, Elem, LS)`` (Equations_mod.F90:21-55): ``set_equations_bulk(TL, EU,
flag_nr, b, vals)`` with ``flag_nr`` 'NRP' (residual and Jacobian) or 'MNR'
(residual only), adding into ``b`` and the AIJ ``vals`` like ADD_VALUES.

The library is loaded from this package's ``_build`` directory; there is no
CPU fallback: without the built library (or without a GPU) calls fail loudly.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libvefem.so")

VEFEM_RESIDUAL = 0x1
VEFEM_JAC_FD64 = 0x2
VEFEM_JAC_EXACT64 = 0x4
VEFEM_JAC_EXACT32 = 0x8
JACOBIANS = {"fd64": VEFEM_JAC_FD64, "exact64": VEFEM_JAC_EXACT64, "exact32": VEFEM_JAC_EXACT32}
VEFEM_ZERO_FIRST = 0x100
VEFEM_OUTLET_EDGES = 0x200
VEFEM_TIMING = 0x1000
VEFEM_STAB_AS_WRITTEN = 0x2000

EXPORTED = ["vefem_abi_version", "vefem_create", "vefem_set_params", "vefem_assemble",
            "vefem_last_timing", "vefem_last_launch_count", "vefem_stream", "vefem_destroy",
            "vefem_last_error", "vefem_build_pattern", "vefem_apply_dirichlet",
            "vefem_algorithmic_ops", "vefem_assemble_residual_noalloc",
            "vefem_mlp_create", "vefem_mlp_num_params", "vefem_mlp_set_params",
            "vefem_mlp_get_params", "vefem_mlp_forward", "vefem_mlp_loss_grad", "vefem_mlp_train",
            "vefem_mlp_reset_optimizer", "vefem_mlp_destroy", "vefem_mlp_last_error",
            "vefem_batch_create", "vefem_batch_set_params", "vefem_assemble_batched",
            "vefem_batch_autotune", "vefem_batch_set_tiles", "vefem_batch_info",
            "vefem_batch_last_timing", "vefem_batch_destroy", "vefem_batch_last_error",
            "vefem_stability_pattern", "vefem_stability_assemble",
            "vefem_frontal_create", "vefem_frontal_factor", "vefem_frontal_solve",
            "vefem_frontal_destroy", "vefem_frontal_last_error", "vefem_frontal_solve_path"]
VEFEM_ERR_SINGULAR = 6
BATCH_CLASSES = 6


class VefemError(RuntimeError):
    pass


class c_params(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("form", ctypes.c_int32), ("nex", ctypes.c_int32),
                ("device", ctypes.c_int32), ("ReN", ctypes.c_double), ("WiN", ctypes.c_double),
                ("BvN", ctypes.c_double), ("VeN", ctypes.c_double), ("DfN", ctypes.c_double),
                ("Wi0", ctypes.c_double), ("dt", ctypes.c_double), ("fd_eps", ctypes.c_double)]


class c_mesh(ctypes.Structure):
    _fields_ = [("nnodes", ctypes.c_int32), ("nel", ctypes.c_int32), ("conn", ctypes.c_void_p),
                ("xyz", ctypes.c_void_p), ("n_outlet_edges", ctypes.c_int32),
                ("outlet_edge_elem", ctypes.c_void_p), ("outlet_edge_id", ctypes.c_void_p)]


class c_csr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("rowptr", ctypes.c_void_p), ("colind", ctypes.c_void_p)]


_lib = None


def load(path: str = LIB_PATH):
    """Load libvefem.so (built by ``build.py``); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise VefemError(f"{path} is missing: run ve_flow_around_cylinder_fortran_gb300/build.py")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    L.vefem_abi_version.restype = ctypes.c_int
    L.vefem_create.argtypes = [P, P, P, ctypes.POINTER(P)]
    L.vefem_set_params.argtypes = [P, P]
    L.vefem_assemble.argtypes = [P, P, P, ctypes.c_int, P, P, ctypes.c_int]
    L.vefem_last_timing.argtypes = [P, P, ctypes.c_int]
    L.vefem_last_launch_count.argtypes = [P]
    L.vefem_stream.argtypes = [P]
    L.vefem_stream.restype = P
    L.vefem_destroy.argtypes = [P]
    L.vefem_last_error.argtypes = [P]
    L.vefem_last_error.restype = ctypes.c_char_p
    L.vefem_build_pattern.argtypes = [P, ctypes.c_int, P, P, P, P]
    L.vefem_apply_dirichlet.argtypes = [P, ctypes.c_int, P, P, P, P, P, ctypes.c_int, ctypes.c_int]
    I, I64, F = ctypes.c_int, ctypes.c_int64, ctypes.c_float
    L.vefem_mlp_create.argtypes = [I, I, I, I, ctypes.c_uint64, I, ctypes.POINTER(P)]
    L.vefem_mlp_num_params.argtypes = [P]
    L.vefem_mlp_num_params.restype = I64
    L.vefem_mlp_set_params.argtypes = [P, P, I64]
    L.vefem_mlp_get_params.argtypes = [P, P, I64]
    L.vefem_mlp_forward.argtypes = [P, P, I, P]
    L.vefem_mlp_loss_grad.argtypes = [P, P, P, I, P, P]
    L.vefem_mlp_train.argtypes = [P, P, P, I, I, F, P]
    L.vefem_mlp_reset_optimizer.argtypes = [P]
    L.vefem_mlp_destroy.argtypes = [P]
    L.vefem_mlp_last_error.argtypes = [P]
    L.vefem_mlp_last_error.restype = ctypes.c_char_p
    L.vefem_batch_create.argtypes = [I, P, P, P, ctypes.POINTER(P)]
    L.vefem_batch_set_params.argtypes = [P, I, P]
    L.vefem_assemble_batched.argtypes = [P, P, P, I, P, P, I]
    L.vefem_batch_autotune.argtypes = [P, I, I, P]
    L.vefem_batch_set_tiles.argtypes = [P, P]
    L.vefem_batch_info.argtypes = [P, P]
    L.vefem_batch_last_timing.argtypes = [P, P]
    L.vefem_batch_destroy.argtypes = [P]
    L.vefem_batch_last_error.argtypes = [P]
    L.vefem_batch_last_error.restype = ctypes.c_char_p
    L.vefem_stability_pattern.argtypes = [P, P, P, P, P]
    L.vefem_stability_assemble.argtypes = [P, P, I, P, I, P, P, I]
    L.vefem_frontal_create.argtypes = [I, I, P, P, P, P, P, P, P, I64, ctypes.POINTER(P)]
    L.vefem_frontal_factor.argtypes = [P, P, P, ctypes.c_double, P]
    L.vefem_frontal_solve.argtypes = [P, P, P, P, P]
    L.vefem_frontal_destroy.argtypes = [P]
    L.vefem_frontal_destroy.restype = None
    L.vefem_frontal_last_error.argtypes = [P]
    L.vefem_frontal_last_error.restype = ctypes.c_char_p
    L.vefem_frontal_solve_path.argtypes = [P]
    _lib = L
    return L


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):           # torch tensor on the device
        return a.data_ptr()
    return int(a)


def make_params(phys, device: int = 0) -> c_params:
    from .state import FORMS, MODELS
    return c_params(MODELS[phys.model], FORMS[phys.form], phys.nex, device, phys.ReN, phys.WiN,
                    phys.BvN, phys.VeN, phys.DfN, phys.Wi0, phys.dt, phys.eps)


def build_pattern(conn: np.ndarray, nnodes: int, nex: int):
    """AIJ pattern of preAllocatePetsc through the library's host helper."""
    L = load()
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    m = c_mesh(nnodes, conn.shape[1], conn.ctypes.data, None, 0, None, None)
    n = ctypes.c_int64()
    nnz = ctypes.c_int64()
    rc = L.vefem_build_pattern(ctypes.byref(m), nex, ctypes.byref(n), ctypes.byref(nnz), None, None)
    if rc:
        raise VefemError(L.vefem_last_error(None).decode())
    rowptr = np.zeros(n.value + 1, dtype=np.int64)
    colind = np.zeros(nnz.value, dtype=np.int32)
    rc = L.vefem_build_pattern(ctypes.byref(m), nex, ctypes.byref(n), ctypes.byref(nnz),
                               rowptr.ctypes.data, colind.ctypes.data)
    if rc:
        raise VefemError(L.vefem_last_error(None).decode())
    return rowptr, colind


class BulkAssembler:
    """One mesh, one frozen AIJ pattern, one physics parameter set."""

    def __init__(self, mesh, phys, rowptr: np.ndarray, colind: np.ndarray,
                 outlet_edges: bool = False, device: int = 0):
        L = load()
        self._L = L
        self.phys = phys
        self._conn = np.ascontiguousarray(mesh.conn, dtype=np.int32)
        self._xyz = np.ascontiguousarray(mesh.xyz, dtype=np.float64)
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        self.colind = np.ascontiguousarray(colind, dtype=np.int32)
        self.nnodes = int(mesh.nnodes)
        self.nel = int(mesh.nel)
        self.N = int(self.rowptr.shape[0] - 1)
        self.nnz = int(self.colind.shape[0])
        if outlet_edges and len(mesh.outlet_edges):
            self._ee = np.ascontiguousarray(mesh.outlet_edges[:, 0], dtype=np.int32)
            self._ei = np.ascontiguousarray(mesh.outlet_edges[:, 1], dtype=np.int32)
            ne = len(self._ee)
        else:
            self._ee = self._ei = None
            ne = 0
        cm = c_mesh(self.nnodes, self.nel, self._conn.ctypes.data, self._xyz.ctypes.data, ne,
                    _ptr(self._ee), _ptr(self._ei))
        cc = c_csr(self.N, self.rowptr.ctypes.data, self.colind.ctypes.data)
        self.device = device
        self._params = make_params(phys, device)
        h = ctypes.c_void_p()
        rc = L.vefem_create(ctypes.byref(cm), ctypes.byref(cc), ctypes.byref(self._params),
                            ctypes.byref(h))
        if rc:
            raise VefemError(f"vefem_create failed ({rc}): {L.vefem_last_error(None).decode()}")
        self._h = h

    def _check(self, rc):
        if rc:
            raise VefemError(f"vefem error {rc}: {self._L.vefem_last_error(self._h).decode()}")

    def set_params(self, phys):
        self.phys = phys
        self._params = make_params(phys, self.device)
        self._check(self._L.vefem_set_params(self._h, ctypes.byref(self._params)))

    def assemble(self, TL, EU, flags: int, b=None, vals=None, on_device: bool = False):
        """Raw entry point: arrays are numpy (host) or torch CUDA tensors (device)."""
        self._check(self._L.vefem_assemble(self._h, _ptr(TL), _ptr(EU), int(flags), _ptr(b),
                                           _ptr(vals), 1 if on_device else 0))

    def set_equations_bulk(self, TL, EU, flag_nr: str = "NRP", b=None, vals=None,
                           zero_first: bool = False, outlet_edges: bool = False,
                           jacobian: str = "fd64"):
        """setEquationsBulk on host arrays; returns (b, vals).  ``jacobian``:
        'fd64' (the reference's forward difference, bit-exact), 'exact64' or
        'exact32' (exact derivative; float32 values for 'exact32')."""
        if flag_nr not in ("NRP", "MNR"):
            raise ValueError("flag_nr must be 'NRP' or 'MNR'")
        TL = np.ascontiguousarray(TL, dtype=np.float64)
        EU = np.ascontiguousarray(EU if EU is not None and len(EU) else np.zeros(1), dtype=np.float64)
        if b is None:
            b = np.zeros(self.N)
        flags = VEFEM_RESIDUAL
        if flag_nr == "NRP":
            flags |= JACOBIANS[jacobian]
            dt = np.float32 if jacobian == "exact32" else np.float64
            if vals is None:
                vals = np.zeros(self.nnz, dtype=dt)
            elif vals.dtype != dt:
                raise ValueError(f"vals must be {np.dtype(dt).name} for jacobian={jacobian}")
        else:
            vals = None
        if zero_first:
            flags |= VEFEM_ZERO_FIRST
        if outlet_edges:
            flags |= VEFEM_OUTLET_EDGES
        self.assemble(TL, EU, flags, b, vals, on_device=False)
        return b, vals

    def apply_dirichlet(self, rows, values, TL, b, vals, flags: int, on_device: bool = False,
                        nrows: int | None = None):
        """Dirichlet rows after assembly (applyDirichletBC): b = TL - value and,
        with a Jacobian flag, MatZeroRows(diag = 1) on vals."""
        n = int(nrows if nrows is not None else len(rows))
        if not on_device:
            rows = np.ascontiguousarray(rows, dtype=np.int64)
            values = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self._L.vefem_apply_dirichlet(self._h, n, _ptr(rows), _ptr(values), _ptr(TL),
                                                  _ptr(b), _ptr(vals), int(flags),
                                                  1 if on_device else 0))

    def last_timing(self):
        t = (ctypes.c_float * 5)()
        self._check(self._L.vefem_last_timing(self._h, t, 5))
        return list(t)

    def last_launch_count(self) -> int:
        return int(self._L.vefem_last_launch_count(self._h))

    def stream(self) -> int:
        return int(self._L.vefem_stream(self._h) or 0)

    def stability_pattern(self):
        """AIJ pattern of the stability matrices (10 unknowns per node)."""
        n, nnz = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._L.vefem_stability_pattern(self._h, ctypes.byref(n), ctypes.byref(nnz),
                                                    None, None))
        rowptr = np.zeros(n.value + 1, dtype=np.int64)
        colind = np.zeros(nnz.value, dtype=np.int32)
        self._check(self._L.vefem_stability_pattern(self._h, ctypes.byref(n), ctypes.byref(nnz),
                                                    rowptr.ctypes.data, colind.ctypes.data))
        return rowptr, colind

    def stability_assemble(self, TLb, kws, flags: int = VEFEM_ZERO_FIRST, As=None, B=None,
                           on_device: bool = False):
        """setEquationsBulkStability for every wavenumber of ``kws``: adds A(k)
        into As[k] and the k-independent B into B (float64 arrays on the
        stability pattern; allocated on the host when not given)."""
        if As is None:
            _, ci = self.stability_pattern()
            As = [np.zeros(len(ci)) for _ in kws]
            if B is None:
                B = np.zeros(len(ci))
        kw = np.ascontiguousarray(kws, dtype=np.float64)
        if on_device:
            import torch
            kw_arg = torch.from_numpy(kw).to(f"cuda:{self.device}")
        else:
            kw_arg = kw
        arr = (ctypes.c_void_p * max(1, len(As)))()
        for i, a in enumerate(As):
            arr[i] = _ptr(a)
        tlb = TLb if on_device else np.ascontiguousarray(TLb, dtype=np.float64)
        self._check(self._L.vefem_stability_assemble(self._h, _ptr(tlb), len(kws), _ptr(kw_arg),
                                                     flags, arr, _ptr(B), 1 if on_device else 0))
        return As, B

    def close(self):
        if getattr(self, "_h", None):
            self._L.vefem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MLP:
    """The learned predictor's network on the GPU (vefem_mlp_* in vefem.h):
    ``in_dim -> width (GELU) x hidden -> out_dim``, BF16 weights with FP32
    accumulation, trained by the library's own forward, backward and Adam
    kernels.  Arrays cross the boundary as host float32."""

    def __init__(self, in_dim: int, out_dim: int, width: int = 256, hidden: int = 3,
                 seed: int = 0, device: int = 0):
        self._L = load()
        self.in_dim, self.out_dim, self.width, self.hidden = in_dim, out_dim, width, hidden
        h = ctypes.c_void_p()
        rc = self._L.vefem_mlp_create(in_dim, width, out_dim, hidden, seed, device,
                                      ctypes.byref(h))
        if rc:
            raise VefemError(f"vefem_mlp_create failed ({rc}): "
                             f"{self._L.vefem_last_error(None).decode()}")
        self._h = h
        self.n_params = int(self._L.vefem_mlp_num_params(h))

    def _check(self, rc):
        if rc:
            raise VefemError(f"vefem_mlp error {rc}: {self._L.vefem_mlp_last_error(self._h).decode()}")

    @staticmethod
    def _f32(a, shape=None):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if shape is not None and a.shape != shape:
            raise ValueError(f"expected shape {shape}, got {a.shape}")
        return a

    def get_params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        self._check(self._L.vefem_mlp_get_params(self._h, p.ctypes.data, self.n_params))
        return p

    def set_params(self, p):
        p = self._f32(p, (self.n_params,))
        self._check(self._L.vefem_mlp_set_params(self._h, p.ctypes.data, self.n_params))

    def forward(self, X) -> np.ndarray:
        X = self._f32(X)
        n = X.shape[0]
        self._f32(X, (n, self.in_dim))
        Y = np.empty((n, self.out_dim), np.float32)
        self._check(self._L.vefem_mlp_forward(self._h, X.ctypes.data, n, Y.ctypes.data))
        return Y

    def loss_grad(self, X, T):
        X = self._f32(X)
        n = X.shape[0]
        self._f32(X, (n, self.in_dim))
        T = self._f32(T, (n, self.out_dim))
        loss = np.zeros(1, np.float32)
        g = np.empty(self.n_params, np.float32)
        self._check(self._L.vefem_mlp_loss_grad(self._h, X.ctypes.data, T.ctypes.data, n,
                                                loss.ctypes.data, g.ctypes.data))
        return float(loss[0]), g

    def train(self, X, T, iters: int, lr: float = 1e-3) -> float:
        X = self._f32(X)
        n = X.shape[0]
        self._f32(X, (n, self.in_dim))
        T = self._f32(T, (n, self.out_dim))
        loss = np.zeros(1, np.float32)
        self._check(self._L.vefem_mlp_train(self._h, X.ctypes.data, T.ctypes.data, n, iters,
                                            ctypes.c_float(lr), loss.ctypes.data))
        return float(loss[0])

    def reset_optimizer(self):
        self._check(self._L.vefem_mlp_reset_optimizer(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._L.vefem_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchAssembler:
    """Batched form (vefem_batch_* in vefem.h): many instances -- meshes of
    uneven size, each with its own parameters -- assembled together by one
    persistent launch per kernel, replayed as a CUDA graph."""

    def __init__(self, meshes, physs, patterns, device: int = 0):
        L = load()
        self._L = L
        n = len(meshes)
        if not (n == len(physs) == len(patterns)) or n == 0:
            raise ValueError("meshes, physs and patterns must have the same non-zero length")
        self.n = n
        self._keep = []
        cms = (c_mesh * n)()
        ccs = (c_csr * n)()
        cps = (c_params * n)()
        self.N, self.nnz, self.nel, self.nnodes = [], [], [], []
        for i, (m, p, (rp, ci)) in enumerate(zip(meshes, physs, patterns)):
            conn = np.ascontiguousarray(m.conn, dtype=np.int32)
            xyz = np.ascontiguousarray(m.xyz, dtype=np.float64)
            rp = np.ascontiguousarray(rp, dtype=np.int64)
            ci = np.ascontiguousarray(ci, dtype=np.int32)
            self._keep += [conn, xyz, rp, ci]
            cms[i] = c_mesh(int(m.nnodes), int(m.nel), conn.ctypes.data, xyz.ctypes.data, 0,
                            None, None)
            ccs[i] = c_csr(len(rp) - 1, rp.ctypes.data, ci.ctypes.data)
            cps[i] = make_params(p, device)
            self.N.append(len(rp) - 1)
            self.nnz.append(len(ci))
            self.nel.append(int(m.nel))
            self.nnodes.append(int(m.nnodes))
        h = ctypes.c_void_p()
        rc = L.vefem_batch_create(n, cms, ccs, cps, ctypes.byref(h))
        if rc:
            raise VefemError(f"vefem_batch_create failed ({rc}): "
                             f"{L.vefem_last_error(None).decode()}")
        self._h = h
        self.device = device

    def _check(self, rc):
        if rc:
            raise VefemError(f"vefem batch error {rc}: "
                             f"{self._L.vefem_batch_last_error(self._h).decode()}")

    @staticmethod
    def _parr(xs):
        arr = (ctypes.c_void_p * len(xs))()
        for i, x in enumerate(xs):
            arr[i] = _ptr(x)
        return arr

    def set_params(self, i: int, phys):
        p = make_params(phys, self.device)
        self._check(self._L.vefem_batch_set_params(self._h, i, ctypes.byref(p)))

    def assemble(self, TLs, EUs, flags: int, bs=None, valss=None, on_device: bool = False):
        n = self.n
        bs = bs if bs is not None else [None] * n
        valss = valss if valss is not None else [None] * n
        EUs = EUs if EUs is not None else [None] * n
        self._check(self._L.vefem_assemble_batched(
            self._h, self._parr(TLs), self._parr(EUs), flags, self._parr(bs), self._parr(valss),
            1 if on_device else 0))

    def autotune(self, flags: int, reps: int = 3):
        t = (ctypes.c_int * BATCH_CLASSES)()
        self._check(self._L.vefem_batch_autotune(self._h, flags, reps, t))
        return list(t)

    def set_tiles(self, tiles):
        t = (ctypes.c_int * BATCH_CLASSES)(*tiles)
        self._check(self._L.vefem_batch_set_tiles(self._h, t))

    def info(self) -> dict:
        o = (ctypes.c_int64 * 6)()
        self._check(self._L.vefem_batch_info(self._h, o))
        return {"instances": o[0], "elements": o[1], "work_items": o[2], "grid": o[3],
                "launches": o[4], "replays": o[5]}

    def last_timing(self):
        t = (ctypes.c_float * 3)()
        self._check(self._L.vefem_batch_last_timing(self._h, t))
        return list(t)

    def close(self):
        if getattr(self, "_h", None):
            self._L.vefem_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
