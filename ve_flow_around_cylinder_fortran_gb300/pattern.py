"""AIJ (CSR) sparsity pattern of the Newton Jacobian, as preAllocatePetsc
(Petsc_mod.F90:629-743) freezes it.

Every element contributes its dense 54 x 54 block: rows and columns
``(gnode - 1) * Neq + ieq - 1`` of its nine nodes (getRows, Tools_mod.F90:
735-752; Storage_mod.F90:41-79).  With arclength continuation (``nex`` = 1,
problem 'Main') the last column is filled by every element row
(storeJacobian_Ac, Storage_mod.F90:83-115) and the last row and column are
preallocated dense (Petsc_mod.F90:727-737).  Columns are sorted within each
row, as PETSc's AIJ format keeps them.
"""
from __future__ import annotations

import numpy as np

NEQ = 6


def node_adjacency(elem_nodes: np.ndarray, nnodes: int):
    """Sorted unique (row node, col node) pairs from [Nel, 9] 0-based nodes.
    Returns (ptr [nnodes+1] int64, nbr [npairs] int64)."""
    a = np.repeat(elem_nodes, 9, axis=1).ravel().astype(np.int64)
    b = np.tile(elem_nodes, (1, 9)).ravel().astype(np.int64)
    key = np.unique(a * nnodes + b)
    rows = key // nnodes
    nbr = key % nnodes
    ptr = np.zeros(nnodes + 1, dtype=np.int64)
    np.add.at(ptr, rows + 1, 1)
    return np.cumsum(ptr), nbr


def build_pattern(elem_nodes: np.ndarray, nnodes: int, nex: int = 1):
    """Return (rowptr int64 [N+1], colind int32 [nnz]) with N = nnodes*6 + nex."""
    if nex not in (0, 1):
        raise ValueError("nex must be 0 or 1")
    ptr, nbr = node_adjacency(elem_nodes, nnodes)
    deg = np.diff(ptr)
    n_dof = nnodes * NEQ
    N = n_dof + nex
    row_len = np.repeat(deg * NEQ + nex, NEQ)
    if nex:
        row_len = np.concatenate([row_len, [N]])
    rowptr = np.zeros(N + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum(row_len)
    # columns of one node row: neighbour blocks of 6 (+ last column)
    block_cols = (nbr[:, None] * NEQ + np.arange(NEQ)[None, :]).ravel()      # per node, in order
    colind = np.empty(int(rowptr[-1]), dtype=np.int64)
    node_start = ptr[:-1] * NEQ                                               # into block_cols
    for ieq in range(NEQ):
        rows = np.arange(nnodes) * NEQ + ieq
        starts = rowptr[rows]
        # scatter each node's block column list into its row
        lens = deg * NEQ
        idx_rows = np.repeat(starts, lens) + (np.arange(lens.sum()) - np.repeat(np.cumsum(lens) - lens, lens))
        colind[idx_rows] = block_cols
        if nex:
            colind[starts + lens] = n_dof
    if nex:
        colind[rowptr[n_dof]:] = np.arange(N)
    del node_start
    return rowptr, colind.astype(np.int32)


def dense_from_csr(rowptr: np.ndarray, colind: np.ndarray, vals: np.ndarray, n: int) -> np.ndarray:
    out = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    out[rows, colind] = vals
    return out
