"""Solution checkpoints in the reference's on-disk format.

writeSolution / readSolution (Post_Process_mod.F90:1271-1420) store a state
as a Fortran unformatted sequential file ``<name>.DTA``: one record per
value, element-major -- for each element, for each of its 9 nodes (local
order of the connectivity), for each of the Neq = 6 equations, the value
TL(gnode, ieq) -- followed by one record per extra unknown EU(ieq).  Each
record is a 4-byte little-endian length (8), the FP64 value and the same
length again (the gfortran / ifort default record markers).  Values of a
node shared by several elements are written once per element; the reader
takes the last occurrence, like the Fortran loop.  The transient method
adds the previous and the one-before states as ``<name>_o.DTA`` and
``<name>_b.DTA``.
"""
from __future__ import annotations

import os

import numpy as np

_REC = np.dtype([("head", "<i4"), ("value", "<f8"), ("tail", "<i4")])


def _records(values: np.ndarray) -> np.ndarray:
    r = np.empty(values.size, _REC)
    r["head"] = 8
    r["value"] = values
    r["tail"] = 8
    return r


def write_solution(prefix: str, element_nodes: np.ndarray, TL: np.ndarray, EU,
                   TLo=None, EUo=None, TLb=None, EUb=None) -> list:
    """Write ``prefix.DTA`` (and ``prefix_o.DTA``, ``prefix_b.DTA`` when the
    previous states are given).  element_nodes [nel][9] 0-based, TL [6][nnodes]
    (field-major, the library's layout), EU [nex].  Returns the paths."""
    en = np.asarray(element_nodes)
    paths = []
    for suffix, tl, eu in (("", TL, EU), ("_o", TLo, EUo), ("_b", TLb, EUb)):
        if tl is None:
            continue
        tl = np.asarray(tl, dtype=np.float64)
        vals = tl[:, en].transpose(1, 2, 0).reshape(-1)          # [nel][9][6]
        eu = np.asarray(eu if eu is not None else [], dtype=np.float64).reshape(-1)
        path = prefix + suffix + ".DTA"
        with open(path, "wb") as f:
            f.write(_records(np.concatenate([vals, eu])).tobytes())
        paths.append(path)
    return paths


def read_solution(prefix: str, element_nodes: np.ndarray, nnodes: int, nex: int,
                  suffix: str = "", neq: int = 6, EU_before=None):
    """Read ``prefix{suffix}.DTA``; returns (TL [6][nnodes], EU [nex]).  The
    reference stops reading EU at the first missing record and keeps the
    values it had: those entries come from ``EU_before`` (zeros if not
    given).  Raises ValueError on a malformed file."""
    en = np.asarray(element_nodes)
    path = prefix + suffix + ".DTA"
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size % _REC.itemsize:
        raise ValueError(f"{path}: size {raw.size} is not a whole number of 16-byte records")
    rec = raw.view(_REC)
    if np.any(rec["head"] != 8) or np.any(rec["tail"] != 8):
        raise ValueError(f"{path}: record markers are not 8")
    ntl = en.size * neq
    if rec.size < ntl:
        raise ValueError(f"{path}: {rec.size} records, the mesh needs {ntl}")
    vals = rec["value"][:ntl].reshape(en.shape[0], en.shape[1], neq)
    TL = np.zeros((neq, nnodes))
    # element-major assignment: a later element overwrites an earlier one
    flat_nodes = en.reshape(-1)
    flat_vals = vals.reshape(-1, neq)
    last = np.full(nnodes, -1, dtype=np.int64)
    np.maximum.at(last, flat_nodes, np.arange(flat_nodes.size))   # last occurrence per node
    seen = last >= 0
    TL[:, seen] = flat_vals[last[seen]].T
    EU = np.zeros(nex) if EU_before is None else np.array(EU_before, dtype=np.float64)
    extra = rec["value"][ntl:ntl + nex]
    EU[:extra.size] = extra
    return TL, EU


def exists(prefix: str, suffix: str = "") -> bool:
    return os.path.exists(prefix + suffix + ".DTA")
