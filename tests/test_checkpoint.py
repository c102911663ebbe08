"""Solution checkpoints in the reference's unformatted sequential format
(writeSolution / readSolution, Post_Process_mod.F90:1271-1420)."""
import struct

import numpy as np
import pytest

from ve_flow_around_cylinder_fortran_gb300 import checkpoint as CK
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import state as S


def _case():
    mesh = M.build_cylinder_mesh(120, exact=False)
    phys = S.oldroyd_b(0.3, 0.59, "SQRT", nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, seed=3)
    return mesh, TL, np.array([1.25])


def test_round_trip_is_bit_exact(tmp_path):
    mesh, TL, EU = _case()
    en = mesh.element_nodes()
    p = str(tmp_path / "Cylinder_2D")
    CK.write_solution(p, en, TL, EU)
    TL2, EU2 = CK.read_solution(p, en, mesh.nnodes, 1)
    assert np.array_equal(TL, TL2) and np.array_equal(EU, EU2)


def test_record_layout(tmp_path):
    mesh, TL, EU = _case()
    en = mesh.element_nodes()
    p = str(tmp_path / "s")
    CK.write_solution(p, en, TL, EU)
    raw = open(p + ".DTA", "rb").read()
    nrec = mesh.nel * 9 * 6 + 1
    assert len(raw) == 16 * nrec
    # record k: element k // 54, local node (k // 6) % 9, equation k % 6
    for k in (0, 1, 7, 54 * 5 + 13, nrec - 2):
        head, val, tail = struct.unpack("<idi", raw[16 * k:16 * k + 16])
        e, n, q = k // 54, (k // 6) % 9, k % 6
        assert head == tail == 8 and val == TL[q, en[e, n]]
    assert struct.unpack("<idi", raw[-16:])[1] == EU[0]


def test_missing_extra_unknowns_and_last_occurrence(tmp_path):
    mesh, TL, EU = _case()
    en = mesh.element_nodes()
    p = str(tmp_path / "s")
    CK.write_solution(p, en, TL, [])
    TL2, EU2 = CK.read_solution(p, en, mesh.nnodes, 1)
    assert np.array_equal(TL, TL2) and EU2[0] == 0.0
    _, EU3 = CK.read_solution(p, en, mesh.nnodes, 1, EU_before=[0.7])
    assert EU3[0] == 0.7
    # a duplicated node value that differs between elements: the last element wins
    raw = bytearray(open(p + ".DTA", "rb").read())
    g = en[0, 2]
    later = [(e, n) for e in range(mesh.nel) for n in range(9) if en[e, n] == g]
    e, n = later[-1]
    k = e * 54 + n * 6 + 4
    raw[16 * k + 4:16 * k + 12] = struct.pack("<d", 42.0)
    open(p + ".DTA", "wb").write(bytes(raw))
    TL3, _ = CK.read_solution(p, en, mesh.nnodes, 1)
    assert TL3[4, g] == 42.0


def test_transient_companions(tmp_path):
    mesh, TL, EU = _case()
    en = mesh.element_nodes()
    p = str(tmp_path / "t")
    paths = CK.write_solution(p, en, TL, EU, TLo=TL * 2, EUo=EU, TLb=TL * 3, EUb=EU)
    assert [x[-6:] for x in paths] == ["/t.DTA", "_o.DTA", "_b.DTA"]
    TLb, _ = CK.read_solution(p, en, mesh.nnodes, 1, suffix="_b")
    assert np.array_equal(TLb, TL * 3)


def test_malformed_files_are_rejected(tmp_path):
    mesh, TL, EU = _case()
    en = mesh.element_nodes()
    p = str(tmp_path / "m")
    open(p + ".DTA", "wb").write(b"\x00" * 17)
    with pytest.raises(ValueError):
        CK.read_solution(p, en, mesh.nnodes, 1)
    open(p + ".DTA", "wb").write(struct.pack("<idi", 4, 1.0, 8))
    with pytest.raises(ValueError):
        CK.read_solution(p, en, mesh.nnodes, 1)
