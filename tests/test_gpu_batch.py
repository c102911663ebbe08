"""Batched form: many instances in one persistent launch per kernel, replayed
as a CUDA graph, against one vefem_assemble per instance.

The batched kernels run the same per-element arithmetic and the same
element-ordered sums as the single-mesh kernels, so every instance's residual
and AIJ values must equal the single-mesh call's bit for bit, for any tile
the autotuner picks, through device and host buffers, and after a parameter
change of one instance.
"""
import numpy as np
import pytest

from ve_flow_around_cylinder_fortran_gb300 import build as B
from ve_flow_around_cylinder_fortran_gb300 import mesh as M
from ve_flow_around_cylinder_fortran_gb300 import state as S
from ve_flow_around_cylinder_fortran_gb300 import vefem as V

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    V.load()


def _instances(sizes, wis, form="SQRT", nex=1, model="oldroyd_b"):
    out = []
    for k, (n, wi) in enumerate(zip(sizes, wis)):
        mesh = M.build_cylinder_mesh(n, exact=False)
        if model == "oldroyd_b":
            phys = S.oldroyd_b(wi, 0.59, form, nex=nex)
        else:
            phys = S.giesekus(0.1, wi, 0.59, form, nex=nex)
        TL, EU = S.seeded_state(mesh.xyz, phys, seed=k)
        pat = V.build_pattern(mesh.conn, mesh.nnodes, nex)
        out.append((mesh, phys, pat, TL, EU))
    return out


def _single(inst, flags, f32):
    mesh, phys, (rp, ci), TL, EU = inst
    a = V.BulkAssembler(mesh, phys, rp, ci)
    b = np.zeros(len(rp) - 1)
    v = np.zeros(len(ci), np.float32 if f32 else np.float64)
    a.assemble(TL, EU, flags, b, v)
    a.close()
    return b, v


def _batched_device(bt, insts, flags, f32):
    d = torch.device("cuda:0")
    TLs = [torch.from_numpy(i[3]).to(d) for i in insts]
    EUs = [torch.from_numpy(i[4]).to(d) for i in insts]
    bs = [torch.zeros(len(i[2][0]) - 1, dtype=torch.float64, device=d) for i in insts]
    vs = [torch.zeros(len(i[2][1]), dtype=torch.float32 if f32 else torch.float64, device=d)
          for i in insts]
    bt.assemble(TLs, EUs, flags, bs, vs, on_device=True)
    return [b.cpu().numpy() for b in bs], [v.cpu().numpy() for v in vs], (TLs, EUs, bs, vs)


@pytest.mark.parametrize("jac", ["exact32", "exact64"])
def test_batched_equals_single(jac):
    f32 = jac == "exact32"
    insts = _instances([300, 1200, 130, 2500, 700], [0.1, 0.35, 0.6, 0.85, 1.0])
    flags = V.VEFEM_RESIDUAL | V.JACOBIANS[jac] | V.VEFEM_ZERO_FIRST
    bt = V.BatchAssembler([i[0] for i in insts], [i[1] for i in insts], [i[2] for i in insts])
    bb, vv, bufs = _batched_device(bt, insts, flags, f32)
    for k, inst in enumerate(insts):
        b, v = _single(inst, flags, f32)
        assert np.array_equal(bb[k], b), k
        assert np.array_equal(vv[k], v), k
    # graph replay on the same buffers, filled with garbage first, gives the
    # same bits (VEFEM_ZERO_FIRST clears every entry, the lambda row included)
    info0 = bt.info()
    for x in list(bufs[2]) + list(bufs[3]):
        x.fill_(7.0)
    bt.assemble(*bufs[:2], flags, bufs[2], bufs[3], on_device=True)
    assert bt.info()["replays"] == info0["replays"] + 1
    for k in range(len(insts)):
        assert np.array_equal(bufs[2][k].cpu().numpy(), bb[k])
        assert np.array_equal(bufs[3][k].cpu().numpy(), vv[k])
    bt.close()


def test_batched_host_buffers_and_add_semantics():
    insts = _instances([400, 900], [0.2, 0.7], form="T", model="giesekus")
    flags = V.VEFEM_RESIDUAL | V.VEFEM_JAC_EXACT32
    bt = V.BatchAssembler([i[0] for i in insts], [i[1] for i in insts], [i[2] for i in insts])
    bs = [np.full(len(i[2][0]) - 1, 0.25) for i in insts]
    vs = [np.full(len(i[2][1]), 0.5, np.float32) for i in insts]
    bt.assemble([i[3] for i in insts], [i[4] for i in insts], flags, bs, vs)
    for k, inst in enumerate(insts):
        mesh, phys, (rp, ci), TL, EU = inst
        a = V.BulkAssembler(mesh, phys, rp, ci)
        b = np.full(len(rp) - 1, 0.25)
        v = np.full(len(ci), 0.5, np.float32)
        a.assemble(TL, EU, flags, b, v)
        a.close()
        assert np.array_equal(bs[k], b) and np.array_equal(vs[k], v)
    bt.close()


def test_autotune_and_tiles_keep_bits():
    insts = _instances([1500, 3000, 5000, 9000], [0.3, 0.4, 0.5, 0.6])
    flags = V.VEFEM_RESIDUAL | V.VEFEM_JAC_EXACT32 | V.VEFEM_ZERO_FIRST
    bt = V.BatchAssembler([i[0] for i in insts], [i[1] for i in insts], [i[2] for i in insts])
    b0, v0, _ = _batched_device(bt, insts, flags, True)
    tiles = bt.autotune(flags, reps=2)
    assert len(tiles) == V.BATCH_CLASSES and all(t in (1, 2, 4, 8) for t in tiles)
    b1, v1, _ = _batched_device(bt, insts, flags, True)
    bt.set_tiles([8, 4, 2, 1, 8, 8])
    b2, v2, _ = _batched_device(bt, insts, flags, True)
    for k in range(len(insts)):
        assert np.array_equal(b0[k], b1[k]) and np.array_equal(v0[k], v1[k])
        assert np.array_equal(b0[k], b2[k]) and np.array_equal(v0[k], v2[k])
    bt.close()


def test_set_params_of_one_instance():
    insts = _instances([300, 500], [0.2, 0.4])
    flags = V.VEFEM_RESIDUAL | V.VEFEM_JAC_EXACT32 | V.VEFEM_ZERO_FIRST
    bt = V.BatchAssembler([i[0] for i in insts], [i[1] for i in insts], [i[2] for i in insts])
    _batched_device(bt, insts, flags, True)
    new = S.oldroyd_b(0.9, 0.59, "SQRT", nex=1)
    bt.set_params(1, new)
    bb, vv, _ = _batched_device(bt, insts, flags, True)
    mesh, _, pat, TL, EU = insts[1]
    b, v = _single((mesh, new, pat, TL, EU), flags, True)
    assert np.array_equal(bb[1], b) and np.array_equal(vv[1], v)
    bt.close()


def test_unsupported_flags_and_mixed_forms_are_errors():
    insts = _instances([200, 300], [0.2, 0.4])
    bt = V.BatchAssembler([i[0] for i in insts], [i[1] for i in insts], [i[2] for i in insts])
    with pytest.raises(V.VefemError):
        bt.assemble([i[3] for i in insts], [i[4] for i in insts],
                    V.VEFEM_RESIDUAL | V.VEFEM_JAC_FD64, [np.zeros(len(i[2][0]) - 1) for i in insts],
                    [np.zeros(len(i[2][1])) for i in insts])
    bt.close()
    mixed = _instances([200], [0.2], form="T") + _instances([200], [0.2], form="SQRT")
    with pytest.raises(V.VefemError):
        V.BatchAssembler([i[0] for i in mixed], [i[1] for i in mixed], [i[2] for i in mixed])
