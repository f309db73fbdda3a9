"""gbx_relax_batch_static -- the relaxation for callers that cannot allocate
device memory -- against gbx_relax_batch with a caller-owned workspace.

Collected last on purpose. The batch (Birkhoff order 64, node vectors too large
for shared memory) needs global scratch, so the library-owned array is really
used; two calls in a row check that the reused array carries nothing over. The
FP64 path is deterministic, so results must be identical."""
import ctypes as C

import numpy as np
import pytest

from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances

pytestmark = pytest.mark.gpu


def _batch(lb, ub, eps, dev):
    import torch
    N, n = lb.shape
    t = {k: torch.from_numpy(v).to(dev) for k, v in dict(x=lb.copy(), lb=lb, ub=ub, eps=eps).items()}
    t["it"] = torch.zeros(N, dtype=torch.int32, device=dev)
    t["st"] = torch.zeros(N, dtype=torch.uint8, device=dev)
    t["gap"] = torch.zeros(N, dtype=torch.float64, device=dev)
    t["val"] = torch.zeros(N, dtype=torch.float64, device=dev)
    t["bv"] = torch.zeros(N, n, dtype=torch.float64, device=dev)
    t["bvv"] = torch.zeros(N, dtype=torch.float64, device=dev)
    t["flags"] = torch.ones(n, dtype=torch.uint8, device=dev)
    b = A.NodeBatch(N, 6, 1e-6, t["x"].data_ptr(), t["lb"].data_ptr(), t["ub"].data_ptr(), t["eps"].data_ptr(),
                    t["it"].data_ptr(), t["st"].data_ptr(), t["gap"].data_ptr(), t["val"].data_ptr(),
                    t["bv"].data_ptr(), t["bvv"].data_ptr(), t["flags"].data_ptr())
    return b, t


def _host(t):
    return {k: v.cpu().numpy() for k, v in t.items() if k not in ("lb", "ub", "eps", "flags")}


def test_static_scratch_matches_workspace_variant_twice():
    import torch
    assert torch.cuda.is_available()
    from gpuboscia_gb300 import build
    build.build()
    lib = A.load()
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    inst = instances.birkhoff_gnp(order=64, seed=13)
    keep = api._Keep()
    obj = inst.objective.to_c("cuda", keep)
    lmo = inst.lmo.to_c(64 * 64, "cuda", keep)
    alg = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    for seed in (3, 4):   # two calls in a row on different batches
        lb, ub = instances.birkhoff_node_batch(64, 6, seed=seed)
        eps = np.full(6, 1e-6)
        need = lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(lmo), C.byref(alg), 6)
        assert 256 < need <= A.STATIC_SCRATCH_BYTES
        b_ref, t_ref = _batch(lb, ub, eps, dev)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        rc = lib.gbx_relax_batch(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b_ref), ws.data_ptr(), need,
                                 stream)
        assert rc == A.OK, lib.gbx_last_error()
        b_st, t_st = _batch(lb, ub, eps, dev)
        rc = lib.gbx_relax_batch_static(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b_st), stream)
        assert rc == A.OK, lib.gbx_last_error()
        torch.cuda.synchronize()
        ref, got = _host(t_ref), _host(t_st)
        for k in ref:
            assert np.array_equal(ref[k], got[k]), k
        assert (got["it"] == 6).all()


def test_static_scratch_rejects_oversized_batches():
    import torch
    assert torch.cuda.is_available()
    from gpuboscia_gb300 import build
    build.build()
    lib = A.load()
    inst = instances.birkhoff_gnp(order=64, seed=13)
    keep = api._Keep()
    obj = inst.objective.to_c("cuda", keep)
    lmo = inst.lmo.to_c(64 * 64, "cuda", keep)
    alg = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    one = lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(lmo), C.byref(alg), 1)
    per_node = lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(lmo), C.byref(alg), 2) - one
    too_many = A.STATIC_SCRATCH_BYTES // max(per_node, 1) + 2
    b = A.NodeBatch()
    b.n_nodes = int(too_many)
    rc = lib.gbx_relax_batch_static(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b), None)
    assert rc == A.ERR_WORKSPACE
    assert b"static scratch" in lib.gbx_last_error()


@pytest.mark.parametrize("order,nodes", [(120, 3), (400, 2)])
def test_static_scratch_mixed_precision_twice(order, nodes):
    """The mixed path keeps more in the scratch than the FP64 path: its FP32
    arrays, the integer oracles' warm state and, at order 400, the oracle
    costs, edge codes and the graphs' nonzero lists. Two calls in a row on
    different batches must equal the caller-workspace variant (the mixed
    path is deterministic at a fixed launch shape), so no word of the shared
    array is read before the call writes it."""
    import torch
    assert torch.cuda.is_available()
    from gpuboscia_gb300 import build
    build.build()
    lib = A.load()
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    inst = (instances.birkhoff_regular_perturbed(order=order) if order == 120
            else instances.birkhoff_regular_isomorphic(order=order))
    keep = api._Keep()
    obj = inst.objective.to_c("cuda", keep)
    lmo = inst.lmo.to_c(order * order, "cuda", keep)
    alg = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_MIXED)
    for seed in (7, 8):
        lb, ub = instances.birkhoff_node_batch(order, nodes, seed=seed)
        eps = np.full(nodes, 1e-6)
        need = lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(lmo), C.byref(alg), nodes)
        assert 256 < need <= A.STATIC_SCRATCH_BYTES
        b_ref, t_ref = _batch(lb, ub, eps, dev)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        rc = lib.gbx_relax_batch(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b_ref), ws.data_ptr(), need,
                                 stream)
        assert rc == A.OK, lib.gbx_last_error()
        b_st, t_st = _batch(lb, ub, eps, dev)
        rc = lib.gbx_relax_batch_static(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b_st), stream)
        assert rc == A.OK, lib.gbx_last_error()
        torch.cuda.synchronize()
        ref, got = _host(t_ref), _host(t_st)
        for k in ref:
            assert np.array_equal(ref[k], got[k]), k
