"""Multi-process shot sharding on CPU (gloo, world size 2): each rank runs
the oracle gradient of its shots, the kernels are summed across ranks, and
the result equals the gradient of all shots in one process."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _gradient(shots):
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    from tests import cases

    case = cases.make_case(wave="sh", nx=60, nz=40, nt=200, nsrc=4, nrec=12, sfe=10, seed=3, abs_width=8)
    pb = cases.oracle_problem(orc, case)
    rng = np.random.default_rng(7)
    ads = [(rng.standard_normal((pb.nrec, pb.nt)) * 1e-3) for _ in range(case["nsrc"])]
    kern = [np.zeros(pb.nx * pb.nz) for _ in range(3)]
    for s in shots:
        ck = orc.forward(pb, s, adj=True, precision="f64")[3]
        z = np.zeros((pb.nrec, pb.nt))
        kern = orc.adjoint(pb, [z, ads[s], z], ck, kern, precision="f64")
    return {"k_lambda": kern[0], "k_mu": kern[1], "k_rho": kern[2]}, float(len(shots))


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge

    pkg = ge.load_package()
    from invcu_gb300 import shards

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shards.shard_shots(4, rank, world)
    k, m = _gradient(mine)
    total, mis = shards.reduce_gradient(k, m)
    dist.destroy_process_group()
    q.put((rank, mine, {n: v.tolist() for n, v in total.items()}, mis))


def test_sharded_gradient_equals_single_process():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert res[0][1] == [0, 2] and res[1][1] == [1, 3]
    full, _ = _gradient([0, 1, 2, 3])
    for r in res:
        assert r[3] == 4.0
        for n in ("k_mu", "k_rho"):
            got = np.array(r[2][n])
            assert np.abs(got - full[n]).max() <= 1e-12 * np.abs(full[n]).max()
