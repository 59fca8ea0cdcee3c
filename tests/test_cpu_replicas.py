"""The replica split on CPU with torch.distributed (gloo, world size 2): two
ranks run disjoint photon ranges through the oracle and sum their tallies
once; the result equals one process running all photons."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from nmc_gb300 import abi
from nmc_gb300.replicas import photon_range

N = 3000


def test_photon_range_partition():
    for world in (1, 2, 3, 7):
        for total in (0, 1, 10, 1001):
            spans = [photon_range(r, world, total, first=5) for r in range(world)]
            assert sum(n for _, n in spans) == total
            assert all(spans[i][0] + spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            assert spans[0][0] == 5
    with pytest.raises(ValueError):
        photon_range(2, 2, 10)


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import bindings
    from nmc_gb300.replicas import reduce_tallies
    import nmc_cases as cases

    rp, tp, ext = cases.mcsub_case()
    first, n = photon_range(rank, world, N)
    o = bindings.run(abi.SIM_MCSUB, rp, tp, ext=ext, first=first, n=n, nthreads=1)
    s = reduce_tallies({"J": o["J"], "F": o["F"], "sums": [o["S"], o["A"], o["E"], o["photons"]]})
    if rank == 0:
        q.put({k: v.tolist() for k, v in s.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process(oracle):
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    import nmc_cases as cases

    rp, tp, ext = cases.mcsub_case()
    o = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, first=0, n=N, nthreads=1)
    np.testing.assert_allclose(got["J"], o["J"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(got["F"], o["F"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(got["sums"], [o["S"], o["A"], o["E"], o["photons"]], rtol=1e-12)
