"""Instance sharding for multi-GPU batches, exercised with two gloo ranks on
the CPU: every instance is run by exactly one rank, the cost split is
balanced, and the gathered energies equal a single-rank run (here the runner
is the oracle, so no GPU is needed)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from _pkg import pkg


def _oracle_energies(instances):
    from oracle import oracle as O

    out = []
    for inst in instances:
        o = O.OracleQV(inst["n"])
        for k, q0, q1, p in inst["gates"]:
            if k in (0, 1, 2):
                o.apply_rotation([q0], k, inst["theta"][p])
            elif k == 3:
                o.apply_mcx([q0, q1])
        out.append(sum(c * o.expval_pauli(q, lab) for (q, lab), c in zip(inst["terms"], inst["coeffs"])))
    return out


def _worker(rank, world, port, result_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    P = pkg()
    insts = P.batched.config5_instances(9, seed=3, qmin=3, qmax=7, dmin=1, dmax=3, tmin=3, tmax=6, shots=10)
    e = P.batched.run_sharded(insts, _oracle_energies)
    if rank == 0:
        np.save(result_path, e)
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_shard_covers_and_balances():
    P = pkg()
    insts = P.batched.config5_instances(40, seed=1, qmin=3, qmax=10, dmin=1, dmax=5, tmin=3, tmax=5, shots=4)
    parts = [P.batched.shard(insts, r, 3) for r in range(3)]
    assert sorted(i for p in parts for i in p) == list(range(40))
    cost = [[insts[i]["depth"] * (1 << insts[i]["n"]) for i in p] for p in parts]
    loads = [sum(c) for c in cost]
    assert max(loads) - min(loads) <= max(max(c) for c in cost if c)


def test_two_gloo_ranks_match_one(tmp_path):
    P = pkg()
    path = str(tmp_path / "e.npy")
    mp.start_processes(_worker, args=(2, _free_port(), path), nprocs=2, start_method="spawn")
    e2 = np.load(path)
    insts = P.batched.config5_instances(9, seed=3, qmin=3, qmax=7, dmin=1, dmax=3, tmin=3, tmax=6, shots=10)
    e1 = np.array(_oracle_energies(insts))
    np.testing.assert_allclose(e2, e1, atol=1e-12)
