"""Multi-process host logic (qcsim_gb300/replicas.py) on CPU: instance sharding by cost, and two gloo
ranks that each run their share of a QAOA batch (energies from the CPU oracle standing in for the
GPU engine), gather the energies, and reduce a timing with max over ranks."""
import ctypes as C
import os
import socket

import numpy as np
import pytest

from qcsim_gb300 import circuits, replicas


def test_shard_by_cost_covers_and_balances():
    rng = np.random.default_rng(0)
    costs = [float(1 << int(n)) for n in rng.integers(6, 20, 300)]
    for world in (1, 2, 3, 8):
        shards = replicas.shard_by_cost(costs, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shards]
        # LPT: no rank exceeds the lightest by more than the largest single item
        assert max(loads) - min(loads) <= max(costs)
    assert replicas.shard_by_cost([], 4) == [[], [], [], []]
    with pytest.raises(ValueError):
        replicas.shard_by_cost([1.0], 0)


def _energy(inst):
    from oracle import bind as B
    lib = B.oracle()
    e = np.array(inst["edges"], dtype=np.uint32).reshape(-1)
    J, h = np.array(inst["J"]), np.array(inst["h"])
    g, b = np.array(inst["gammas"]), np.array(inst["betas"])
    reg = B.OracleRegister(inst["n"])
    pu = e.ctypes.data_as(C.POINTER(C.c_uint32))
    assert lib.qo_qaoa_exec(reg.h, len(inst["edges"]), pu, B.dp(J), B.dp(h), len(g), B.dp(g), B.dp(b)) == 0
    return lib.qo_expected_energy(reg.h, len(inst["edges"]), pu, B.dp(J), B.dp(h))


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    insts = circuits.qaoa_instances(10, seed=5, nmin=6, nmax=10, p=2)
    mine = replicas.shard_by_cost(replicas.qaoa_costs(insts), world)[rank]
    energies = [_energy(insts[i]) for i in mine]
    full = replicas.gather_values(dist, mine, energies, len(insts))
    slowest = replicas.max_over_ranks(dist, float(rank + 1))
    dist.barrier()
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.append(full, slowest))
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_shard_and_gather(tmp_path):
    import torch.multiprocessing as mp
    from oracle import bind as B
    B.build_oracle()
    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    insts = circuits.qaoa_instances(10, seed=5, nmin=6, nmax=10, p=2)
    want = np.array([_energy(inst) for inst in insts])
    for rank in range(2):
        got = np.load(tmp_path / f"rank{rank}.npy")
        assert got[-1] == 2.0  # max over ranks of (rank + 1)
        assert np.array_equal(got[:-1], want)
