"""Replica-parallel runs on two gloo ranks (CPU): each rank builds its own
replica of the bench workload from its rank seed, advances it on the CPU
restatement, and the measurement reduction gives the slowest time and the
total particle-steps on every rank."""
import json
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from bromoc_gb300 import abi, replicas, synth
        from oracle import oracle
        oracle.build()
        spec = synth.bulk_kcl(seed=replicas.replica_seed(3, rank), n_per=20, L=30.0)
        o = oracle.create(200)
        spec.push(o)
        o.bd_steps(2, seed=replicas.replica_seed(11, rank), step0=0)
        x = o.get_particles()[0]
        t_ms, ps = 10.0 + rank, 2.0 * len(x) * (rank + 1)
        tmax, ptot = replicas.aggregate(t_ms, ps)
        with open(os.path.join(outdir, f"r{rank}.json"), "w") as f:
            json.dump({"tmax": tmax, "ptot": ptot, "x0": float(x[0]), "n": len(x)}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn",
                       join=True)
    r = [json.load(open(tmp_path / f"r{k}.json")) for k in range(2)]
    n = r[0]["n"]
    for k in range(2):
        assert r[k]["tmax"] == 11.0
        assert r[k]["ptot"] == 2.0 * n * 1 + 2.0 * n * 2
    assert not np.isclose(r[0]["x0"], r[1]["x0"])  # independent replicas
