"""The replica path of bench.py --gpus N (one process per GPU, no data-path
collective) with world_size 2 on CPU over gloo: barrier, the maximum of the
ranks' times, the whole-job rate, and ranks that each run their own oracle
replica of a case."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _oracle_replica(seed):
    """One rank's replica: 5 first-order steps of the explosion on its own
    numbering of a 10 x 10 mesh; returns the total mass."""
    import mallard_gb300 as mg
    from cases import GAS, explosion
    from oracle import OracleCase, OracleMesh
    m = mg.Mesh.generate("cartesian_tri", 10, 10, 1.0, 1.0)
    m.permute_cells(seed)
    om = OracleMesh.from_arrays(m)
    oc = OracleCase(om, recon="FO", basis="legendre", poly_order=1, riemann="HLLC", **GAS)
    for z in m.zone_names[1:]:
        oc.add_boundary(m.zone_index(z), "symmetry", ())
    U, W = explosion(m)
    oc.set_state(U, W)
    oc.run(0.5, 5)
    Uo, _ = oc.get_state()
    return float((Uo[:, 0] * m.cell_volume).sum())


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from mallard_gb300.replicas import Replicas
    r = Replicas("gloo", cuda=False)
    assert (r.rank, r.world) == (rank, world)
    r.barrier()
    # rank k processed 1000 (k + 1) units in 0.5 (k + 1) seconds
    mx = r.max(0.5 * (rank + 1))
    rate = r.rate(1000.0 * (rank + 1), 0.5 * (rank + 1))
    # each rank runs its own replica (no collective on the data)
    mass = _oracle_replica(seed=rank)
    total = r.sum(mass)
    out.put((rank, mx, rate, mass, total))
    r.close()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=90) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    for rank, mx, rate, mass, total in res:
        assert mx == 1.0                                  # the slowest rank's time
        assert rate == pytest.approx(3000.0 / 1.0)        # all ranks' units over it
        assert total == pytest.approx(res[0][3] + res[1][3])
    # the replicas are the same case under two numberings: the same mass
    assert res[0][3] == pytest.approx(res[1][3], rel=1e-12)
    assert np.isfinite([r[3] for r in res]).all()


def test_single_process_needs_no_backend(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    from mallard_gb300.replicas import Replicas
    r = Replicas("gloo", cuda=False)
    assert (r.rank, r.world) == (0, 1)
    r.barrier()
    assert r.max(2.5) == 2.5 and r.rate(10.0, 2.0) == 5.0
    r.close()
