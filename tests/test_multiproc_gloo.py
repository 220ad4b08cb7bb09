"""Two ranks over gloo: replicas over event shards reproduce the single-process result (CPU, oracle compute)."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    import oracle as O
    from gwfast_gb300 import shard, synthetic
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    ev = synthetic.bbh_events(5, seed=21)
    f0 = np.geomspace(10., 1e4, 500)
    det = O.Detector(46.455, -119.408, 171., 'L', fmin=10., psd_f=f0, psd_S=O.aligo_psd(f0), earth=True)

    def fn(e):
        return O.snr(det, O.Model('PhenomD'), O.to_params(e), 128).numpy()
    full = shard.run_sharded(fn, ev, rank, world)
    if rank == 0:
        q.put((full, fn(ev)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_matches_single_process():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    full, single = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert np.array_equal(full, single) or np.allclose(full, single, rtol=1e-14)
