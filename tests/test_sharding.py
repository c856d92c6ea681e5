"""Member sharding over ranks: two gloo ranks on CPU each filter their share
of an ensemble with the oracle; the gathered result equals the whole-ensemble
run, and the timing reduction takes the max over ranks."""
import os
import socket

import numpy as np
import pytest

from standalone_mgbf_loc_gb300.sharding import member_range


def test_member_range_partitions():
    for n in (0, 1, 7, 80):
        for w in (1, 2, 3, 8):
            got = [member_range(n, r, w) for r in range(w)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            assert max(e - b for b, e in got) - min(e - b for b, e in got) <= 1
    with pytest.raises(ValueError):
        member_range(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, members, lm, out_dir):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from standalone_mgbf_loc_gb300.sharding import max_over_ranks
    from tests.helpers import canonical, canonical_z
    b, e = member_range(members, rank, world)
    x = np.random.default_rng(0).standard_normal((16, 16, members * lm))
    mine = x[..., b * lm:e * lm]
    oc = O.OracleConfig(I=16, J=16, nk=(e - b) * lm, hx=3, hy=3, hz=1, p=2, ampl01=canonical_z(1),
                        ampl02=canonical(3), gm=2, weights=[1.0, 0.5], proc=6, lm=lm, nzcol=e - b, nthreads=1)
    y = O.filter_compact(oc, mine)
    np.save(os.path.join(out_dir, f"r{rank}.npy"), y)
    m = max_over_ranks(float(rank + 1))
    np.save(os.path.join(out_dir, f"max{rank}.npy"), np.array([m]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_members(tmp_path):
    import torch.multiprocessing as mp
    members, lm, world = 5, 4, 2
    mp.start_processes(_worker, args=(world, _free_port(), members, lm, str(tmp_path)), nprocs=world,
                       start_method="spawn")
    from oracle import oracle as O
    from tests.helpers import canonical, canonical_z
    x = np.random.default_rng(0).standard_normal((16, 16, members * lm))
    oc = O.OracleConfig(I=16, J=16, nk=members * lm, hx=3, hy=3, hz=1, p=2, ampl01=canonical_z(1),
                        ampl02=canonical(3), gm=2, weights=[1.0, 0.5], proc=6, lm=lm, nzcol=members)
    full = O.filter_compact(oc, x)
    parts = [np.load(tmp_path / f"r{r}.npy") for r in range(world)]
    assert np.array_equal(np.concatenate(parts, axis=2), full)
    assert all(float(np.load(tmp_path / f"max{r}.npy")[0]) == 2.0 for r in range(world))
