"""The multi-GPU decomposition on CPU: two gloo ranks each track their shard
of one particle set (the oracle stands in for the GPU kernel, so no GPU is
needed) and sum their diagnostics; rank 0 compares with one process tracking
all particles.  Spectra and particles-remaining counts must agree exactly,
diffusion sums to rounding."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _case():
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden as mg
    from oracle import pyoracle as po
    sc = mg.scenarios()["pic"]
    f = mg.field_from(sc, bc_flag=1)  # open boundary: some particles leave
    s = po.spectrum(50, 1e-3, 1e1)
    p0 = mg.particles_for(sc, np.random.default_rng(3), 300)
    return po, f, s, p0


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from test_particle_gb300 import shard
    dist.init_process_group("gloo", rank=rank, world_size=world)
    po, f, s, p0 = _case()
    a, b = shard.shard_range(len(p0), rank, world)
    res = po.track_fixed(f, s, p0[a:b], 0.05, 3)
    shard.reduce_diagnostics(res, dist)
    if rank == 0:
        np.savez(os.path.join(out_dir, "sharded.npz"), **{k: res[k] for k in
                                                          ("espect", "espect_escape", "dsum", "remain")})
    dist.barrier()
    dist.destroy_process_group()


def test_shard_counts_match_reference_split():
    from test_particle_gb300 import shard
    assert shard.shard_counts(10, 3) == [4, 3, 3]
    assert shard.shard_range(10, 2, 3) == (7, 10)
    assert sum(shard.shard_counts(1048577, 8)) == 1048577
    with pytest.raises(ValueError):
        shard.shard_range(10, 3, 3)


def test_two_gloo_ranks_reproduce_one_process(tmp_path):
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2,
                       start_method="spawn", join=True)
    got = np.load(tmp_path / "sharded.npz")
    po, f, s, p0 = _case()
    ref = po.track_fixed(f, s, p0, 0.05, 3)
    assert np.array_equal(got["espect"], ref["espect"])
    assert np.array_equal(got["espect_escape"], ref["espect_escape"])
    assert np.array_equal(got["remain"], ref["remain"])
    np.testing.assert_allclose(got["dsum"], ref["dsum"], rtol=1e-12, atol=1e-300)
    assert ref["espect_escape"].sum() > 0
