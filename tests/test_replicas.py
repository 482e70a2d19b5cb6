"""Two CPU ranks (gloo) trace disjoint particle ranges and sum their tallies; the sum equals
one process tracing both ranges (the multi-GPU decomposition, tested without GPUs)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, out_dir, fail_rank):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    from molflow_sources_gb300.model import build_pipe
    from molflow_sources_gb300.replicas import rank_particle_offset, reduce_state
    from oracle.oracle import Oracle
    m = build_pipe(step=16)
    m.tex_width[3] = 8
    m.tex_height[3] = 8
    m.count_flags[3] = 4
    if rank == fail_rank:
        dist.destroy_process_group()
        raise SystemExit(3)   # a rank that leaves before the reduction
    st, _ = Oracle(m).run(n, seed=99, first_particle=rank_particle_offset(rank), threads=1)
    try:
        reduce_state(st)
    except Exception as e:   # the surviving rank learns of the loss from the collective
        np.save(os.path.join(out_dir, "error_%d.npy" % rank), np.array([1]))
        dist.destroy_process_group() if dist.is_initialized() else None
        return
    if rank == 0:
        np.save(os.path.join(out_dir, "fc.npy"), st.facet_counts)
        np.save(os.path.join(out_dir, "tex.npy"), st.texture)
    dist.destroy_process_group()


def test_two_rank_sum_equals_single_process(tmp_path):
    n = 3000
    port = _free_port()
    mp.spawn(_worker, args=(2, port, n, str(tmp_path), -1), nprocs=2, join=True)
    from molflow_sources_gb300.model import build_pipe, SimuState
    from molflow_sources_gb300.replicas import rank_particle_offset
    from oracle.oracle import Oracle
    m = build_pipe(step=16)
    m.tex_width[3] = 8
    m.tex_height[3] = 8
    m.count_flags[3] = 4
    orc = Oracle(m)
    ref = SimuState(m)
    for r in range(2):
        orc.run(n, seed=99, first_particle=rank_particle_offset(r), state=ref, threads=1)
    assert np.array_equal(np.load(tmp_path / "fc.npy"), ref.facet_counts)
    np.testing.assert_allclose(np.load(tmp_path / "tex.npy"), ref.texture, rtol=1e-12)


def test_lost_rank_is_reported_not_hung(tmp_path):
    port = _free_port()
    ctx = mp.start_processes(_worker, args=(2, port, 500, str(tmp_path), 1), nprocs=2, join=False, start_method="spawn")
    for p in ctx.processes:
        p.join(timeout=60)
        assert not p.is_alive()
    assert ctx.processes[1].exitcode == 3
    assert (tmp_path / "error_0.npy").exists() or ctx.processes[0].exitcode != 0
