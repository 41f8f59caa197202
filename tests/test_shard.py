"""Multi-rank split of halo parts, on CPU: LPT assignment, and world-size-2
gloo ranks whose partial counts (CPU oracle standing in for the GPU count)
sum to the whole graph's count."""
import os
import socket

import numpy as np
import pytest

import oracle
from trianglecount_gb300 import generators as gen
from trianglecount_gb300.shard import assign_parts


def test_lpt_assignment_balances_and_covers():
    work = [100, 1, 50, 49, 30, 20, 10, 5]
    a = assign_parts(work, 3)
    assert sorted(i for r in a for i in r) == list(range(len(work)))
    loads = [sum(work[i] for i in r) for r in a]
    assert max(loads) - min(loads) <= max(work)
    assert assign_parts(work, 1) == [list(range(len(work)))]
    with pytest.raises(ValueError):
        assign_parts(work, 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, k, out_path):
    import torch.distributed as dist

    from trianglecount_gb300.shard import count_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    src, dst = gen.rmat(11)
    rp, col = oracle.clean(src, dst)
    part = gen.parts_random(len(rp) - 1, k)
    parts = [oracle.halo_part(rp, col, np.diff(rp), part, p) for p in range(k)]
    total = count_sharded(parts, rank, world, lambda hp: oracle.count(hp[0], hp[1], n_roots=hp[2]),
                          work=[len(hp[1]) for hp in parts])
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(str(total))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("k", [2, 5])
def test_two_gloo_ranks_sum_to_whole(tmp_path, k):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "total")
    mp.start_processes(_rank_main, args=(2, _free_port(), k, out), nprocs=2, join=True, start_method="spawn")
    src, dst = gen.rmat(11)
    whole = oracle.pipeline(src, dst)[2]
    assert [int(open(f"{out}.{r}").read()) for r in range(2)] == [whole, whole]


def test_contiguous_parts_match_reference_construction():
    for n, k in ((10, 3), (100, 8), (5, 8), (64, 4)):
        ref = np.zeros(n, dtype=int)  # Halo_creation_preprocess.py:293-299
        l = n // k
        for i in range(k):
            ref[i * l:(i + 1) * l] = i
        assert np.array_equal(gen.parts_contig(n, k), ref)


def _gpu_rank_main(rank, world, port, k, out_path):
    """One rank: the library extracts the counting-halo parts on cuda:0 and
    counts this rank's share in one batched launch; gloo sums the ranks."""
    import torch.distributed as dist

    import trianglecount_gb300 as tc
    from trianglecount_gb300.shard import count_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    with tc.Context(0) as ctx:
        ug = ctx.ugraph_from_edges(*gen.rmat(14))
        parts = ctx.halo_extract(ug, gen.parts_random(ug.info()[0], k), k, mode="count")
        mine = assign_parts([p.nnz for p in parts], world)[rank]
        outs = ctx.batch([parts[i] for i in mine]).run() if mine else []
        by_part = dict(zip(mine, (int(x) for x in outs)))
        total = count_sharded(parts, rank, world, lambda p: by_part[parts.index(p)])
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(f"{total} {len(mine)}")
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.gpu
@pytest.mark.parametrize("k", [3, 8])
def test_two_gloo_ranks_count_parts_on_the_gpu(tmp_path, k):
    """Two processes share cuda:0 (their kernels never wait on each other):
    each counts its LPT share of the parts with libtc, and the gloo sum
    equals the oracle's count of the whole graph."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "gpu_total")
    mp.start_processes(_gpu_rank_main, args=(2, _free_port(), k, out), nprocs=2, join=True, start_method="spawn")
    whole = oracle.pipeline(*gen.rmat(14))[2]
    res = [open(f"{out}.{r}").read().split() for r in range(2)]
    assert [int(t) for t, _ in res] == [whole, whole]
    assert sum(int(n) for _, n in res) == k
