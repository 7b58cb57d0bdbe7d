"""Multi-rank placement of a batch of independent systems, run as two gloo
ranks on CPU: every system lands on exactly one rank, the loads balance,
each rank packs its shard into the batch plan's C-ABI arguments (the code
the multi-GPU benchmark runs before gbsym_batch_create_kind) and the
library's host-side argument checks accept them and reject a corrupted
copy, and each rank's shard is solved independently (oracle arithmetic, no
data exchanged) to the same answer a single rank gives."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from sympiler_gb300 import matgen as mg
from sympiler_gb300.shard import column_range, partition_systems, shard_systems, system_cost


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _systems(seed=3, count=12):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(count):
        A = mg.lap2d(int(rng.integers(5, 40)), int(rng.integers(5, 40)))
        out.append(mg.tril(A))
    return out


def _worker(rank, world, port, result_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    import torch
    import ctypes as C

    from sympiler_gb300._lib import ERR_BAD_MATRIX, LOWER_DIAG_LAST, F64, lib
    from sympiler_gb300.plans import batch_arguments
    orc = oracle.orc()
    systems = _systems()
    costs = [system_cost(L.n, L.nnz) for L in systems]
    mine = partition_systems(costs, world)[rank]
    # the benchmark's shard-to-batch-plan path, host side
    idx, shard = shard_systems([(L.n, *L.astuple()) for L in systems], rank, world)
    assert idx == mine
    nsys, ns, ps, is_, xs, keep = batch_arguments(shard)
    assert nsys == len(mine) and [ns[q] for q in range(nsys)] == [systems[q].n for q in mine]
    for (n, p, i, x) in shard:
        assert p[0] == 0 and p[n] == len(i) and i.min() >= 0 and i.max() < n
    # a shard whose system has a column outside it is refused before any device work
    n0, p0, i0, x0 = shard[0]
    bad_i = i0.copy()
    bad_i[p0[1] - 1] = n0  # the first row's diagonal now points past its system
    bad = [(n0, p0, bad_i, x0)] + list(shard[1:])
    nb, nsb, psb, isb, xsb, keepb = batch_arguments(bad)
    h = C.c_void_p()
    st = lib().gbsym_batch_create_kind(C.byref(h), nb, nsb, psb, isb, xsb, LOWER_DIAG_LAST, F64, None)
    assert st == ERR_BAD_MATRIX and not h.value
    # each rank solves only its systems; nothing is exchanged on the data path
    sums = np.zeros(len(systems))
    for q in mine:
        L = systems[q]
        x = np.ones(L.n)
        orc.sptrsv_csr(L.n, *L.astuple(), x)
        sums[q] = x.sum()
    # gather only for the check
    t = torch.from_numpy(sums)
    dist.all_reduce(t)
    owners = torch.zeros(len(systems), dtype=torch.int64)
    for q in mine:
        owners[q] += 1
    dist.all_reduce(owners)
    load = torch.tensor([sum(costs[q] for q in mine)], dtype=torch.int64)
    loads = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(loads, load)
    if rank == 0:
        np.save(os.path.join(result_dir, "sums.npy"), t.numpy())
        np.save(os.path.join(result_dir, "owners.npy"), owners.numpy())
        np.save(os.path.join(result_dir, "loads.npy"), np.array([int(v.item()) for v in loads]))
    dist.destroy_process_group()


def test_partition_is_exact_cover_and_balanced():
    costs = [5, 9, 1, 7, 3, 3, 8, 2]
    parts = partition_systems(costs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) <= (4 / 3) * (sum(costs) / 3) + max(costs)


def test_two_gloo_ranks_solve_disjoint_shards(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    owners = np.load(tmp_path / "owners.npy")
    assert np.all(owners == 1)
    loads = np.load(tmp_path / "loads.npy")
    assert loads.max() <= 1.34 * loads.mean() + 1
    import oracle
    orc = oracle.orc()
    ref = []
    for L in _systems():
        x = np.ones(L.n)
        orc.sptrsv_csr(L.n, *L.astuple(), x)
        ref.append(x.sum())
    assert np.array_equal(np.load(tmp_path / "sums.npy"), np.array(ref))


def _column_worker(rank, world, port, result_dir):
    """One solve's right-hand-side columns split over the ranks: each rank
    solves its block against its own copy of the factor (oracle arithmetic
    on CPU), nothing crosses ranks but the final check's gather."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    import torch
    orc = oracle.orc()
    L = mg.tril(mg.lap2d(30, 20))
    k = 7
    B = np.random.default_rng(21).standard_normal((k, L.n))
    c0, c1 = column_range(k, rank, world)
    out = np.zeros((k, L.n))
    for c in range(c0, c1):
        x = B[c].copy()
        orc.sptrsv_csr(L.n, *L.astuple(), x)
        out[c] = x
    t = torch.from_numpy(out)
    dist.all_reduce(t)
    if rank == 0:
        np.save(os.path.join(result_dir, "cols.npy"), t.numpy())
    dist.destroy_process_group()


def test_column_ranges_cover_every_column_once():
    for k in (1, 7, 64, 65):
        for world in (1, 2, 3, 8):
            spans = [column_range(k, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == k
            assert all(spans[r][1] == spans[r + 1][0] for r in range(world - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_split_the_columns(tmp_path):
    world = 2
    mp.spawn(_column_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    import oracle
    orc = oracle.orc()
    L = mg.tril(mg.lap2d(30, 20))
    B = np.random.default_rng(21).standard_normal((7, L.n))
    for c in range(7):
        orc.sptrsv_csr(L.n, *L.astuple(), B[c])
    assert np.array_equal(np.load(tmp_path / "cols.npy"), B)
