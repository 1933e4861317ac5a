"""The multi-rank halo path (minife_gb300.halo: the reference's
box_partition, make_local_matrix, exchange_externals and distributed CG) on
CPU ranks: the partition covers the box, every rank's local matrix applied
to its owned entries and exchanged externals gives its rows of the global
matvec, and the CG over gloo ranks (2 and 3, the second an uneven recursive
bisection) reaches the oracle's single-rank solution.  The per-rank
arithmetic here is the oracle's (a CPU restatement); the library's GPU
kernels take its place on GPU ranks."""
import os
import socket

import numpy as np
import pytest

from oracle import oracle as O
from minife_gb300 import halo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class HostOps:
    """Per-rank arithmetic on the host with the oracle's kernels."""

    def prepare(self, A):
        self.A = A
        self.xext = np.zeros(A.nrows + A.n_external)
        self.n = A.nrows

    def empty(self, n):
        return np.zeros(n)

    def copy_owned(self, v, xext):
        xext[: self.n] = v

    def matvec(self, xext, out):
        out[:] = O.matvec(self.A.row_offsets, self.A.cols, self.A.vals, xext)

    def dot(self, u, v):
        return O.dot(u, v)

    def waxpby(self, a, u, b, v, w):
        w[:] = O.waxpby(a, u, b, v)

    def pack(self, xext, i):
        return xext[self.A.send_rows[i]]

    def put(self, xext, off, values):
        xext[off:off + values.size] = values


@pytest.mark.parametrize("dims", [(6, 5, 7), (9, 4, 3), (2, 2, 2)])
@pytest.mark.parametrize("nranks", [1, 2, 3, 4, 5, 8])
def test_partition_owns_every_node_once(dims, nranks):
    d = halo.Decomposition(*dims, nranks)
    owned = np.concatenate(d.nodes)
    assert np.array_equal(np.sort(owned), np.arange((dims[0] + 1) * (dims[1] + 1) * (dims[2] + 1)))
    assert np.array_equal(np.sort(d.row_of_node), np.arange(d.nrows))
    # element boxes tile the global box
    cells = sum((b[0][1] - b[0][0]) * (b[1][1] - b[1][0]) * (b[2][1] - b[2][0])
                for b in d.elem_boxes)
    assert cells == dims[0] * dims[1] * dims[2]
    for p, ids in enumerate(d.nodes):
        assert (d.owner(d.row_of_node[ids]) == p).all()


@pytest.mark.parametrize("dims,nranks", [((6, 5, 7), 2), ((6, 5, 7), 3), ((5, 6, 4), 4),
                                         ((7, 3, 5), 5)])
def test_local_matvec_is_the_global_rows(dims, nranks):
    """Each rank's local matrix times (its owned entries, then its externals
    in local order) equals its rows of the global matvec; the externals are
    exactly the off-rank columns, each requested once from its owner, and
    every request matches the owner's send list."""
    ro, cols, vals, b = O.build_system(*dims)
    d = halo.Decomposition(*dims, nranks)
    x = np.random.default_rng(3).standard_normal(ro.size - 1)
    y = O.matvec(ro, cols, vals, x)
    xr = np.empty_like(x)
    xr[d.row_of_node] = x          # x in the multi-rank numbering
    locs = []
    for p in range(nranks):
        gro, gcols, gvals, gb = halo.global_rows_of(d, p, ro, cols, vals, b)
        A = halo.make_local_matrix(d, p, gro, gcols, gvals)
        locs.append(A)
        start = d.start_row[p]
        offrank = np.unique(gcols[(gcols < start) | (gcols >= start + A.nrows)])
        assert np.array_equal(np.sort(A.external_rows), offrank)
        xext = np.concatenate([xr[start:start + A.nrows], xr[A.external_rows]])
        yl = O.matvec(A.row_offsets, A.cols, A.vals, xext)
        ref = y[d.nodes[p]]
        scale = O.matvec(ro, cols, np.abs(vals), np.abs(x))[d.nodes[p]] + 1e-300
        assert np.all(np.abs(yl - ref) <= 30 * 2.0 ** -53 * scale)
    # send lists: what rank q sends to p is what p receives from q, in p's order
    for p, A in enumerate(locs):
        off = A.nrows
        for q, n in zip(A.neighbors, A.recv_length):
            B = locs[q]
            i = B.neighbors.index(p)
            sent_rows = B.send_rows[i] + d.start_row[q]
            assert np.array_equal(sent_rows, A.external_rows[off - A.nrows:off - A.nrows + n])
            off += n
        assert off == A.nrows + A.n_external


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, dims, tol, tol_mode, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from oracle import oracle as Oo
    from minife_gb300 import halo as H
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ro, cols, vals, b = Oo.build_system(*dims)
        d = H.Decomposition(*dims, world)
        comm = H.DistComm()
        gro, gcols, gvals, gb = H.global_rows_of(d, rank, ro, cols, vals, b)
        A = H.make_local_matrix(d, rank, gro, gcols, gvals, comm)
        x = np.zeros(A.nrows)
        it, nr, nr0 = H.cg_solve(A, gb, x, HostOps(), comm, max_iter=500, tol=tol,
                                 tol_mode=tol_mode)
        parts = [None] * world
        dist.all_gather_object(parts, (rank, x))
        if rank == 0:
            xg = np.empty(d.nrows)
            for p, xp in parts:
                xg[d.nodes[p]] = xp
            np.save(os.path.join(out, "x.npy"), xg)
            with open(os.path.join(out, "it.txt"), "w") as f:
                f.write("%d %r %r" % (it, nr, nr0))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("tol,mode", [(1e-10, "relative"), (2.220446049250313e-16, "absolute")])
def test_distributed_cg_matches_single_rank(tmp_path, world, tol, mode):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    dims = (8, 6, 9)
    mp.start_processes(_rank_main, args=(world, free_port(), dims, tol, mode, str(tmp_path)),
                       nprocs=world, start_method="spawn")
    xg = np.load(os.path.join(tmp_path, "x.npy"))
    it, nr, nr0 = open(os.path.join(tmp_path, "it.txt")).read().split()
    ro, cols, vals, b = O.build_system(*dims)
    xo, ito, nro, st = O.cg_solve(ro, cols, vals, b, max_iter=500, tol=tol,
                                  tol_mode=1 if mode == "relative" else 0)
    # the ranks sum the dots in another order: counts may part by an iteration
    # or two near the rounding floor; the converged solutions agree closely
    assert abs(int(it) - ito) <= (1 if mode == "relative" else 3)
    assert np.linalg.norm(xg - xo) <= 1e-9 * np.linalg.norm(xo)
