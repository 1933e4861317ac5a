"""The reference's multi-rank decomposition of the box, its local matrices and
its halo exchange, over torch.distributed ranks.

miniFE runs one MPI rank per box piece (ref/src/main.cpp:112): each rank owns
the nodes of its piece, builds the CSR rows of those nodes with global column
numbers, turns them into a local matrix whose off-rank columns ("externals")
follow the owned ones (ref/src/make_local_matrix.hpp:42-442), and before
every matvec receives the externals' values from their owners
(ref/src/exchange_externals.hpp:44-161); dots are summed over the ranks
(ref/src/Vector_functions.hpp:196-222).  This module restates that path:

* ``box_partition`` -- the recursive bisection of ref/utils/BoxPartition.cpp
  :80-130 (halve the rank range, cutting along z, then y, then x, then z
  again, ...);
* ``Decomposition`` -- each rank's element box, its node box (the element
  box plus the last node layer on the global high faces,
  simple_mesh_description.hpp:44-53) and the global row numbering of
  create_map_id_to_row (box_utils.hpp:233-315): rank after rank, each
  rank's nodes in box order;
* ``make_local_matrix`` -- a rank's rows (columns sorted by global row, as
  MatrixInitOp.hpp:40-56 sorts them), owned columns renumbered to local
  rows, externals numbered after them grouped by owning rank in the order
  the owners first appear (make_local_matrix.hpp:65-120), and the send
  lists each owner builds from its neighbours' requests (:200-330);
* ``exchange_externals`` -- packs the send buffers, exchanges them with the
  neighbours (non-blocking point-to-point) and places the received values
  after the owned entries of x;
* ``cg_solve`` -- cg_solve.hpp:69-229 on the local pieces, every dot an
  all-reduce of the local dots.

The per-rank arithmetic comes from an operations object -- prepare(A)
(which sets ``xext``, the owned entries followed by the externals),
empty(n), copy_owned(v, xext), matvec(xext, out), dot(u, v), waxpby(a, u,
b, v, w) (w = a u + b v), pack(xext, i) (neighbour i's send buffer, on the
host), put(xext, off, values) and, optionally, finish() (raises if the
device reported an error during the solve): ``DeviceOps`` runs it on the rank's GPU
with the library's kernels (generic CSR matvec, dot, waxpby, gather),
staging the halo through host memory for the transport; tests run the
same logic on CPU ranks (gloo) with operations of their own.
One GPU per rank is assumed; nothing here lets kernels of different ranks
wait on one another (every exchange is a host-side step between launches).
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field

import numpy as np


# --------------------------------------------------------------------------
# partition and row numbering
# --------------------------------------------------------------------------
def box_partition(nprocs: int, box):
    """Element boxes of nprocs ranks for the global element box
    ``box`` = [[x0, x1], [y0, y1], [z0, z1]] (BoxPartition.cpp:80-130: split
    the rank range in halves, the axis z first, then y, then x, ...; the
    upper half gets floor(n * np_upp / np) of the n cells)."""
    out = [None] * nprocs

    def rec(ip, up, axis, b):
        np_ = up - ip
        if np_ == 1:
            out[ip] = copy.deepcopy(b)
            return
        n = b[axis][1] - b[axis][0]
        np_low = np_ // 2
        np_upp = np_ - np_low
        n_upp = int(float(n) * (float(np_upp) / float(np_)))
        n_low = n - n_upp
        nxt = (axis + 2) % 3
        if np_low:
            d = copy.deepcopy(b)
            d[axis][1] = d[axis][0] + n_low
            rec(ip, ip + np_low, nxt, d)
        if np_upp:
            d = copy.deepcopy(b)
            d[axis][0] += n_low
            d[axis][1] = d[axis][0] + n_upp
            rec(ip + np_low, ip + np_low + np_upp, nxt, d)

    rec(0, nprocs, 2, [list(box[0]), list(box[1]), list(box[2])])
    return out


def node_box(global_box, elem_box):
    """Nodes a rank owns (simple_mesh_description.hpp:44-53): its element
    box, plus one node layer along each axis where the box reaches the
    global high face."""
    nb = copy.deepcopy(elem_box)
    for i in range(3):
        if elem_box[i][1] > elem_box[i][0] and elem_box[i][1] == global_box[i][1]:
            nb[i][1] += 1
    return nb


class Decomposition:
    """nranks pieces of the nx x ny x nz element box.  Node ids are the
    single-rank row numbers (x fastest); ``row_of_node[id]`` is the global
    row of the multi-rank numbering, ``start_row[p]`` rank p's first row,
    ``nodes[p]`` the node ids rank p owns in its row order."""

    def __init__(self, nx: int, ny: int, nz: int, nranks: int):
        self.dims = (nx, ny, nz)
        self.nranks = nranks
        self.Nx, self.Ny, self.Nz = nx + 1, ny + 1, nz + 1
        gbox = [[0, nx], [0, ny], [0, nz]]
        self.elem_boxes = box_partition(nranks, gbox)
        self.node_boxes = [node_box(gbox, b) for b in self.elem_boxes]
        n = self.Nx * self.Ny * self.Nz
        self.row_of_node = np.full(n, -1, np.int64)
        self.nodes = []
        self.start_row = []
        start = 0
        for nb in self.node_boxes:
            ix = np.arange(nb[0][0], nb[0][1])
            iy = np.arange(nb[1][0], nb[1][1])
            iz = np.arange(nb[2][0], nb[2][1])
            ids = (iz[:, None, None] * self.Ny + iy[None, :, None]) * self.Nx + ix[None, None, :]
            ids = ids.reshape(-1)
            self.nodes.append(ids)
            self.start_row.append(start)
            self.row_of_node[ids] = start + np.arange(ids.size)
            start += ids.size
        if start != n or (self.row_of_node < 0).any():
            raise RuntimeError("the node boxes do not partition the nodes")
        self.nrows = n
        self.owner_of_row = np.repeat(np.arange(nranks), [a.size for a in self.nodes])

    def owner(self, rows):
        """Owning rank of global rows (the last rank whose first row is at
        or below each, make_local_matrix.hpp:110-118)."""
        return np.searchsorted(np.asarray(self.start_row), rows, side="right") - 1


# --------------------------------------------------------------------------
# local matrix and exchange plan
# --------------------------------------------------------------------------
@dataclass
class LocalMatrix:
    """Rank p's piece: rows start_row .. start_row + nrows - 1 of the global
    numbering; columns < nrows are owned rows, the others externals."""
    rank: int
    start_row: int
    nrows: int
    row_offsets: np.ndarray          # int32, nrows + 1
    cols: np.ndarray                 # int32, local column numbers
    vals: np.ndarray                 # float64
    external_rows: np.ndarray        # global row of each external, local order
    neighbors: list = field(default_factory=list)      # exchange partners, in order
    recv_length: list = field(default_factory=list)    # externals from each partner
    send_rows: list = field(default_factory=list)      # per partner: local rows to send

    @property
    def n_external(self) -> int:
        return int(self.external_rows.size)


def global_rows_of(dec: Decomposition, rank: int, ro, cols, vals, b):
    """Rank ``rank``'s rows of the single-rank system (ro, cols, vals, b in
    node numbering) in the multi-rank numbering, each row's columns sorted
    (MatrixInitOp.hpp:40-56); returns (row_offsets, global cols, vals, b)."""
    ids = dec.nodes[rank]
    lens = (ro[ids + 1] - ro[ids]).astype(np.int64)
    out_ro = np.zeros(ids.size + 1, np.int64)
    np.cumsum(lens, out=out_ro[1:])
    total = int(out_ro[-1])
    idx = np.repeat(ro[ids].astype(np.int64), lens) + (np.arange(total) - np.repeat(out_ro[:-1], lens))
    gcols = dec.row_of_node[cols[idx]]
    gvals = vals[idx]
    # sort each row's entries by global column
    row_id = np.repeat(np.arange(ids.size), lens)
    order = np.lexsort((gcols, row_id))
    return out_ro, gcols[order], gvals[order], b[ids].copy()


def make_local_matrix(dec: Decomposition, rank: int, row_offsets, gcols, vals, comm=None):
    """make_local_matrix.hpp:42-442 for rank ``rank``: owned columns become
    local rows, externals are numbered after them -- grouped by owning rank,
    the groups in the order their ranks first appear and each group in the
    order its columns first appear in the rows -- and the send lists are
    built from the neighbours' requests (``comm``: a torch.distributed
    handle exchanging the request lists; None computes them for every rank
    from the decomposition alone, as a single process can)."""
    start = dec.start_row[rank]
    nrows = dec.nodes[rank].size
    stop = start + nrows - 1
    owned = (gcols >= start) & (gcols <= stop)
    # externals in order of first appearance
    ext_cols = gcols[~owned]
    _, first = np.unique(ext_cols, return_index=True)
    ext_first = ext_cols[np.sort(first)]
    ext_proc = dec.owner(ext_first)
    # group by processor, groups in order of first appearance
    proc_order = []
    for p in ext_proc:
        if not proc_order or p not in proc_order:
            proc_order.append(int(p))
    new_order = np.concatenate([ext_first[ext_proc == p] for p in proc_order]) if proc_order \
        else np.zeros(0, np.int64)
    local_of_ext = {int(g): nrows + k for k, g in enumerate(new_order)}
    lcols = np.where(owned, gcols - start, 0).astype(np.int64)
    if (~owned).any():
        lcols[~owned] = np.fromiter((local_of_ext[int(g)] for g in gcols[~owned]), np.int64,
                                    count=int((~owned).sum()))
    recv_length = [int((dec.owner(new_order) == p).sum()) for p in proc_order]
    # requests: what every rank needs from each other rank
    requests = {p: new_order[dec.owner(new_order) == p] for p in proc_order}
    if comm is None:
        incoming = _requests_from_decomposition(dec, rank)
    else:
        incoming = comm.exchange_requests(rank, requests)
    neighbors = list(proc_order)
    for q in sorted(incoming):
        if q not in neighbors:
            neighbors.append(q)      # a rank that only receives from us
    recv = {p: n for p, n in zip(proc_order, recv_length)}
    send_rows = [np.asarray(incoming.get(q, np.zeros(0, np.int64)), np.int64) - start
                 for q in neighbors]
    return LocalMatrix(rank, start, nrows, np.asarray(row_offsets, np.int32),
                       lcols.astype(np.int32), np.ascontiguousarray(vals, np.float64),
                       new_order.astype(np.int64), neighbors,
                       [recv.get(q, 0) for q in neighbors], send_rows)


def _requests_from_decomposition(dec: Decomposition, rank: int):
    """The rows every other rank requests from ``rank``, in the requesting
    rank's external order, computed from the box structure alone (each
    requester's externals are the off-rank 27-point neighbours of its rows,
    in first-appearance order over its sorted rows)."""
    out = {}
    for q in range(dec.nranks):
        if q == rank:
            continue
        need = _external_order(dec, q)
        mine = need[dec.owner(need) == rank]
        if mine.size:
            out[q] = mine
    return out


def _external_order(dec: Decomposition, q: int):
    Nx, Ny, Nz = dec.Nx, dec.Ny, dec.Nz
    ids = dec.nodes[q]
    iz, rem = np.divmod(ids, Nx * Ny)
    iy, ix = np.divmod(rem, Nx)
    nb = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                jx, jy, jz = ix + dx, iy + dy, iz + dz
                ok = (jx >= 0) & (jx < Nx) & (jy >= 0) & (jy < Ny) & (jz >= 0) & (jz < Nz)
                col = np.where(ok, dec.row_of_node[np.clip((jz * Ny + jy) * Nx + jx, 0,
                                                           dec.nrows - 1)], -1)
                nb.append(col)
    cols = np.stack(nb, 1)                   # rows x 27, -1 where absent
    cols = np.sort(np.where(cols < 0, np.iinfo(np.int64).max, cols), 1)
    start, stop = dec.start_row[q], dec.start_row[q] + ids.size - 1
    flat = cols.reshape(-1)
    flat = flat[(flat != np.iinfo(np.int64).max) & ((flat < start) | (flat > stop))]
    _, first = np.unique(flat, return_index=True)
    ext_first = flat[np.sort(first)]
    procs = dec.owner(ext_first)
    order = []
    for p in procs:
        if p not in order:
            order.append(int(p))
    return np.concatenate([ext_first[procs == p] for p in order]) if order else ext_first


class DistComm:
    """Point-to-point and all-reduce over torch.distributed (gloo for CPU
    ranks; a GPU build stages the halo through host buffers)."""

    def __init__(self):
        import torch.distributed as dist
        self.dist = dist
        self.rank = dist.get_rank()
        self.size = dist.get_world_size()

    def exchange_requests(self, rank, requests):
        """Send each owner the global rows we need from it; return the rows
        each other rank needs from us (make_local_matrix.hpp:200-330)."""
        objs = [None] * self.size
        self.dist.all_gather_object(objs, {int(p): np.asarray(v, np.int64)
                                           for p, v in requests.items()})
        return {q: objs[q][rank] for q in range(self.size) if q != rank and rank in objs[q]}

    def allreduce_sum(self, v: float) -> float:
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t)
        return float(t.item())

    def exchange(self, A: LocalMatrix, send_buffers, recv_buffers):
        """Non-blocking receives from every neighbour, then the sends, then
        the waits (exchange_externals.hpp:96-152); buffers are CPU float64
        tensors, recv_buffers[i] of length A.recv_length[i]."""
        reqs = []
        for q, rb in zip(A.neighbors, recv_buffers):
            if rb.numel():
                reqs.append(self.dist.irecv(rb, src=q))
        for q, sb in zip(A.neighbors, send_buffers):
            if sb.numel():
                reqs.append(self.dist.isend(sb, dst=q))
        for r in reqs:
            r.wait()


def exchange_externals(A: LocalMatrix, x_ext, ops, comm):
    """x_ext holds A.nrows owned entries followed by A.n_external slots:
    pack the send buffers (x[elements_to_send]), exchange them, and place
    the received values after the owned entries, each neighbour's block in
    neighbour order (exchange_externals.hpp:44-161)."""
    if comm is None or comm.size < 2:
        return
    import torch
    sends = [torch.as_tensor(np.ascontiguousarray(ops.pack(x_ext, i), np.float64))
             for i in range(len(A.neighbors))]
    recvs = [torch.empty(n, dtype=torch.float64) for n in A.recv_length]
    comm.exchange(A, sends, recvs)
    off = A.nrows
    for rb in recvs:
        n = rb.numel()
        if n:
            ops.put(x_ext, off, rb.numpy())
        off += n


# --------------------------------------------------------------------------
# distributed CG
# --------------------------------------------------------------------------
def cg_solve(A: LocalMatrix, b, x, ops, comm, max_iter: int = 200,
             tol: float = 2.220446049250313e-16, tol_mode: str = "absolute"):
    """cg_solve (cg_solve.hpp:69-229) on the rank's piece: b, x hold the
    owned entries (x updated in place); every matvec exchanges the
    externals first (matvec_std, SparseMatrix_functions.hpp:548-556), every
    dot is the all-reduced sum of the ranks' dots.  Returns (num_iters,
    normr, normr0)."""
    ops.prepare(A)
    n = A.nrows
    size = 1 if comm is None else comm.size

    def gdot(u, v):
        d = ops.dot(u, v)
        return d if size < 2 else comm.allreduce_sum(d)

    def matvec(v_owned, out):
        ops.copy_owned(v_owned, ops.xext)
        exchange_externals(A, ops.xext, ops, comm)
        ops.matvec(ops.xext, out)

    r = ops.empty(n)
    p = ops.empty(n)
    Ap = ops.empty(n)
    matvec(x, Ap)
    ops.waxpby(1.0, b, -1.0, Ap, r)
    rtrans = gdot(r, r)
    normr = math.sqrt(rtrans)
    normr0 = normr
    tol_abs = tol * normr0 if tol_mode == "relative" else tol
    num_iters = 0
    k = 1
    while k <= max_iter and normr > tol_abs:
        if k == 1:
            ops.waxpby(1.0, r, 0.0, r, p)
        else:
            oldrtrans = rtrans
            rtrans = gdot(r, r)
            beta = rtrans / oldrtrans
            ops.waxpby(1.0, r, beta, p, p)
        normr = math.sqrt(rtrans)
        matvec(p, Ap)
        p_ap = gdot(Ap, p)
        if p_ap <= 0:
            break  # breakdown (cg_solve.hpp:186-198): the caller sees num_iters
        alpha = rtrans / p_ap
        ops.waxpby(1.0, x, alpha, p, x)
        ops.waxpby(1.0, r, -alpha, Ap, r)
        num_iters = k
        k += 1
    finish = getattr(ops, "finish", None)
    if finish is not None:
        finish()
    return num_iters, normr, normr0


class DeviceOps:
    """The per-rank arithmetic on the rank's GPU with the library's kernels:
    the local CSR (owned and external columns) through the generic CSR
    matvec, dot and waxpby, the send buffers packed by mfe_gather and staged
    through host memory for the transport."""

    def __init__(self, device: int = 0):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)

    def finish(self):
        """The context's error word of the solve's products (bounded waits):
        MiniFEError (MFE_TIMEOUT) if one gave up."""
        self.M.default_context().synchronize()

    def prepare(self, A: LocalMatrix):
        import minife_gb300 as M
        t = self.torch
        self.M = M
        self.A = M.CSRMatrix(t.as_tensor(A.row_offsets).to(self.dev),
                             t.as_tensor(A.cols).to(self.dev),
                             t.as_tensor(A.vals).to(self.dev),
                             num_cols=A.nrows + A.n_external)
        self.send_idx = [t.as_tensor(s.astype(np.int32)).to(self.dev) for s in A.send_rows]
        self.xext = t.zeros(A.nrows + A.n_external, dtype=t.float64, device=self.dev)
        self.n = A.nrows

    def empty(self, n):
        return self.torch.zeros(n, dtype=self.torch.float64, device=self.dev)

    def copy_owned(self, v, xext):
        xext[: self.n].copy_(v)

    def matvec(self, xext, out):
        self.M.matvec(self.A, xext, out)

    def dot(self, u, v):
        return self.M.dot(u, v)

    def waxpby(self, a, u, b, v, w):
        self.M.waxpby(a, u, b, v, w)

    def pack(self, xext, i):
        return self.M.gather(xext, self.send_idx[i]).cpu().numpy()

    def put(self, xext, off, values):
        xext[off:off + values.size].copy_(self.torch.as_tensor(values))
