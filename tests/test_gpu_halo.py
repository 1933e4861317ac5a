"""The multi-rank halo path with the library's kernels doing each rank's
arithmetic (minife_gb300.halo.DeviceOps: the local CSR matvec, dot, waxpby
and the send-buffer gather on the GPU, the halo staged through host memory
and exchanged over gloo).  Two rank processes share the one GPU here: their
kernels never wait on one another (every exchange is a host-side step
between launches).  The solution matches the oracle's single-rank CG."""
import os
import socket

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU-only machines
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, dims, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch as T
    import torch.distributed as dist
    from oracle import oracle as Oo
    from minife_gb300 import halo as H
    T.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ro, cols, vals, b = Oo.build_system(*dims)
        d = H.Decomposition(*dims, world)
        comm = H.DistComm()
        gro, gcols, gvals, gb = H.global_rows_of(d, rank, ro, cols, vals, b)
        A = H.make_local_matrix(d, rank, gro, gcols, gvals, comm)
        ops = H.DeviceOps(0)
        bd = T.as_tensor(gb).cuda()
        x = T.zeros(A.nrows, dtype=T.float64, device="cuda")
        it, nr, nr0 = H.cg_solve(A, bd, x, ops, comm, max_iter=1000, tol=1e-10,
                                 tol_mode="relative")
        parts = [None] * world
        dist.all_gather_object(parts, (rank, x.cpu().numpy()))
        if rank == 0:
            xg = np.empty(d.nrows)
            for p, xp in parts:
                xg[d.nodes[p]] = xp
            np.save(os.path.join(out, "x.npy"), xg)
            with open(os.path.join(out, "it.txt"), "w") as f:
                f.write("%d" % it)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [1, 2])
def test_halo_cg_on_gpu_ranks(tmp_path, world):
    import torch.multiprocessing as mp
    dims = (12, 10, 14)
    mp.start_processes(_rank_main, args=(world, free_port(), dims, str(tmp_path)), nprocs=world,
                       start_method="spawn")
    xg = np.load(os.path.join(tmp_path, "x.npy"))
    it = int(open(os.path.join(tmp_path, "it.txt")).read())
    ro, cols, vals, b = O.build_system(*dims)
    xo, ito, nro, st = O.cg_solve(ro, cols, vals, b, max_iter=1000, tol=1e-10, tol_mode=1)
    assert abs(it - ito) <= 1
    assert np.linalg.norm(xg - xo) <= 1e-9 * np.linalg.norm(xo)
