"""Column shard of the s-grid ring over several GPUs (one process per GPU).

The reference's MPI build (compiled with -DMPI_enable=1) splits the grid's
rows of columns over the ranks and exchanges the new slot after every update:

    lsGridSpline::compute_mpi_partition   lsgrid_spline.cpp:652-664
    cfdwm_mpi::partition_weighted         mpi_utils.h:46-64
    per-rank fill of the owned rows       lsgrid_spline.cpp:866-903
    cfdwm_mpi::allgather_columns          mpi_utils.h:69-79 (MPI_Allgatherv)
    all-gather of ETA, UX, UY, UZ         lsgrid_spline.cpp:907-910
    gradients on every rank               lsgrid_spline.cpp:912-922

Here each process loads the same model on its own GPU; ``ShardedRing`` does
one such step per ring update with the library's block calls
(``cfdwm_sgrid_step_block`` / ``_block_export`` / ``_block_import`` /
``_step_finish``) and ``allgather_rows`` over ``torch.distributed``: NCCL
between GPUs (each rank's blocks are copied into every GPU's own memory; no
multicast), gloo between CPU processes.  ``wave_force_update`` stays the
single-GPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np


def partition(weights, nranks, lib=None):
    """Rows [bounds[r], bounds[r+1]) of rank r: the work-balanced contiguous
    partition of mpi_utils.h:46-64, computed by the library on the host."""
    from . import load
    lib = lib or load()
    w = np.ascontiguousarray(weights, dtype=np.int64)
    b = np.zeros(nranks + 1, dtype=np.int32)
    rc = lib.cfdwm_partition_columns(w.ctypes.data_as(C.POINTER(C.c_long)), int(w.size), int(nranks),
                                     b.ctypes.data_as(C.POINTER(C.c_int)))
    if rc != 0:
        raise ValueError("cfdwm_partition_columns: %d" % rc)
    return [int(v) for v in b]


def _world(group):
    """(rank, size) of the process group; one process without a group is rank 0 of 1."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(group), dist.get_world_size(group)
    return 0, 1


def allgather_rows(local, bounds, group=None):
    """All-gather of row blocks.  Rank r holds rows [bounds[r], bounds[r+1])
    of an array as ``local`` (a tensor [rows_r, ...]); every rank receives the
    whole array [bounds[-1], ...], blocks in rank order (MPI_Allgatherv's
    result, mpi_utils.h:69-79).  The collective moves equal-size buffers, so
    each block is padded to the largest block."""
    import torch
    import torch.distributed as dist
    rank, ws = _world(group)
    sizes = [bounds[r + 1] - bounds[r] for r in range(ws)]
    if local.shape[0] != sizes[rank]:
        raise ValueError("rank %d holds %d rows, its block has %d" % (rank, local.shape[0], sizes[rank]))
    if ws == 1:
        return local
    m = max(max(sizes), 1)
    rest = tuple(local.shape[1:])
    pad = torch.zeros((m,) + rest, dtype=local.dtype, device=local.device)
    pad[:sizes[rank]] = local
    parts = [torch.empty_like(pad) for _ in range(ws)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([parts[r][:sizes[r]] for r in range(ws)], dim=0)


class ShardedRing:
    """One rank's share of the s-grid ring of the loaded wave type 5 model.

    All ranks must load the same waveinput.dat and call ``force_update`` with
    the same times, as the reference requires of wave_force_update under MPI
    (it is collective).  Queries (wave_Kinematics_batch and friends) then read
    the complete ring on every rank."""

    def __init__(self, wm, group=None, device=None):
        import torch
        self.wm, self.lib, self.group = wm, wm.lib, group
        self.rank, self.size = _world(group)
        b = np.zeros(self.size + 1, dtype=np.int32)
        rc = self.lib.cfdwm_sgrid_partition(self.size, b.ctypes.data_as(C.POINTER(C.c_int)))
        if rc != 0:
            raise RuntimeError("cfdwm_sgrid_partition: %d" % rc)
        self.bounds = [int(v) for v in b]
        self.i0, self.i1 = self.bounds[self.rank], self.bounds[self.rank + 1]
        self.nx = self.bounds[-1]
        self.device = device or (torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available()
                                 else torch.device("cpu"))
        self.fields = []
        for f in range(5):
            n_all = self.lib.cfdwm_sgrid_block_count(f, 0, self.nx)
            if n_all < 0:
                break
            self.fields.append(n_all // max(self.nx, 1))     # elements per row
        self.steps = 0

    def step(self):
        """One ring update: this rank's rows, the exchange, the gradients."""
        import torch
        from . import _ptr
        rc = self.lib.cfdwm_sgrid_step_block(self.i0, self.i1)
        if rc != 0:
            raise RuntimeError("cfdwm_sgrid_step_block: %d" % rc)
        for f, per_row in enumerate(self.fields):
            mine = torch.empty((self.i1 - self.i0, per_row), dtype=torch.float32, device=self.device)
            if mine.numel():
                rc = self.lib.cfdwm_sgrid_block_export(f, self.i0, self.i1, _ptr(mine))
                if rc != 0:
                    raise RuntimeError("cfdwm_sgrid_block_export: %d" % rc)
            whole = allgather_rows(mine, self.bounds, self.group).contiguous()
            if whole.is_cuda:
                # the collective ran on torch's stream, the import runs on the library's
                torch.cuda.current_stream().synchronize()
            for r in range(self.size):
                a, b = self.bounds[r], self.bounds[r + 1]
                if r == self.rank or a == b:
                    continue
                rc = self.lib.cfdwm_sgrid_block_import(f, a, b, _ptr(whole[a:b]))
                if rc != 0:
                    raise RuntimeError("cfdwm_sgrid_block_import: %d" % rc)
        rc = self.lib.cfdwm_sgrid_step_finish()
        if rc != 0:
            raise RuntimeError("cfdwm_sgrid_step_finish: %d" % rc)
        self.steps += 1

    def force_update(self, t):
        """wave_force_update(t) over the ranks (CFDwavemaker.cpp:2253-2262)."""
        while self.lib.cfdwm_sgrid_due(float(t)):
            self.step()
