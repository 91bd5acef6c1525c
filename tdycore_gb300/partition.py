"""Partition of an extruded mesh into layer slabs, with the halo exchange one
F+J evaluation needs.

The reference distributes cells with DMPlex (overlap 1, src/tdycore.c:687)
and owns each vertex on the lowest rank among the owners of its cells
(``is_local``, src/mesh/tdymeshplex.c:277-445); every rank then evaluates the
fluxes of the interaction regions around its owned cells from its local
(owned + ghost) cells after one ghost update of the pressure.

Here the cells of an extruded mesh (``cell = layer * ncol + column``, the
library's numbering) are split into contiguous layer slabs, one per rank.  A
rank's local mesh is its slab plus one ghost layer on each side that exists:
exactly the cells that share a vertex with an owned cell (the FVM++ overlap
of the Jacobian pattern), so every interaction region of a vertex of an
owned cell is complete locally and the owned rows of R and J are those of
the whole mesh.  Each evaluation needs one exchange: a rank sends its lowest
owned layer down and its highest owned layer up, and receives its ghost
layers.  Ghost rows are computed and discarded; vertices on the outer ghost
planes see a local boundary that touches ghost cells only.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class LocalSlab:
    rank: int
    nranks: int
    ncol: int
    k0: int                # first owned layer
    k1: int                # one past the last owned layer
    g0: int                # first local layer (k0 or k0 - 1)
    g1: int                # one past the last local layer (k1 or k1 + 1)
    cells: np.ndarray = field(repr=False)       # global id of each local cell, local order
    owned: np.ndarray = field(repr=False)       # local mask of owned cells
    owned_local: np.ndarray = field(repr=False)  # local indices of owned cells (ascending)
    # neighbour rank -> local indices sent to it / received from it
    send: dict = field(default_factory=dict, repr=False)
    recv: dict = field(default_factory=dict, repr=False)

    @property
    def nlocal(self) -> int:
        return self.cells.size

    @property
    def nowned(self) -> int:
        return self.owned_local.size

    def levels(self) -> slice:
        """Vertex levels (rows of the extruded mesh's z array) of the local mesh."""
        return slice(self.g0, self.g1 + 1)

    def local_from_global(self, U_global: np.ndarray) -> np.ndarray:
        return np.asarray(U_global)[self.cells]

    def exchange(self, U_local, comm) -> None:
        """Fill the ghost entries of ``U_local`` (1-D tensor or array of
        nlocal values) from the neighbours.  ``comm`` provides ``isend(t, dst)``
        / ``irecv(t, src)`` returning waitable requests, as torch.distributed
        does (gloo on CPU, NCCL on GPU)."""
        import torch

        t = U_local if isinstance(U_local, torch.Tensor) else torch.from_numpy(U_local)
        reqs, bufs = [], []
        for nb, idx in self.send.items():
            buf = t[torch.as_tensor(idx, device=t.device)].contiguous()
            bufs.append(buf)
            reqs.append(comm.isend(buf, dst=nb))
        recvd = []
        for nb, idx in self.recv.items():
            buf = torch.empty(len(idx), dtype=t.dtype, device=t.device)
            recvd.append((idx, buf))
            reqs.append(comm.irecv(buf, src=nb))
        for r in reqs:
            r.wait()
        for idx, buf in recvd:
            t[torch.as_tensor(idx, device=t.device)] = buf

    def global_rows(self, rowptr, colidx, vals):
        """Owned rows of a local CSR matrix with global column ids:
        (global row ids, rowptr, global colidx, vals); columns stay sorted
        because local numbering is monotone in global numbering."""
        rp = np.asarray(rowptr)
        rows = self.owned_local
        counts = rp[rows + 1] - rp[rows]
        out_rp = np.concatenate([[0], np.cumsum(counts)])
        sel = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in rows]) if rows.size else np.zeros(0, int)
        return self.cells[rows], out_rp, self.cells[np.asarray(colidx)[sel]], np.asarray(vals)[sel]


class SlabPartition:
    """Balanced contiguous layer ranges: rank r owns layers
    [r * nl // P + min(r, nl % P) ...) -- the first nl % P ranks get one more."""

    def __init__(self, ncol: int, nlayers: int, nranks: int):
        if nranks < 1 or nranks > nlayers:
            raise ValueError(f"{nranks} ranks for {nlayers} layers: every rank needs at least one layer")
        self.ncol, self.nlayers, self.nranks = ncol, nlayers, nranks
        base, extra = divmod(nlayers, nranks)
        self.starts = [r * base + min(r, extra) for r in range(nranks + 1)]

    def owner_of_layer(self, k: int) -> int:
        return int(np.searchsorted(self.starts, k, side="right") - 1)

    def owner_of_cell(self, cell: int) -> int:
        return self.owner_of_layer(cell // self.ncol)

    def owner_of_vertex_level(self, kv: int) -> int:
        """Lowest-owner rule: a vertex on level kv touches layers kv-1 and kv."""
        ks = [k for k in (kv - 1, kv) if 0 <= k < self.nlayers]
        return min(self.owner_of_layer(k) for k in ks)

    def local(self, rank: int) -> LocalSlab:
        k0, k1 = self.starts[rank], self.starts[rank + 1]
        g0, g1 = max(k0 - 1, 0), min(k1 + 1, self.nlayers)
        nc = self.ncol
        cells = np.arange(g0 * nc, g1 * nc)
        owned = (cells >= k0 * nc) & (cells < k1 * nc)
        s = LocalSlab(rank, self.nranks, nc, k0, k1, g0, g1, cells, owned, np.nonzero(owned)[0])
        lay = lambda k: np.arange((k - g0) * nc, (k - g0 + 1) * nc)  # noqa: E731  local indices of layer k
        if g0 < k0:  # ghost layer below, owned by rank - 1
            s.recv[rank - 1] = lay(k0 - 1)
            s.send[rank - 1] = lay(k0)
        if g1 > k1:  # ghost layer above, owned by rank + 1
            s.recv[rank + 1] = lay(k1)
            s.send[rank + 1] = lay(k1 - 1)
        return s
