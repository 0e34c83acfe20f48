"""A mesh partitioned into parts: the multi-rank ot::DA of the reference.

The reference runs fem::matvec on every MPI rank over that rank's share of
the tree, on a ghosted node layout [pre-ghosts | owned | post-ghosts]
(include/oda.h:180-264), with the ghost read before the product and the ghost
accumulate after it (include/oda.tcc:210-435, readFromGhost* /
writeToGhosts*), built from send maps (SFC_NodeSort::computeScattermap,
include/nsort.tcc:809-872) and their receive side (scatter2gather,
include/nsort.tcc:1971-2010; ghostExchange / ghostReverse, :2013-2095).

Here, from a plan's flattened traversal (leaves in SFC order):
  * the parts are contiguous leaf ranges of equal length (the SFC partition);
  * every node touched by a part's leaves (own ranks, and the parent ranks of
    its hanging leaves) is in the part's ghosted layout; the node is owned by
    the lowest-numbered part that touches it, and is a pre-ghost of the
    parts after its owner, a post-ghost of none (owners come first);
  * send[q] lists, in global node order, the owned nodes of the part that are
    ghosts of part q (local indices in the sending part), recv[p] where those
    values land in part p's layout (local indices in the receiving part);
  * the part's plan (dkt_plan_create_part) is the part's leaves on its own
    node numbering.
Product: the ghost read copies each owned value into the ghost slots of the
other parts, every part multiplies locally, and the ghost accumulate adds
every ghost slot into its owner (and clears it).  The owned slots then hold
the global product.

Within one process the parts' vectors are device tensors exchanged with
index copies; across processes (one part per rank) `exchange_read` and
`exchange_accumulate` send the same slices with torch.distributed
point-to-point calls.  Plans that read stale slots of the reference's static
parent buffer are not partitioned: that buffer is one sequential chain over
the whole traversal (the reference's own ranks each keep their own chain, so
there the partitioned product differs from the one-rank product).
"""
import ctypes

import numpy as np


def partition_maps(e2n, hidx, p2n, n_nodes, nparts):
    """The partition of a flattened traversal (numpy arrays: e2n [n_leaf][npe],
    hidx [n_leaf], p2n [n_hang][npe]) into `nparts` contiguous leaf ranges.
    Returns a list of dicts, one per part: leaf_begin, leaf_end, nodes (global
    ids in local order: pre-ghosts, owned, post-ghosts), n_pre, n_owned,
    n_post, node_map (global -> local, -1 off the part), send {q: local
    indices sent to part q}, recv {q: local indices received from part q}."""
    e2n = np.asarray(e2n)
    hidx = np.asarray(hidx)
    p2n = np.asarray(p2n)
    n_leaf = e2n.shape[0]
    if not 1 <= nparts <= max(n_leaf, 1):
        raise ValueError("nparts must be in [1, number of leaves]")
    bounds = np.linspace(0, n_leaf, nparts + 1).round().astype(np.int64)
    touched = []
    for p in range(nparts):
        b0, b1 = bounds[p], bounds[p + 1]
        ids = e2n[b0:b1].ravel()
        h = hidx[b0:b1]
        h = h[h >= 0]
        if h.size:
            ids = np.concatenate([ids, p2n[h].ravel()])
        touched.append(np.unique(ids[ids >= 0]))
    owner = np.full(n_nodes, nparts, np.int64)
    for p in range(nparts):
        np.minimum.at(owner, touched[p], p)
    owner[owner == nparts] = 0            # a node no leaf touches: part 0 keeps it
    parts = []
    for p in range(nparts):
        owned = np.flatnonzero(owner == p)
        t = touched[p]
        ghosts = t[owner[t] != p]
        pre, post = ghosts[owner[ghosts] < p], ghosts[owner[ghosts] > p]
        nodes = np.concatenate([pre, owned, post])
        node_map = np.full(n_nodes, -1, np.int32)
        node_map[nodes] = np.arange(nodes.size, dtype=np.int32)
        parts.append(dict(leaf_begin=int(bounds[p]), leaf_end=int(bounds[p + 1]), nodes=nodes, n_pre=pre.size,
                          n_owned=owned.size, n_post=post.size, node_map=node_map, send={}, recv={},
                          owner_of_ghosts=owner[ghosts]))
    for p in range(nparts):
        ghosts = np.concatenate([parts[p]["nodes"][:parts[p]["n_pre"]],
                                 parts[p]["nodes"][parts[p]["n_pre"] + parts[p]["n_owned"]:]])
        gown = owner[ghosts]
        for q in np.unique(gown):
            g = np.sort(ghosts[gown == q])
            parts[q]["send"][p] = parts[q]["node_map"][g].astype(np.int64)
            parts[p]["recv"][q] = parts[p]["node_map"][g].astype(np.int64)
    return parts


def owned_slice(part):
    return slice(part["n_pre"], part["n_pre"] + part["n_owned"])


def read_from_ghosts(parts, local):
    """Ghost read within one process: every ghost slot of every part takes
    its owner's value (local: one vector per part, torch or numpy)."""
    for p, part in enumerate(parts):
        for q, idx in part["recv"].items():
            local[p][_ix(local[p], idx)] = local[q][_ix(local[q], parts[q]["send"][p])]


def write_to_ghosts_accumulate(parts, local):
    """Ghost accumulate within one process: every ghost slot is added into its
    owner's slot, then cleared."""
    for p, part in enumerate(parts):
        for q, idx in part["recv"].items():
            dst = _ix(local[q], parts[q]["send"][p])
            src = _ix(local[p], idx)
            if hasattr(local[q], "index_add_"):
                local[q].index_add_(0, dst, local[p][src])
            else:
                np.add.at(local[q], dst, local[p][src])
            local[p][src] = 0


def _ix(v, idx):
    if hasattr(v, "device"):
        import torch
        return torch.as_tensor(idx, device=v.device)
    return idx


def exchange_read(part, local, group=None):
    """Ghost read across processes (this process holds `part`): sends its
    owned values that other parts hold as ghosts and receives its own ghost
    values, with torch.distributed point-to-point calls."""
    import torch
    import torch.distributed as dist
    reqs, bufs = [], []
    for q, idx in sorted(part["send"].items()):
        t = local[torch.as_tensor(idx, device=local.device)].contiguous()
        bufs.append(t)
        reqs.append(dist.isend(t, q, group=group))
    recv = []
    for q, idx in sorted(part["recv"].items()):
        t = torch.empty(len(idx), dtype=local.dtype, device=local.device)
        recv.append((idx, t))
        reqs.append(dist.irecv(t, q, group=group))
    for r in reqs:
        r.wait()
    for idx, t in recv:
        local[torch.as_tensor(idx, device=local.device)] = t


def exchange_accumulate(part, local, group=None):
    """Ghost accumulate across processes: sends its ghost slots to their
    owners (and clears them), receives the contributions to its owned nodes
    from the parts that hold them as ghosts, and adds them."""
    import torch
    import torch.distributed as dist
    reqs, bufs = [], []
    for q, idx in sorted(part["recv"].items()):
        ix = torch.as_tensor(idx, device=local.device)
        t = local[ix].contiguous()
        bufs.append(t)
        local[ix] = 0
        reqs.append(dist.isend(t, q, group=group))
    got = []
    for q, idx in sorted(part["send"].items()):
        t = torch.empty(len(idx), dtype=local.dtype, device=local.device)
        got.append((idx, t))
        reqs.append(dist.irecv(t, q, group=group))
    for r in reqs:
        r.wait()
    for idx, t in got:
        local.index_add_(0, torch.as_tensor(idx, device=local.device), t)


class PartitionedMatrix:
    """A Matrix's mesh in `nparts` parts on this GPU, each with its own plan
    (dkt_plan_create_part), and the ghost exchange around their products."""

    def __init__(self, matrix, nparts):
        from . import load, _check, _p
        e2n, info, hidx, p2n, fill = matrix.export()
        self.parts = partition_maps(e2n, hidx, p2n, matrix.n, nparts)
        self.n = matrix.n
        self.matrix = matrix
        self.plans = []
        L = load()
        for part in self.parts:
            h = ctypes.c_void_p()
            nm = np.ascontiguousarray(part["node_map"])
            _check(L.dkt_plan_create_part(matrix._h, part["leaf_begin"], part["leaf_end"], _p(nm),
                                          part["nodes"].size, ctypes.byref(h)))
            self.plans.append(_PartPlan(h, part["nodes"].size))

    def matvec_raw(self, x_dev, y_dev):
        """fem::matvec of the whole mesh through the parts: distribute the
        owned values, ghost read, local products, ghost accumulate, gather
        the owned values (device tensors of the mesh's node count)."""
        import torch
        xs = []
        for part in self.parts:
            v = torch.zeros(part["nodes"].size, dtype=x_dev.dtype, device=x_dev.device)
            o = owned_slice(part)
            v[o] = x_dev[torch.as_tensor(part["nodes"][o], device=x_dev.device)]
            xs.append(v)
        read_from_ghosts(self.parts, xs)
        ys = []
        for part, plan, xp in zip(self.parts, self.plans, xs):
            yp = torch.empty_like(xp)
            plan.matvec_raw(xp, yp)
            ys.append(yp)
        write_to_ghosts_accumulate(self.parts, ys)
        for part, yp in zip(self.parts, ys):
            o = owned_slice(part)
            y_dev[torch.as_tensor(part["nodes"][o], device=y_dev.device)] = yp[o]

    def __del__(self):
        self.plans = []


class _PartPlan:
    def __init__(self, h, n):
        self._h = h
        self.n = n

    def matvec_raw(self, x_dev, y_dev):
        from . import load, _check, _p
        _check(load().dkt_matvec(self._h, _p(x_dev), _p(y_dev), 1.0, None))

    def __del__(self):
        try:
            from . import load
            if self._h:
                load().dkt_plan_destroy(self._h)
                self._h = None
        except Exception:
            pass
