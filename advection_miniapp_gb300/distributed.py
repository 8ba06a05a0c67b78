"""Slab-partitioned operator: one mesh over several ranks (one rank per GPU).

The reference distributes cells with parallel::distributed::Triangulation
and, inside MatrixFree::loop, imports the face values of the neighbouring
ranks' cells before the face integrals (DataAccessOnFaces::values,
advection_solver.cc:678-679; values and gradients for SIPG,
advection_diffusion_solver.cc:436-437).  Here the structured mesh is cut into
contiguous slabs of z layers.  Each rank holds an adv_create_slab handle whose
local vectors carry one ghost cell layer below and above its owned layers
(wherever a neighbouring slab exists; always on periodic meshes).  Before
every operator evaluation the ghost layers of the source vector are filled:
each slab sends the face layer of its first owned layer down and of its last
owned layer up (n^2 nodal values per cell; whole cells with diffusion, whose
penalty terms need normal derivatives).  Diagnostics are summed over the
ranks, the time step is the minimum over the ranks.

`DistributedAdvectionOperation` is one rank's operator over torch.distributed
point-to-point messages (NCCL for CUDA tensors, gloo for CPU tensors).
`SlabGroup` runs all slabs of a partition in one process on one GPU, with the
exchange done as device copies.  The kernels never wait on one another: every
exchange completes on the host side before the next launch.
"""
import ctypes

import numpy as np

from . import AdvectionOperation, _lib, make_config


def slab_ranges(n_layers, n_slabs):
    """Contiguous, balanced z-layer ranges [z_begin, z_end) of n_slabs slabs."""
    if n_slabs < 1 or n_slabs > n_layers:
        raise ValueError(f"cannot cut {n_layers} z layers into {n_slabs} slabs")
    base, extra = divmod(n_layers, n_slabs)
    out, z = [], 0
    for r in range(n_slabs):
        cnt = base + (1 if r < extra else 0)
        out.append((z, z + cnt))
        z += cnt
    return out


class SlabLayout:
    """Local vector layout of a slab (adv_slab_layout; no GPU needed)."""

    def __init__(self, config, z_begin, z_end):
        out = (ctypes.c_int64 * 10)()
        _lib.check(_lib.load().adv_slab_layout(ctypes.byref(config), int(z_begin), int(z_end), out),
                   "adv_slab_layout")
        (self.n_dofs, self.owned_begin, self.owned_dofs, self.layer_cells, self.dofs_per_cell, ghost_lo, ghost_hi,
         self.halo_values, self.layers, self.zoff) = list(out)
        self.ghost_lo, self.ghost_hi = bool(ghost_lo), bool(ghost_hi)
        self.z_begin, self.z_end = int(z_begin), int(z_end)
        self.n = config.degree + 1
        self.global_layers = config.n_cells[2]
        self.periodic = bool(config.periodic)
        self.first_owned_layer = 1 if self.ghost_lo else 0
        self.last_owned_layer = self.first_owned_layer + (self.z_end - self.z_begin) - 1

    @property
    def full_cells(self):
        return self.halo_values == self.dofs_per_cell

    def halo_views(self, vec):
        """(send_down, send_up, ghost_below, ghost_above): views into vec of
        the face layers this slab sends to the slab below / above and of the
        ghost layers it receives (None where there is no ghost layer)."""
        n = self.n
        v = vec.view(self.layers, self.layer_cells, n, n * n)
        f, l = self.first_owned_layer, self.last_owned_layer
        if self.full_cells:
            send_down, send_up = v[f], v[l]
            below = v[0] if self.ghost_lo else None
            above = v[self.layers - 1] if self.ghost_hi else None
        else:
            # nodal values on the shared face: z index 0 of the upper cell,
            # z index n - 1 of the lower cell
            send_down, send_up = v[f, :, 0, :], v[l, :, n - 1, :]
            below = v[0, :, n - 1, :] if self.ghost_lo else None
            above = v[self.layers - 1, :, 0, :] if self.ghost_hi else None
        return send_down, send_up, below, above

    def owned(self, vec):
        return vec[self.owned_begin:self.owned_begin + self.owned_dofs]

    def from_global(self, global_vec, out=None):
        """Local vector (owned and ghost layers) cut out of a global vector."""
        import torch
        per_layer = self.layer_cells * self.dofs_per_cell
        g = global_vec.view(self.global_layers, per_layer)
        idx = [(self.zoff + i) % self.global_layers for i in range(self.layers)]
        loc = g[torch.tensor(idx, device=global_vec.device)].reshape(-1)
        if out is None:
            return loc.clone()
        out.copy_(loc)
        return out


def _neighbours(rank, world_size, periodic):
    below = rank - 1 if rank > 0 else (world_size - 1 if periodic else None)
    above = rank + 1 if rank < world_size - 1 else (0 if periodic else None)
    return below, above


class TorchExchange:
    """Ghost-layer exchange of one rank with torch.distributed point-to-point
    messages, in two phases (upward, then downward) so that every pair of
    ranks matches its messages in order, also with two slabs on a periodic
    mesh where the rank below is the rank above."""

    def __init__(self, rank, world_size, periodic, group=None):
        self.rank, self.world_size, self.periodic, self.group = rank, world_size, periodic, group
        self.below, self.above = _neighbours(rank, world_size, periodic)

    def _phase(self, send, send_to, recv_view, recv_from, tag):
        import torch
        import torch.distributed as dist
        ops, buf = [], None
        if send_to is not None:
            ops.append(dist.P2POp(dist.isend, send.contiguous(), send_to, self.group, tag))
        if recv_from is not None:
            buf = torch.empty(recv_view.shape, dtype=recv_view.dtype, device=recv_view.device)
            ops.append(dist.P2POp(dist.irecv, buf, recv_from, self.group, tag))
        if ops:
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        if buf is not None:
            recv_view.copy_(buf)

    def update_ghost_values(self, layout, vec):
        send_down, send_up, below, above = layout.halo_views(vec)
        if self.world_size == 1:
            if self.periodic:
                below.copy_(send_up)
                above.copy_(send_down)
            return
        self._phase(send_up, self.above, below, self.below, 1)
        self._phase(send_down, self.below, above, self.above, 2)

    def all_reduce(self, values, op="sum"):
        """Sum (or minimum) of float64 values over the ranks, on the device
        the group's backend communicates from."""
        import torch
        import torch.distributed as dist
        t = torch.as_tensor(np.asarray(values, dtype=np.float64))
        if self.world_size > 1:
            if dist.get_backend(self.group) == "nccl":
                t = t.cuda()
            dist.all_reduce(t, op=dist.ReduceOp.SUM if op == "sum" else dist.ReduceOp.MIN, group=self.group)
        return t.cpu().numpy()


class DistributedAdvectionOperation:
    """One rank's share of the operator: the reference's AdvectionOperation
    interface (apply, perform_stage, project_initial, compute_mass_and_energy,
    l2_error, time_step, vmult) on the rank's slab, with the ghost exchange
    before each operator evaluation and reductions across ranks.  Runs with
    LowStorageRungeKuttaIntegrator.perform_time_step like the reference's
    operator (advection_solver.cc:906-939)."""

    def __init__(self, config=None, rank=None, world_size=None, group=None, exchange=None, **kw):
        import torch.distributed as dist
        self.config = config if config is not None else make_config(**kw)
        if rank is None:
            rank, world_size = dist.get_rank(group), dist.get_world_size(group)
        self.rank, self.world_size = rank, world_size
        self.ranges = slab_ranges(self.config.n_cells[2], world_size)
        zb, ze = self.ranges[rank]
        self.layout = SlabLayout(self.config, zb, ze)
        self.op = AdvectionOperation(self.config, slab=(zb, ze))
        self.exchange = exchange or TorchExchange(rank, world_size, bool(self.config.periodic), group)
        self.n_dofs = self.op.n_dofs
        self.degree = self.config.degree

    def close(self):
        self.op.close()

    def initialize_dof_vector(self):
        return self.op.initialize_dof_vector()

    def update_ghost_values(self, vec):
        self.exchange.update_ghost_values(self.layout, vec)

    def apply(self, src, dst, current_time, stream=None):
        self.update_ghost_values(src)
        self.op.apply(src, dst, current_time, stream)

    def perform_stage(self, current_time, factor_solution, factor_ai, current_ri, vec_ki, solution, next_ri,
                      stream=None):
        self.update_ghost_values(current_ri)
        self.op.perform_stage(current_time, factor_solution, factor_ai, current_ri, vec_ki, solution, next_ri,
                              stream)

    def vmult(self, src, dst, mass_factor, time=0.0, stream=None):
        self.update_ghost_values(src)
        self.op.vmult(src, dst, mass_factor, time, stream)

    def project_initial(self, dst, time=0.0, stream=None):
        self.op.project_initial(dst, time, stream)

    def compute_mass_and_energy(self, vec, stream=None):
        return self.exchange.all_reduce(self.op.compute_mass_and_energy(vec, stream))

    def l2_error(self, vec, time, stream=None):
        e, nrm = self.op.l2_error(vec, time, stream)
        s = self.exchange.all_reduce([e * e, nrm * nrm])
        return float(np.sqrt(s[0])), float(np.sqrt(s[1]))

    def time_step(self, courant=0.5):
        return float(self.exchange.all_reduce([self.op.time_step(courant)], op="min")[0])


class SlabGroup:
    """All slabs of a partition in one process (one GPU): the operator calls
    take and return lists of local vectors, one per slab, and the ghost
    exchange is a set of device copies.  Usable with
    LowStorageRungeKuttaIntegrator.perform_time_step."""

    def __init__(self, config, n_slabs):
        self.config = config
        self.ranges = slab_ranges(config.n_cells[2], n_slabs)
        self.layouts = [SlabLayout(config, zb, ze) for zb, ze in self.ranges]
        self.ops = [AdvectionOperation(config, slab=r) for r in self.ranges]
        self.periodic = bool(config.periodic)

    def close(self):
        for op in self.ops:
            op.close()

    def initialize_dof_vector(self):
        return [op.initialize_dof_vector() for op in self.ops]

    def update_ghost_values(self, vecs):
        views = [lay.halo_views(v) for lay, v in zip(self.layouts, vecs)]
        ns = len(vecs)
        for r in range(ns):
            below, above = _neighbours(r, ns, self.periodic)
            if below is not None:
                views[r][2].copy_(views[below][1])
            if above is not None:
                views[r][3].copy_(views[above][0])

    def apply(self, src, dst, current_time):
        self.update_ghost_values(src)
        for op, s, d in zip(self.ops, src, dst):
            op.apply(s, d, current_time)

    def perform_stage(self, current_time, factor_solution, factor_ai, current_ri, vec_ki, solution, next_ri,
                      stream=None):
        self.update_ghost_values(current_ri)
        for i, op in enumerate(self.ops):
            op.perform_stage(current_time, factor_solution, factor_ai, current_ri[i], vec_ki[i], solution[i],
                             next_ri[i] if next_ri is not None else None, stream)

    def project_initial(self, dst, time=0.0):
        for op, d in zip(self.ops, dst):
            op.project_initial(d, time)

    def l2_error(self, vecs, time):
        e2 = n2 = 0.0
        for op, v in zip(self.ops, vecs):
            e, nrm = op.l2_error(v, time)
            e2, n2 = e2 + e * e, n2 + nrm * nrm
        return float(np.sqrt(e2)), float(np.sqrt(n2))

    def compute_mass_and_energy(self, vecs):
        return sum(op.compute_mass_and_energy(v) for op, v in zip(self.ops, vecs))

    def time_step(self, courant=0.5):
        return min(op.time_step(courant) for op in self.ops)

    def to_global(self, vecs):
        """Owned parts of the local vectors, concatenated in z order."""
        import torch
        return torch.cat([lay.owned(v) for lay, v in zip(self.layouts, vecs)])
