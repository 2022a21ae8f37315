"""Element-partitioned assembly across ranks (one process per GPU).

The reference's only parallel assembly is oomph-lib's MPI split of the
element loop into contiguous ranges (``First_el_for_assembly`` /
``Last_el_plus_one_for_assembly``, ``problem.cc:5354-5358``) followed by a
redistribution of the assembled rows (``parallel_sparse_assemble``,
``problem.cc:4131-4155``).  Here:

* ranks own contiguous element ranges (balanced by element count) and
  contiguous row ranges (balanced by non-zeros);
* each rank assembles its elements on its own GPU into a local CSR (the
  engine on the rank's element subset) and maps local slots to the global
  pattern, which every rank builds identically on the host
  (``fe_pattern_host``);
* one exchange completes the assembly: the *halo* slots -- slots of a row
  that a rank other than the row's owner touches -- go to their row's owner
  only (one all-to-all: every rank sends owner k its values of k's halo),
  and each owner sums what it receives in rank order, so the result is
  deterministic.  Everything else is touched by its owner alone and is
  already final.

The plan (slot maps, halo lists) is built once per mesh; the exchange moves
only halo values.  Works with any torch.distributed backend (gloo on CPU
tensors for the tests, NCCL on device tensors).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Tuple

import numpy as np


def element_ranges(n_elem: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous element ranges, sizes differing by at most one."""
    q, r = divmod(n_elem, world)
    out, lo = [], 0
    for k in range(world):
        hi = lo + q + (1 if k < r else 0)
        out.append((lo, hi))
        lo = hi
    return out


def row_ranges(rowptr: np.ndarray, world: int) -> List[Tuple[int, int]]:
    """Contiguous row ranges with balanced non-zero counts."""
    n = rowptr.shape[0] - 1
    nnz = int(rowptr[-1])
    cuts = [0]
    for k in range(1, world):
        cuts.append(int(np.searchsorted(rowptr, nnz * k / world)))
    cuts.append(n)
    cuts = np.maximum.accumulate(np.array(cuts))
    return [(int(cuts[k]), int(cuts[k + 1])) for k in range(world)]


def _slot_keys(rowptr: np.ndarray, colidx: np.ndarray, n_dof: int) -> np.ndarray:
    rows = np.repeat(np.arange(rowptr.shape[0] - 1, dtype=np.int64), np.diff(rowptr))
    return rows * n_dof + colidx.astype(np.int64)


@dataclass
class ShardPlan:
    rank: int
    world: int
    n_dof: int
    nnz: int
    rows: Tuple[int, int]            # owned rows [lo, hi)
    local_to_global: np.ndarray      # [local nnz] global slot of each local slot
    local_rows: np.ndarray           # [local n_dof] touched rows (global numbers)
    halo_slots: np.ndarray           # global slots exchanged (all owners), sorted
    halo_rows: np.ndarray            # global rows whose residual is exchanged, sorted
    halo_slot_ptr: np.ndarray = None  # [world + 1] owner k's halo slots: halo_slots[ptr[k]:ptr[k+1]]
    halo_row_ptr: np.ndarray = None   # [world + 1] the same for the halo rows


def make_plan(rank: int, world: int, rowptr: np.ndarray, colidx: np.ndarray,
              local_rowptr: np.ndarray, local_colidx: np.ndarray, group=None) -> ShardPlan:
    """Slot map of this rank's local pattern into the global one, and the
    halo lists (setup collective: one all_gather_object of touched slots)."""
    import torch.distributed as dist
    n_dof = rowptr.shape[0] - 1
    gkeys = _slot_keys(rowptr, colidx, n_dof)
    order = np.argsort(gkeys, kind="stable")
    lkeys = _slot_keys(local_rowptr, local_colidx, n_dof)
    pos = np.searchsorted(gkeys[order], lkeys)
    if np.any(pos >= gkeys.size) or np.any(gkeys[order][np.minimum(pos, gkeys.size - 1)] != lkeys):
        raise RuntimeError("local pattern is not contained in the global pattern")
    l2g = order[pos].astype(np.int64)
    touched_rows = np.nonzero(np.diff(local_rowptr) > 0)[0].astype(np.int64)
    mine = (np.sort(l2g), touched_rows)
    allv = [None] * world
    dist.all_gather_object(allv, mine, group=group)
    # a slot/row is exchanged if a rank other than its owner touches it
    rr = row_ranges(rowptr, world)
    row_owner = np.zeros(n_dof, dtype=np.int32)
    for k, (a, b) in enumerate(rr):
        row_owner[a:b] = k
    slot_owner = np.repeat(row_owner, np.diff(rowptr))
    foreign_s = np.zeros(int(rowptr[-1]), dtype=bool)
    foreign_r = np.zeros(n_dof, dtype=bool)
    for k, (s, r) in enumerate(allv):
        foreign_s[s[slot_owner[s] != k]] = True
        foreign_r[r[row_owner[r] != k]] = True
    hs = np.nonzero(foreign_s)[0].astype(np.int64)
    hr = np.nonzero(foreign_r)[0].astype(np.int64)
    # owners' row ranges are contiguous and ascending: each owner's halo is a run
    sp = np.searchsorted(hs, [int(rowptr[a]) for a, _ in rr] + [int(rowptr[-1])])
    rp_ = np.searchsorted(hr, [a for a, _ in rr] + [n_dof])
    return ShardPlan(rank, world, n_dof, int(rowptr[-1]), rr[rank], l2g, touched_rows, hs, hr,
                     sp.astype(np.int64), rp_.astype(np.int64))


def reduce_owned(plan: ShardPlan, local_vals, local_R_global, group=None):
    """Complete the assembly: returns (values of the global CSR slots, with
    the owned rows final; residual, owned rows final).  local_vals: this
    rank's values on its local pattern; local_R_global: this rank's partial
    residual as a full-length vector (zeros where untouched).  One
    all-to-all: owner k receives from every rank that rank's values of k's
    halo slots and rows (zeros where it touches none) and sums them in rank
    order.  Tensors may live on CPU (gloo) or GPU (NCCL); the result stays
    on the same device."""
    import torch
    import torch.distributed as dist
    dev = local_vals.device
    full = torch.zeros(plan.nnz, dtype=local_vals.dtype, device=dev)
    full[torch.as_tensor(plan.local_to_global, device=dev)] = local_vals
    hs = torch.as_tensor(plan.halo_slots, device=dev)
    hr = torch.as_tensor(plan.halo_rows, device=dev)
    R = local_R_global.clone()
    sends, sizes = [], []
    for k in range(plan.world):
        s_k = hs[int(plan.halo_slot_ptr[k]):int(plan.halo_slot_ptr[k + 1])]
        r_k = hr[int(plan.halo_row_ptr[k]):int(plan.halo_row_ptr[k + 1])]
        sends.append(torch.cat([full[s_k], R[r_k].to(full.dtype)]))
        sizes.append(int(s_k.numel() + r_k.numel()))
    me = plan.rank
    mine = sizes[me]
    inp = torch.cat(sends) if sends else torch.zeros(0, dtype=full.dtype, device=dev)
    out = torch.empty(mine * plan.world, dtype=full.dtype, device=dev)
    dist.all_to_all_single(out, inp, output_split_sizes=[mine] * plan.world, input_split_sizes=sizes,
                           group=group)
    if mine:
        parts = out.view(plan.world, mine)
        acc = parts[0].clone()
        for k in range(1, plan.world):
            acc += parts[k]              # rank order: deterministic
        ns = int(plan.halo_slot_ptr[me + 1] - plan.halo_slot_ptr[me])
        full[hs[int(plan.halo_slot_ptr[me]):int(plan.halo_slot_ptr[me + 1])]] = acc[:ns]
        R[hr[int(plan.halo_row_ptr[me]):int(plan.halo_row_ptr[me + 1])]] = acc[ns:].to(R.dtype)
    return full, R


def owned_view(plan: ShardPlan, rowptr: np.ndarray, full_vals, R):
    lo, hi = plan.rows
    return full_vals[int(rowptr[lo]):int(rowptr[hi])], R[lo:hi]
