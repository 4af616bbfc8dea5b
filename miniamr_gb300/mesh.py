"""Host-side mesh bookkeeping for uniform meshes on one rank.

This is the metadata the reference's host code keeps in ``blocks[]`` and
``sorted_list`` for the two cases the benchmarks and tests build without the
reference's driver: the initial lattice of ``init()`` and uniform refinement
(``refine(0)`` with ``--uniform_refine 1``).  Numbering, slot assignment and
sorted order follow the reference:

* initial blocks: one rank, ``lb_method`` 0 -- slot ``o`` == block number
  ``n``, lattice order x fastest (ref/init.c:453-495); neighbours are the
  lattice neighbours, ``nei_level`` -2 on the domain boundary
  (ref/init.c:500-560);
* split: levels ascending, parents in slot order, each child in the first
  free slot at or after a running index, a freed parent slot reusable by
  later children (ref/block.c:60-173, 305-307); child number from the
  parent's lattice position (ref/block.c:66-70, 143-146);
* sorted list: level ascending, block number descending (ref/block.c:
  610-625).

Neighbour tables of a uniform mesh are the lattice neighbours at the single
level, so they are recomputed from block numbers after each split.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .abi import BLOCK_DTYPE, SPLIT_DTYPE


@dataclass
class UniformMesh:
    init_x: int
    init_y: int
    init_z: int
    num_refine: int
    max_blocks: int
    # per slot; number < 0 means the slot is free
    number: np.ndarray = field(default=None)
    level: np.ndarray = field(default=None)

    @property
    def n0(self) -> int:
        return self.init_x * self.init_y * self.init_z

    def block_start(self, level: int) -> int:
        # ref/init.c:60-66 with one rank
        start, num = 0, self.n0
        for _ in range(level):
            start += num
            num *= 8
        return start

    def dims(self, level: int):
        p = 2 ** level
        return self.init_x * p, self.init_y * p, self.init_z * p

    def active_slots(self) -> np.ndarray:
        return np.nonzero(self.number >= 0)[0].astype(np.int32)

    def sorted_slots(self) -> np.ndarray:
        """Slots in sorted_list order: level ascending, number descending."""
        s = self.active_slots()
        key = np.lexsort((-self.number[s], self.level[s]))
        return s[key].astype(np.int32)

    def lattice(self, slot: int):
        lev = int(self.level[slot])
        nx, ny, _ = self.dims(lev)
        nl = int(self.number[slot]) - self.block_start(lev)
        return nl % nx, (nl // nx) % ny, nl // (nx * ny), lev

    def blocks(self) -> np.ndarray:
        """The active mesh as mamr_block records in sorted_list order.

        All active blocks must be at one level (a uniform mesh)."""
        order = self.sorted_slots()
        levels = np.unique(self.level[order])
        if len(levels) != 1:
            raise ValueError("UniformMesh.blocks needs a single-level mesh")
        lev = int(levels[0])
        nx, ny, nz = self.dims(lev)
        start = self.block_start(lev)
        nl = self.number[order] - start
        x, y, z = nl % nx, (nl // nx) % ny, nl // (nx * ny)
        # the slot holding each lattice position of the level
        slot_at = np.full(nx * ny * nz, -1, dtype=np.int64)
        slot_at[nl] = order
        out = np.zeros(len(order), dtype=BLOCK_DTYPE)
        out["slot"] = order
        out["level"] = lev
        for l, (dx, dy, dz) in enumerate(((-1, 0, 0), (1, 0, 0), (0, -1, 0),
                                          (0, 1, 0), (0, 0, -1), (0, 0, 1))):
            xx, yy, zz = x + dx, y + dy, z + dz
            inside = ((xx >= 0) & (xx < nx) & (yy >= 0) & (yy < ny) &
                      (zz >= 0) & (zz < nz))
            pos = np.where(inside, (zz * ny + yy) * nx + xx, 0)
            out["nei_level"][:, l] = np.where(inside, lev, -2)
            out["nei"][:, l, 0, 0] = np.where(inside, slot_at[pos], 0)
        return out

    def split_all(self) -> np.ndarray:
        """Refines every active block once (one uniform-refine pass) and
        returns the split jobs in the reference's order.  Free slots are
        kept negated in an ascending list -- the lowest slots last, where
        the running index takes them and freed parents return -- so "the
        first free slot at or after the running index" is one bisection and
        taking or returning a slot moves few list entries."""
        fast = self._split_fresh_lattice()
        if fast is not None:
            return fast
        import bisect
        number = self.number.tolist()
        level = self.level.tolist()
        neg = [-q for q in range(self.max_blocks - 1, -1, -1)
               if number[q] < 0]
        jobs = []
        m = 0
        active = [q for q in range(self.max_blocks) if number[q] >= 0]
        cur_max = max(level[q] for q in active)
        max_active = active[-1] + 1
        for lev in range(cur_max + 1):
            cnx, cny, _ = self.dims(lev + 1)
            cstart = self.block_start(lev + 1)
            nx, ny, _ = self.dims(lev)
            start = self.block_start(lev)
            n = 0
            while n < max_active:
                if number[n] >= 0 and level[n] == lev:
                    nl = number[n] - start
                    x, y, z = nl % nx, (nl // nx) % ny, nl // (nx * ny)
                    child = [0] * 8
                    for o in range(8):
                        i = bisect.bisect_right(neg, -m) - 1
                        if i < 0:
                            raise RuntimeError("No inactive blocks available")
                        m = -neg.pop(i)
                        max_active = max(max_active, m + 1)
                        i1, j1, k1 = o % 2, (o // 2) % 2, o // 4
                        number[m] = ((2 * z + k1) * cny + (2 * y + j1)) \
                            * cnx + 2 * x + i1 + cstart
                        level[m] = lev + 1
                        child[o] = m
                    jobs.append((n, child))
                    number[n] = -1
                    bisect.insort(neg, -n)
                    if n < m:
                        m = n
                n += 1
        self.number[:] = number
        self.level[:] = level
        out = np.zeros(len(jobs), dtype=SPLIT_DTYPE)
        for q, (p, ch) in enumerate(jobs):
            out["parent"][q] = p
            out["child"][q] = ch
        return out


    def _split_fresh_lattice(self):
        """split_all when the active blocks are one level filling slots
        0 .. A-1 and every later slot is free (the initial lattice): the
        reference's slot walk then has a closed form -- job 0's children
        take A .. A+7; job t >= 1's take the slot job t-1 freed, then the
        next seven of A+8 ... -- computed without the walk; None otherwise."""
        act = np.nonzero(self.number >= 0)[0]
        a = len(act)
        if a == 0 or act[-1] != a - 1:
            return None
        lev = int(self.level[0])
        if not (self.level[:a] == lev).all() or self.max_blocks < 8 * a + 1:
            return None
        nx, ny, _ = self.dims(lev)
        cnx, cny, _ = self.dims(lev + 1)
        start, cstart = self.block_start(lev), self.block_start(lev + 1)
        t = np.arange(a, dtype=np.int64)
        child = np.empty((a, 8), dtype=np.int64)
        child[0] = a + np.arange(8)
        if a > 1:
            child[1:, 0] = t[1:] - 1
            child[1:, 1:] = (a + 8 + 7 * (t[1:, None] - 1) +
                             np.arange(7)[None, :])
        nl = self.number[:a] - start
        x, y, z = nl % nx, (nl // nx) % ny, nl // (nx * ny)
        o = np.arange(8)
        i1, j1, k1 = o % 2, (o // 2) % 2, o // 4
        cnum = (((2 * z[:, None] + k1) * cny + (2 * y[:, None] + j1)) * cnx +
                2 * x[:, None] + i1 + cstart)
        self.number[:a] = -1
        self.number[child.ravel()] = cnum.ravel()
        self.level[child.ravel()] = lev + 1
        out = np.zeros(a, dtype=SPLIT_DTYPE)
        out["parent"] = t
        out["child"] = child
        return out


def initial_mesh(init_x: int, init_y: int, init_z: int, num_refine: int,
                 max_blocks: int) -> UniformMesh:
    """The initial lattice of init() on one rank: slot == number, level 0."""
    m = UniformMesh(init_x, init_y, init_z, num_refine, max_blocks)
    n0 = m.n0
    if n0 > max_blocks:
        raise ValueError("max_blocks smaller than the initial lattice")
    m.number = np.full(max_blocks, -1, dtype=np.int64)
    m.level = np.zeros(max_blocks, dtype=np.int32)
    m.number[:n0] = np.arange(n0)
    return m
