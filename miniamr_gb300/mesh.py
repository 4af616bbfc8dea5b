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
        slot_of = {int(self.number[s]): int(s) for s in order}
        out = np.zeros(len(order), dtype=BLOCK_DTYPE)
        for q, s in enumerate(order):
            x, y, z, _ = self.lattice(int(s))
            out["slot"][q] = s
            out["level"][q] = lev
            for l, (dx, dy, dz) in enumerate(((-1, 0, 0), (1, 0, 0),
                                              (0, -1, 0), (0, 1, 0),
                                              (0, 0, -1), (0, 0, 1))):
                xx, yy, zz = x + dx, y + dy, z + dz
                if 0 <= xx < nx and 0 <= yy < ny and 0 <= zz < nz:
                    out["nei_level"][q, l] = lev
                    out["nei"][q, l, 0, 0] = slot_of[start + (zz * ny + yy)
                                                     * nx + xx]
                else:
                    out["nei_level"][q, l] = -2
                    out["nei"][q, l, 0, 0] = 0
        return out

    def split_all(self) -> np.ndarray:
        """Refines every active block once (one uniform-refine pass) and
        returns the split jobs in the reference's order."""
        jobs = []
        m = 0
        cur_max = int(self.level[self.number >= 0].max())
        max_active = int(np.nonzero(self.number >= 0)[0].max()) + 1
        for lev in range(cur_max + 1):
            n = 0
            while n < max_active:
                if self.number[n] >= 0 and self.level[n] == lev:
                    x, y, z, _ = self.lattice(n)
                    cnx, cny, _ = self.dims(lev + 1)
                    cstart = self.block_start(lev + 1)
                    child = [0] * 8
                    for o in range(8):
                        while m < self.max_blocks and self.number[m] >= 0:
                            m += 1
                        if m == self.max_blocks:
                            raise RuntimeError("No inactive blocks available")
                        max_active = max(max_active, m + 1)
                        i1, j1, k1 = o % 2, (o // 2) % 2, o // 4
                        self.number[m] = ((2 * z + k1) * cny + (2 * y + j1)) \
                            * cnx + 2 * x + i1 + cstart
                        self.level[m] = lev + 1
                        child[o] = m
                    jobs.append((n, child))
                    self.number[n] = -1
                    if n < m:
                        m = n
                n += 1
        out = np.zeros(len(jobs), dtype=SPLIT_DTYPE)
        for q, (p, ch) in enumerate(jobs):
            out["parent"][q] = p
            out["child"][q] = ch
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
