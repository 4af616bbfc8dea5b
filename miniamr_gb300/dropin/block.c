/*
 * Drop-in replacement for the reference's block.c on one rank.
 *
 * split_blocks() and consolidate_blocks() (ref/proto.h:34-35, called from
 * ref/refine.c:112,128) keep the reference's bookkeeping exactly -- slot
 * allocation (first free slot from a running index in split, from 0 in
 * consolidate), parent records, block numbers, num_prime, centres, the
 * sorted list and the neighbour tables -- and hand the cell data movement
 * to the device as one ordered job list per call (mamr_split /
 * mamr_consolidate).  add_sorted_list, del_sorted_list and find_sorted_list
 * (ref/block.c:610-657) keep their semantics: level ascending, block number
 * descending within a level.
 *
 * One rank only: every neighbour is on this rank (nei >= 0), so the
 * reference's off-rank branches (comm lists, par lists) never apply; if one
 * is ever reached the run stops with an error instead.
 */
#include <stdio.h>
#include <stdlib.h>
#include <mpi.h>

#include "block.h"
#include "comm.h"
#include "timer.h"
#include "proto.h"
#include "hilbert.h"
#include "dropin.h"

/* Octant (i1 + 2*j1 + 4*k1) of the child that touches face c (W,E,S,N,D,U)
 * at tangential position (a, b), the indices of nei[c][a][b].  For x faces
 * a runs along z and b along y; for y faces a along z, b along x; for z
 * faces a along y, b along x (the quarter offsets of
 * ref/comm.c:1613-1614,1645-1646,1674-1675). */
static int face_child(int c, int a, int b)
{
   int hi = c % 2, i1, j1, k1;
   switch (c / 2) {
   case 0: i1 = hi; j1 = b; k1 = a; break;
   case 1: j1 = hi; i1 = b; k1 = a; break;
   default: k1 = hi; i1 = b; j1 = a; break;
   }
   return i1 + 2*j1 + 4*k1;
}

/* Octant bit that flips across the faces of direction c/2. */
static int dir_bit(int c)
{
   return 1 << (c / 2);
}

static void one_rank_only(const char *what, long long number, int c)
{
   printf("ERROR: %s (block %lld face %d): off-rank neighbour on a "
          "single-rank run\n", what, number, c);
   exit(-1);
}

static mamr_split_job *split_jobs;
static mamr_consolidate_job *cons_jobs;
static int cap_split, cap_cons;

void split_blocks(void)
{
   int n, m, o, o1, c, a, b, p, level, i1, j1, k1, sib[8], n_jobs = 0;
   num_sz nl, xp, yp, zp;
   block *bp, *bp1;
   parent *pp;

   mamr_dropin_sync_data();
   for (m = level = 0; level <= cur_max_level; level++) {
      /* slot order, not the sorted list: this routine edits the list */
      for (n = 0; n < max_active_block; n++) {
         bp = &blocks[n];
         if (bp->number < 0 || bp->level != level)
            continue;
         if (bp->refine != 1) {
            for (c = 0; c < 6; c++)
               if (bp->nei[c][0][0] < 0 && bp->nei_refine[c] == 1)
                  one_rank_only("split_blocks", (long long) bp->number, c);
            continue;
         }
         /* lattice position of this block at its level */
         nl = bp->number - block_start[level];
         zp = nl/((p2[level]*init_x)*(p2[level]*init_y));
         yp = (nl%((p2[level]*init_x)*(p2[level]*init_y)))/(p2[level]*init_x);
         xp = nl%(p2[level]*init_x);
         if ((num_active + 8) > max_num_blocks) {
            printf("ERROR: Need more blocks %d %d on %d\n",
                   num_active, max_num_blocks, my_pe);
            exit(-1);
         }
         if ((num_active + 8) > local_max_b)
            local_max_b = num_active + 8;
         del_sorted_list(bp->number, level, 1);
         num_active += 7;
         local_num_blocks[level]--;
         local_num_blocks[level+1] += 8;

         /* parent record: first unused entry */
         for (p = 0; p < max_active_parent; p++)
            if (parents[p].number < 0)
               break;
         if (p == max_num_parents) {
            printf("ERROR: Need more parents\n");
            exit(-1);
         }
         if (p == max_active_parent)
            max_active_parent++;
         num_parents++;
         num_refined++;
         pp = &parents[p];
         pp->number = bp->number;
         pp->num_prime = bp->num_prime;
         pp->level = bp->level;
         pp->b_type = bp->b_type;
         pp->parent = bp->parent;
         pp->parent_node = bp->parent_node;
         pp->child_number = bp->child_number;
         if (pp->parent_node != my_pe)
            one_rank_only("split_blocks parent", (long long) bp->number, -1);
         if (pp->parent >= 0)
            parents[pp->parent].child[pp->child_number] = -1 - p;
         pp->refine = 0;
         pp->cen[0] = bp->cen[0];
         pp->cen[1] = bp->cen[1];
         pp->cen[2] = bp->cen[2];

         if (n_jobs == cap_split) {
            cap_split = 2*cap_split + 16;
            split_jobs = (mamr_split_job *)
               realloc(split_jobs, sizeof(mamr_split_job)*cap_split);
            if (!split_jobs) {
               printf("ERROR: split_blocks: out of host memory\n");
               exit(-1);
            }
         }
         split_jobs[n_jobs].parent = n;

         for (o1 = 0; o1 < 8; o1++) {
            /* next free slot, continuing from the last one handed out */
            for ( ; m < max_num_blocks; m++)
               if (blocks[m].number < 0)
                  break;
            if (m == max_num_blocks) {
               printf("Error: No inactive blocks available %d %d %d\n",
                      m, num_active, max_num_blocks);
               exit(-1);
            }
            if ((m+1) > max_active_block)
               max_active_block = m+1;
            bp1 = &blocks[m];
            if (lb_method >= 2) {
               o = hilbert[bp->b_type][o1][0];
               bp1->b_type = hilbert[bp->b_type][o1][1];
            } else {
               o = o1;
               bp1->b_type = 0;
            }
            sib[o] = m;
            pp->child[o] = m;
            pp->child_node[o] = my_pe;
            split_jobs[n_jobs].child[o] = m;
            bp1->refine = 0;
            bp1->level = level + 1;
            bp1->parent = p;
            bp1->parent_node = my_pe;
            bp1->child_number = o;
            i1 = o % 2;
            j1 = (o / 2) % 2;
            k1 = o / 4;
            bp1->number = (num_sz) ((2*zp + k1)*(p2[level+1]*init_y) +
                                    (2*yp + j1))*(p2[level+1]*init_x) +
                          2*xp + i1 + block_start[level+1];
            bp1->num_prime = bp->num_prime + o1*p8[num_refine - level - 1];
            add_sorted_list(m, bp1->number, level+1);
            bp1->cen[0] = bp->cen[0] + (2*i1 - 1)*p2[num_refine - level - 1];
            bp1->cen[1] = bp->cen[1] + (2*j1 - 1)*p2[num_refine - level - 1];
            bp1->cen[2] = bp->cen[2] + (2*k1 - 1)*p2[num_refine - level - 1];
         }
         n_jobs++;

         for (c = 0; c < 6; c++) {
            int opp = c ^ 1;
            /* siblings facing each other across the parent's mid-plane */
            for (a = 0; a < 2; a++)
               for (b = 0; b < 2; b++) {
                  int s = face_child(c, a, b);
                  blocks[sib[s ^ dir_bit(c)]].nei_level[c] = level + 1;
                  blocks[sib[s ^ dir_bit(c)]].nei[c][0][0] = sib[s];
               }
            /* the children on face c take over the parent's neighbour */
            if (bp->nei_level[c] == -2) {
               for (a = 0; a < 2; a++)
                  for (b = 0; b < 2; b++) {
                     blocks[sib[face_child(c, a, b)]].nei_level[c] = -2;
                     blocks[sib[face_child(c, a, b)]].nei[c][0][0] = 0;
                  }
            } else if (bp->nei_level[c] == level - 1) {
               if (bp->nei[c][0][0] >= 0) {
                  printf("%d ERROR: internal misconnect block %lld c %d\n",
                         my_pe, (long long) bp->number, c);
                  exit(-1);
               }
               one_rank_only("split_blocks", (long long) bp->number, c);
            } else if (bp->nei_level[c] == level) {
               int other = bp->nei[c][0][0];
               if (other < 0)
                  one_rank_only("split_blocks", (long long) bp->number, c);
               blocks[other].nei_level[opp] = level + 1;
               for (a = 0; a < 2; a++)
                  for (b = 0; b < 2; b++) {
                     int ch = sib[face_child(c, a, b)];
                     blocks[ch].nei_level[c] = level;
                     blocks[ch].nei[c][0][0] = other;
                     blocks[other].nei[opp][a][b] = ch;
                  }
            } else if (bp->nei_level[c] == level + 1) {
               for (a = 0; a < 2; a++)
                  for (b = 0; b < 2; b++) {
                     int other = bp->nei[c][a][b];
                     int ch = sib[face_child(c, a, b)];
                     if (other < 0)
                        one_rank_only("split_blocks", (long long) bp->number,
                                      c);
                     blocks[ch].nei_level[c] = level + 1;
                     blocks[ch].nei[c][0][0] = other;
                     blocks[other].nei_level[opp] = level + 1;
                     blocks[other].nei[opp][0][0] = ch;
                  }
            } else {
               printf("%d ERROR: misconnected b %d %lld l %d nei[%d] %d\n",
                      my_pe, n, (long long) bp->number, level, c,
                      bp->nei_level[c]);
               exit(-1);
            }
         }
         /* the parent's slot is free again and may take a later child */
         bp->number = -1;
         if (n < m)
            m = n;
      }
      comm_refine();
   }
   if (n_jobs)
      mamr_dropin_check(mamr_split(mamr_dropin_ctx(), split_jobs, n_jobs),
                        "split_blocks");
   mamr_dropin_mesh_changed();
}

void consolidate_blocks(void)
{
   int n, p, o, c, a, b, level, in, n_jobs = 0;
   block *bp, *bp1;
   parent *pp;

   mamr_dropin_sync_data();
   for (level = cur_max_level; level >= 0; level--)
      for (p = 0; p < max_active_parent; p++) {
         pp = &parents[p];
         if (pp->number < 0 || pp->level != level || pp->refine != -1)
            continue;
         /* first free slot from the start of the pool */
         for (n = 0; n < max_num_blocks; n++)
            if (blocks[n].number < 0)
               break;
         if (n == max_num_blocks) {
            printf("Out of free blocks in consolidate_blocks %d\n", my_pe);
            exit(-1);
         }
         bp = &blocks[n];
         if ((n+1) > max_active_block)
            max_active_block = n+1;
         if ((num_active + 1) > local_max_b)
            local_max_b = num_active + 1;
         num_active -= 7;
         num_reformed++;
         local_num_blocks[level]++;
         local_num_blocks[level+1] -= 8;
         bp->number = pp->number;
         bp->num_prime = pp->num_prime;
         pp->number = -1;
         num_parents--;
         bp->level = pp->level;
         bp->b_type = pp->b_type;
         bp->parent = pp->parent;
         bp->parent_node = pp->parent_node;
         bp->child_number = pp->child_number;
         if (bp->level) {
            if (bp->parent_node != my_pe)
               one_rank_only("consolidate_blocks parent",
                             (long long) bp->number, -1);
            parents[bp->parent].child[bp->child_number] = n;
         }
         add_sorted_list(n, bp->number, level);
         bp->refine = 0;
         bp->cen[0] = pp->cen[0];
         bp->cen[1] = pp->cen[1];
         bp->cen[2] = pp->cen[2];

         if (n_jobs == cap_cons) {
            cap_cons = 2*cap_cons + 16;
            cons_jobs = (mamr_consolidate_job *)
               realloc(cons_jobs, sizeof(mamr_consolidate_job)*cap_cons);
            if (!cons_jobs) {
               printf("ERROR: consolidate_blocks: out of host memory\n");
               exit(-1);
            }
         }
         cons_jobs[n_jobs].target = n;
         for (o = 0; o < 8; o++) {
            bp1 = &blocks[pp->child[o]];
            del_sorted_list(bp1->number, level+1, 2);
            bp1->number = -1;
            cons_jobs[n_jobs].child[o] = (int32_t) pp->child[o];
         }
         n_jobs++;

         for (c = 0; c < 6; c++) {
            int opp = c ^ 1;
            int other = (int) pp->child[face_child(c, 0, 0)];
            if (blocks[other].nei_level[c] == -2) {
               bp->nei_level[c] = -2;
               bp->nei_refine[c] = 0;
            } else if (blocks[other].nei_level[c] == level) {
               int nb = blocks[other].nei[c][0][0];
               if (nb < 0)
                  one_rank_only("consolidate_blocks", (long long) bp->number,
                                c);
               bp->nei[c][0][0] = nb;
               bp->nei_level[c] = level;
               bp->nei_refine[c] = 0;
               blocks[nb].nei[opp][0][0] = n;
               blocks[nb].nei_level[opp] = level;
               blocks[nb].nei_refine[opp] = 0;
            } else {
               for (a = 0; a < 2; a++)
                  for (b = 0; b < 2; b++) {
                     int ch = (int) pp->child[face_child(c, a, b)];
                     int nb = blocks[ch].nei[c][0][0];
                     if (nb < 0)
                        one_rank_only("consolidate_blocks",
                                      (long long) bp->number, c);
                     if (blocks[ch].nei_level[c] == level + 2) {
                        printf("%d ERROR: %d con %d block %d c %d wrong level %d\n",
                               my_pe, p, n, ch, c, level);
                        exit(-1);
                     }
                     bp->nei[c][a][b] = nb;
                     bp->nei_level[c] = level + 1;
                     bp->nei_refine[c] = 0;
                     blocks[nb].nei[opp][0][0] = n;
                     blocks[nb].nei_level[opp] = level;
                     blocks[nb].nei_refine[opp] = 0;
                  }
            }
         }
      }

   /* off-rank neighbours that are coarsening: none on one rank */
   for (in = 0; in < sorted_index[num_refine+1]; in++) {
      bp = &blocks[sorted_list[in].n];
      for (c = 0; c < 6; c++)
         if (bp->nei[c][0][0] < 0 && bp->nei_refine[c] == -1)
            one_rank_only("consolidate_blocks", (long long) bp->number, c);
   }
   if (n_jobs)
      mamr_dropin_check(mamr_consolidate(mamr_dropin_ctx(), cons_jobs,
                                         n_jobs), "consolidate_blocks");
   mamr_dropin_mesh_changed();
}

/* Inserts (n, number) into level's run of the sorted list, before the first
 * entry with a smaller block number. */
void add_sorted_list(int n, num_sz number, int level)
{
   int at, j, end = sorted_index[num_refine+1];

   for (at = sorted_index[level]; at < sorted_index[level+1]; at++)
      if (number > sorted_list[at].number)
         break;
   for (j = end; j > at; j--)
      sorted_list[j] = sorted_list[j-1];
   sorted_list[at].number = number;
   sorted_list[at].n = n;
   for (j = level + 1; j <= num_refine + 1; j++)
      sorted_index[j]++;
}

void del_sorted_list(num_sz number, int level, int from)
{
   int at, j, found = 0;

   for (at = sorted_index[level]; at < sorted_index[level+1]; at++)
      if (sorted_list[at].number == number) {
         found = 1;
         break;
      }
   if (!found) {
      printf("ERROR: del_sorted_list on %d - number %lld not found l %d f %d\n",
             my_pe, (long long) number, level, from);
      exit(-1);
   }
   for (j = level + 1; j <= num_refine + 1; j++)
      sorted_index[j]--;
   for (j = at; j < sorted_index[num_refine+1]; j++)
      sorted_list[j] = sorted_list[j+1];
}

int find_sorted_list(num_sz number, int level)
{
   int at;

   for (at = sorted_index[level]; at < sorted_index[level+1]; at++)
      if (sorted_list[at].number == number)
         return sorted_list[at].n;
   printf("ERROR: find_sorted_list on %d - number %lld not found\n",
          my_pe, (long long) number);
   exit(-1);
}
