/*
 * Drop-in replacement for the reference's comm.c on one rank.
 *
 * comm() keeps its signature (ref/proto.h:49, called from
 * ref/driver.c:81) and runs the on-rank exchange (ref/comm.c:162-203) on
 * the device through mamr_comm().  The message paths (ref/comm.c:58-157,
 * 205-239) have no partner on one rank and are not run.  The exchange
 * counters the profile report prints (counter_same/diff/bc,
 * ref/comm.c:169,178,196) are advanced exactly as the reference does.
 * pack_face, unpack_face, on_proc_comm, on_proc_comm_diff and apply_bc
 * (ref/proto.h:50-54) are internal to the reference's comm.c; they are kept
 * for link compatibility and fail loudly if anything calls them.
 */
#include <stdio.h>
#include <stdlib.h>
#include <mpi.h>

#include "block.h"
#include "comm.h"
#include "timer.h"
#include "proto.h"
#include "dropin.h"

void comm(int start, int num_comm, int stage)
{
   static const int perm[6][3] = { {0, 1, 2}, {1, 2, 0}, {2, 0, 1},
                                   {0, 2, 1}, {1, 0, 2}, {2, 1, 0} };
   int o, dir, in, l, i, j, m, n, k;
   double t1, t2;
   block *bp;

   t1 = timer();
   mamr_dropin_sync_state();
   mamr_dropin_check(mamr_comm(mamr_dropin_ctx(), start, num_comm, stage),
                     "comm");
   t2 = timer();

   /* Same accounting as the reference's on-rank loop. */
   for (o = 0; o < 3; o++) {
      dir = permute ? perm[stage % 6][o] : o;
      timer_comm_dir[dir] += (t2 - t1) / 3.0;
      for (in = 0; in < sorted_index[num_refine+1]; in++) {
         bp = &blocks[n = sorted_list[in].n];
         for (l = dir*2; l < dir*2 + 2; l++) {
            if (bp->nei_level[l] == bp->level) {
               if (bp->nei[l][0][0] > n)
                  counter_same[dir] += 2;
            } else if (bp->nei_level[l] == bp->level + 1) {
               for (i = 0; i < 2; i++)
                  for (j = 0; j < 2; j++)
                     if (bp->nei[l][i][j] > n)
                        counter_diff[dir] += 2;
            } else if (bp->nei_level[l] == bp->level - 1) {
               if ((m = bp->nei[l][0][0]) > n) {
                  k = dir*2 + 1 - l%2;
                  for (i = 0; i < 2; i++)
                     for (j = 0; j < 2; j++)
                        if (blocks[m].nei[k][i][j] == n)
                           counter_diff[dir] += 2;
               }
            } else if (bp->nei_level[l] == -2) {
               counter_bc[dir]++;
            }
         }
      }
   }
}

static void not_on_one_rank(const char *what)
{
   printf("ERROR: %s is internal to the reference's comm.c and is not "
          "used by the GB300 back end\n", what);
   exit(-1);
}

void pack_face(double *send_buf, int block_num, int face_case, int dir,
               int start, int num_comm)
{
   (void) send_buf; (void) block_num; (void) face_case; (void) dir;
   (void) start; (void) num_comm;
   not_on_one_rank("pack_face");
}

void unpack_face(double *recv_buf, int block_num, int face_case, int dir,
                 int start, int num_comm)
{
   (void) recv_buf; (void) block_num; (void) face_case; (void) dir;
   (void) start; (void) num_comm;
   not_on_one_rank("unpack_face");
}

void on_proc_comm(int n, int n1, int l, int start, int num_comm)
{
   (void) n; (void) n1; (void) l; (void) start; (void) num_comm;
   not_on_one_rank("on_proc_comm");
}

void on_proc_comm_diff(int n, int n1, int l, int iq, int jq, int start,
                       int num_comm)
{
   (void) n; (void) n1; (void) l; (void) iq; (void) jq; (void) start;
   (void) num_comm;
   not_on_one_rank("on_proc_comm_diff");
}

void apply_bc(int l, block *bp, int start, int num_comm)
{
   (void) l; (void) bp; (void) start; (void) num_comm;
   not_on_one_rank("apply_bc");
}
