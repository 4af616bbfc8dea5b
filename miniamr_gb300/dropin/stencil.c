/*
 * Drop-in replacement for the reference's stencil.c.
 *
 * stencil_driver(var, calc_stage) keeps its signature (ref/proto.h:125,
 * called from ref/driver.c:86) and its dispatch (ref/stencil.c:43-74): for
 * stencil 7 or 27 stencil_calc(var, stencil) (ref/stencil.c:76-145); for
 * stencil 0, var 0 and vars >= 4*mat stencil_calc(var, 7), the others the
 * variable-work kernel of calc_stage % 6 (ref/stencil.c:147-957) and
 * stencil_check (ref/stencil.c:959-983) -- all on the device through
 * mamr_stencil().  The flop counters follow the reference's increments,
 * except stencil_check's, which depend on each cell's value: they feed
 * only the run's printed flop totals, which therefore leave those out.
 */
#include <stdio.h>
#include <stdlib.h>
#include <mpi.h>

#include "block.h"
#include "comm.h"
#include "timer.h"
#include "proto.h"
#include "dropin.h"

/* ref/stencil.c:147-957: the counters of each kernel's branch for var */
static void count_work(int var, int calc_stage)
{
   const double n = (double) num_active*num_cells;
   int cls = var == 1 ? -1 : var < mat ? 0 : var < 2*mat ? 1
           : var < 3*mat ? 2 : 3;
   switch (calc_stage%6) {
   case 0:
      if (cls == -1) {
         total_fp_adds += (double) mat*n;
         total_fp_muls += (double) mat*n;
      } else if (cls == 0) {
         total_fp_adds += 3*n; total_fp_muls += 2*n;
      } else if (cls == 1) {
         total_fp_adds += 3*n; total_fp_muls += 3*n; total_fp_divs += n;
      } else if (cls == 2) {
         total_fp_adds += 4*n; total_fp_muls += 3*n; total_fp_divs += n;
      } else {
         total_fp_adds += 6*n; total_fp_muls += 6*n; total_fp_divs += n;
      }
      break;
   case 1:
   case 2:
   case 3:
      if (cls == -1) {
         total_fp_adds += (double) (mat+1)*n;
         total_fp_muls += (double) mat*n;
         total_fp_divs += n;
      } else if (cls == 0) {
         total_fp_adds += 4*n; total_fp_muls += 2*n; total_fp_divs += n;
      } else {
         total_fp_adds += 12*n; total_fp_muls += 3*n; total_fp_divs += n;
      }
      break;
   case 4:
      total_fp_adds += 7*n; total_fp_muls += 8*n; total_fp_divs += n;
      break;
   default:
      total_fp_adds += 27*n; total_fp_divs += n;
      break;
   }
}

void stencil_driver(int var, int calc_stage)
{
   if (stencil != 0 && stencil != 7 && stencil != 27) {
      printf("ERROR: stencil %d is not run by the GB300 back end\n",
             stencil);
      exit(-1);
   }
   mamr_dropin_sync_state();
   mamr_dropin_check(mamr_stencil(mamr_dropin_ctx(), var, calc_stage),
                     "stencil_driver");
   if (stencil == 0 && var != 0 && var < 4*mat) {
      count_work(var, calc_stage);
   } else {
      total_fp_divs += (double) num_active*num_cells;
      total_fp_adds += (double) (stencil == 27 ? 26 : 6)*num_active*num_cells;
   }
}
