/*
 * Drop-in replacement for the reference's stencil.c.
 *
 * stencil_driver(var, calc_stage) keeps its signature (ref/proto.h:125,
 * called from ref/driver.c:86) and, for stencil 7 or 27, runs
 * stencil_calc(var, stencil) (ref/stencil.c:76-145) on the device through
 * mamr_stencil().  The flop counters follow ref/stencil.c:100-101,142-143.
 * The variable-work stencils of --stencil 0 (ref/stencil.c:147-983) are not
 * run by this back end; selecting them is reported as an error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <mpi.h>

#include "block.h"
#include "comm.h"
#include "timer.h"
#include "proto.h"
#include "dropin.h"

void stencil_driver(int var, int calc_stage)
{
   if (stencil != 7 && stencil != 27) {
      printf("ERROR: stencil %d is not run by the GB300 back end\n",
             stencil);
      exit(-1);
   }
   mamr_dropin_sync_state();
   mamr_dropin_check(mamr_stencil(mamr_dropin_ctx(), var, calc_stage),
                     "stencil_driver");
   total_fp_divs += (double) num_active*num_cells;
   total_fp_adds += (double) (stencil == 7 ? 6 : 26)*num_active*num_cells;
}
