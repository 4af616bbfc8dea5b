// Host-side reproduction of the reference's initial cell values
// (ref/init.c:484-495 with glibc's rand(); rand() is never seeded there, so
// its stream starts from seed 1).  random_r with a private 128-byte state
// initialised by initstate_r(1, ...) yields the same stream as an unseeded
// rand() and leaves the process-wide rand() state alone.
#include <cstdlib>
#include <cstring>

#include "miniamr_gb300.h"

extern "C" int mamr_initial_values(const mamr_config *cfg, int32_t n_blocks,
                                   double *out)
{
   if (!cfg || n_blocks < 0 || (n_blocks && !out) || cfg->nx < 1 ||
       cfg->ny < 1 || cfg->nz < 1 || cfg->num_vars < 1)
      return MAMR_EINVAL;
   char state[128];
   struct random_data rd;
   memset(&rd, 0, sizeof(rd));
   memset(state, 0, sizeof(state));
   if (initstate_r(1u, state, sizeof(state), &rd) != 0)
      return MAMR_EINVAL;
   const int X = cfg->nx + 2, Y = cfg->ny + 2, Z = cfg->nz + 2;
   const size_t bv = (size_t) X * Y * Z;
   for (int32_t b = 0; b < n_blocks; b++)
      for (int v = 0; v < cfg->num_vars; v++) {
         double *a = out + ((size_t) b * cfg->num_vars + v) * bv;
         memset(a, 0, sizeof(double) * bv);
         for (int i = 1; i <= cfg->nx; i++)
            for (int j = 1; j <= cfg->ny; j++)
               for (int k = 1; k <= cfg->nz; k++) {
                  int32_t r;
                  random_r(&rd, &r);
                  a[((size_t) i * Y + j) * Z + k] =
                     ((double) r) / ((double) RAND_MAX);
               }
      }
   return MAMR_OK;
}
