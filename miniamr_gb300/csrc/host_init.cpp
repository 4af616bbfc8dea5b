// Host-side reproduction of the reference's initial cell values
// (ref/init.c:484-495) and stencil-0 coefficients (ref/init.c:418-423) with
// glibc's rand(); rand() is never seeded there, so its stream starts from
// seed 1.  random_r with a private 128-byte state
// initialised by initstate_r(1, ...) yields the same stream as an unseeded
// rand() and leaves the process-wide rand() state alone.
#include <cstdlib>
#include <cstring>

#include "miniamr_gb300.h"

namespace {

// The seed-1 stream of an unseeded rand(), in a private state.
struct RandStream {
   char state[128];
   struct random_data rd;
   bool ok;
   RandStream()
   {
      memset(&rd, 0, sizeof(rd));
      memset(state, 0, sizeof(state));
      ok = initstate_r(1u, state, sizeof(state), &rd) == 0;
   }
   double next()        // rand()/RAND_MAX
   {
      int32_t r;
      random_r(&rd, &r);
      return ((double) r) / ((double) RAND_MAX);
   }
};

}  // namespace

extern "C" int mamr_work_coefficients(int32_t num_vars, double *a1,
                                      double *a0)
{
   if (num_vars < 1 || !a1 || (num_vars >= 4 && !a0))
      return MAMR_EINVAL;
   RandStream rs;
   if (!rs.ok)
      return MAMR_EINVAL;
   *a1 = rs.next();
   for (int i = 0; i < num_vars / 4; i++)
      a0[i] = rs.next();
   return MAMR_OK;
}

extern "C" int mamr_initial_values(const mamr_config *cfg, int32_t n_blocks,
                                   double *out)
{
   if (!cfg || n_blocks < 0 || (n_blocks && !out) || cfg->nx < 1 ||
       cfg->ny < 1 || cfg->nz < 1 || cfg->num_vars < 1)
      return MAMR_EINVAL;
   RandStream rs;
   if (!rs.ok)
      return MAMR_EINVAL;
   // stencil 0: init() draws a1 and a0[] first (ref/init.c:418-423)
   if (cfg->stencil == 0)
      for (int i = 0; i < 1 + cfg->num_vars / 4; i++)
         rs.next();
   const int X = cfg->nx + 2, Y = cfg->ny + 2, Z = cfg->nz + 2;
   const size_t bv = (size_t) X * Y * Z;
   for (int32_t b = 0; b < n_blocks; b++)
      for (int v = 0; v < cfg->num_vars; v++) {
         double *a = out + ((size_t) b * cfg->num_vars + v) * bv;
         memset(a, 0, sizeof(double) * bv);
         for (int i = 1; i <= cfg->nx; i++)
            for (int j = 1; j <= cfg->ny; j++)
               for (int k = 1; k <= cfg->nz; k++)
                  a[((size_t) i * Y + j) * Z + k] = rs.next();
      }
   return MAMR_OK;
}
