/*
 * Call recorder for the drop-in hybrid (oracle/_ref/miniamr_hybrid_trace).
 *
 * Test infrastructure only.  Linked with -Wl,--wrap=mamr_<fn> for every
 * ABI call the drop-in translation units make, so that the reference's own
 * driver, init and refine code run unchanged over the drop-in and the CPU
 * oracle while each call is appended to the file named by MAMR_TRACE.
 * Replaying the file through another implementation of the ABI (the GB300
 * library on a GPU host, where the reference sources do not exist) repeats
 * exactly the calls the reference's driver made, and the recorded check_sum
 * results are the reference's own checksums.
 *
 * File: "MAMRTRC1", then records {int32 op, int32 nbytes, payload}:
 *   1 create      mamr_config
 *   2 upload      int32 n, int32 slots[n], uint64 hash of the doubles
 *                 (sum of bits[q] * (mix64(q) | 1) mod 2^64)
 *   3 set_mesh    int32 n, mamr_block[n], int64 numbers[n]
 *   4 comm        int32 start, num, stage
 *   5 stencil     int32 var, calc_stage
 *   6 check_sum   int32 var, int32 pad, double result
 *   7 split       int32 n, mamr_split_job[n]
 *   8 consolidate int32 n, mamr_consolidate_job[n]
 *   9 work params int32 n, int32 pad, double a1, double a0[n]
 * Little-endian, as written by the host.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>

#include "block.h"
#include "miniamr_gb300.h"

int __real_mamr_create(const mamr_config *cfg, mamr_ctx **out);
int __real_mamr_upload_blocks(mamr_ctx *ctx, const int32_t *slots, int32_t n,
                              const double *host);
int __real_mamr_set_mesh(mamr_ctx *ctx, const mamr_block *b, int32_t n);
int __real_mamr_comm(mamr_ctx *ctx, int32_t start, int32_t num, int32_t stage);
int __real_mamr_stencil(mamr_ctx *ctx, int32_t var, int32_t stage);
int __real_mamr_check_sum(mamr_ctx *ctx, int32_t var, double *sum);
int __real_mamr_split(mamr_ctx *ctx, const mamr_split_job *j, int32_t n);
int __real_mamr_consolidate(mamr_ctx *ctx, const mamr_consolidate_job *j,
                            int32_t n);
int __real_mamr_set_work_params(mamr_ctx *ctx, double a1, const double *a0,
                                int32_t n);

static FILE *fp;
static int opened;

static FILE *trace(void)
{
   if (!opened) {
      const char *p = getenv("MAMR_TRACE");
      opened = 1;
      if (p && *p) {
         fp = fopen(p, "wb");
         if (!fp) {
            fprintf(stderr, "trace_hooks: cannot open %s\n", p);
            exit(-1);
         }
         fwrite("MAMRTRC1", 1, 8, fp);
      }
   }
   return fp;
}

static void rec(int32_t op, const void *a, size_t na, const void *b,
                size_t nb, const void *c, size_t nc)
{
   FILE *f = trace();
   int32_t len = (int32_t) (na + nb + nc);
   if (!f)
      return;
   fwrite(&op, 4, 1, f);
   fwrite(&len, 4, 1, f);
   if (na) fwrite(a, 1, na, f);
   if (nb) fwrite(b, 1, nb, f);
   if (nc) fwrite(c, 1, nc, f);
}

int __wrap_mamr_create(const mamr_config *cfg, mamr_ctx **out)
{
   rec(1, cfg, sizeof(*cfg), NULL, 0, NULL, 0);
   return __real_mamr_create(cfg, out);
}

int __wrap_mamr_upload_blocks(mamr_ctx *ctx, const int32_t *slots, int32_t n,
                              const double *host)
{
   size_t cells = (size_t) n * num_vars * (x_block_size + 2) *
                  (y_block_size + 2) * (z_block_size + 2), q;
   uint64_t h = 0;
   for (q = 0; q < cells; q++) {
      uint64_t bits, z = q;
      memcpy(&bits, &host[q], 8);
      z += 0x9E3779B97F4A7C15ULL;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      z ^= z >> 31;
      h += bits * (z | 1);
   }
   rec(2, &n, 4, slots, sizeof(int32_t) * n, &h, 8);
   return __real_mamr_upload_blocks(ctx, slots, n, host);
}

int __wrap_mamr_set_mesh(mamr_ctx *ctx, const mamr_block *b, int32_t n)
{
   int64_t *num = (int64_t *) malloc(sizeof(int64_t) * (n ? n : 1));
   int32_t q;
   for (q = 0; q < n; q++)
      num[q] = (int64_t) blocks[b[q].slot].number;
   rec(3, &n, 4, b, sizeof(mamr_block) * n, num, sizeof(int64_t) * n);
   free(num);
   return __real_mamr_set_mesh(ctx, b, n);
}

int __wrap_mamr_comm(mamr_ctx *ctx, int32_t start, int32_t num, int32_t stage)
{
   int32_t a[3] = { start, num, stage };
   rec(4, a, sizeof(a), NULL, 0, NULL, 0);
   return __real_mamr_comm(ctx, start, num, stage);
}

int __wrap_mamr_set_work_params(mamr_ctx *ctx, double a1, const double *a0,
                                int32_t n)
{
   int32_t h[2] = { n, 0 };
   rec(9, h, sizeof(h), &a1, sizeof(double), a0, sizeof(double) * n);
   return __real_mamr_set_work_params(ctx, a1, a0, n);
}

int __wrap_mamr_stencil(mamr_ctx *ctx, int32_t var, int32_t stage)
{
   int32_t a[2] = { var, stage };
   rec(5, a, sizeof(a), NULL, 0, NULL, 0);
   return __real_mamr_stencil(ctx, var, stage);
}

int __wrap_mamr_check_sum(mamr_ctx *ctx, int32_t var, double *sum)
{
   int r = __real_mamr_check_sum(ctx, var, sum);
   int32_t a[2] = { var, 0 };
   rec(6, a, sizeof(a), sum, sizeof(double), NULL, 0);
   return r;
}

int __wrap_mamr_split(mamr_ctx *ctx, const mamr_split_job *j, int32_t n)
{
   rec(7, &n, 4, j, sizeof(mamr_split_job) * n, NULL, 0);
   return __real_mamr_split(ctx, j, n);
}

int __wrap_mamr_consolidate(mamr_ctx *ctx, const mamr_consolidate_job *j,
                            int32_t n)
{
   rec(8, &n, 4, j, sizeof(mamr_consolidate_job) * n, NULL, 0);
   return __real_mamr_consolidate(ctx, j, n);
}
