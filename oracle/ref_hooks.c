/*
 * Link-time hooks for the reference build (oracle/_ref/miniamr_ref) and the
 * drop-in hybrid build (oracle/_ref/miniamr_hybrid_oracle).
 *
 * Test infrastructure only.  Linked with -Wl,--wrap=check_sum,--wrap=refine
 * so that the reference's own code runs unchanged and this file only
 * observes it.  When the environment variable MAMR_REF_LOG names a file,
 * every check_sum() call (ref/check_sum.c:36, called from ref/driver.c:91
 * and ref/init.c:682) appends one line
 *
 *     cs <call#> <var> <checksum as 16 hex digits> <cell hash, 16 hex>
 *
 * where the cell hash (var_cell_hash below) covers the bit pattern of
 * every cell, ghosts included, of that variable in every active block, in
 * sorted_list order (ref/block.h:72-77), and each block's number
 * (0 where MAMR_REF_HASH_STRIDE skips it).  Every refine() call (ref/refine.c:38) appends one line
 *
 *     mesh <ts> <n_active> <hash of (slot,number,level,nei_level,nei,cen)>
 *
 * plus, when MAMR_REF_MESH_DUMP is set, the per-block records themselves.
 *
 * With -Wl,--wrap=split_blocks, when MAMR_MARK_DUMP names a file, every
 * split_blocks() call (ref/refine.c:112, right after the marking of
 * ref/refine.c:66-110) first appends the marking's inputs and results:
 *
 *     step <call#> <n_blocks> <n_parent_slots> <num_refine> <refine_ghost>
 *          <uniform_refine> <mesh_size x3> <block size x3> <num_objects>
 *     o <type> <cen x3> <size x3>          (doubles as 16 hex digits)
 *     b <slot> <level> <parent> <cen x3> <nei_level x6> <nei[l][0][0] x6>
 *       <refine>                           (active blocks, sorted order)
 *     p <index> <active> <child x8> <refine>     (parents[0..max_active))
 *
 * MAMR_MARK_DUMP_EVERY=n keeps every n-th call, MAMR_MARK_DUMP_MAX=m at
 * most m of them.
 * The hybrid build holds its cell data behind the mamr_* C ABI; there the
 * drop-in's mamr_dropin_fetch() (a weak reference here) supplies the cells.
 */
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>
#include <mpi.h>

#include "block.h"
#include "comm.h"
#include "proto.h"

double __real_check_sum(int var);
void __real_refine(int ts);
void __real_split_blocks(void);

/* Provided by the drop-in check_sum.c replacement in the hybrid build. */
extern int mamr_dropin_fetch(int slot, int var, double *out)
   __attribute__((weak));

static FILE *log_fp;
static int log_checked;
static long cs_calls;

static FILE *hook_log(void)
{
   if (!log_checked) {
      const char *p = getenv("MAMR_REF_LOG");
      log_checked = 1;
      if (p && *p) {
         log_fp = fopen(p, "w");
         if (!log_fp) {
            fprintf(stderr, "ref_hooks: cannot open %s\n", p);
            exit(-1);
         }
      }
   }
   return log_fp;
}

static uint64_t fnv_bytes(uint64_t h, const void *p, size_t n)
{
   const unsigned char *c = (const unsigned char *) p;
   size_t i;
   for (i = 0; i < n; i++) {
      h ^= c[i];
      h *= 1099511628211ULL;
   }
   return h;
}

/* splitmix64 finaliser: position weights of the cell hash. */
static uint64_t mix64(uint64_t z)
{
   z += 0x9E3779B97F4A7C15ULL;
   z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
   z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
   return z ^ (z >> 31);
}

/* Cell hash of one variable: sum over active blocks (position p in
 * sorted_list) of number * w(p, 2^32-1) plus, over every cell c of the
 * block-variable (ghosts included, [i][j][k] order), bits(cell) * w(p, c),
 * all mod 2^64, with w(p, c) = mix64(p << 32 | c) | 1. */
static uint64_t var_cell_hash(int var)
{
   int in, i, j, k, nx2 = x_block_size + 2, ny2 = y_block_size + 2,
       nz2 = z_block_size + 2;
   uint64_t h = 0;
   double *buf = NULL;

   if (mamr_dropin_fetch)
      buf = (double *) malloc(sizeof(double) * nx2 * ny2 * nz2);
   for (in = 0; in < sorted_index[num_refine+1]; in++) {
      int n = sorted_list[in].n;
      uint64_t c = 0, base = (uint64_t) in << 32;
      h += (uint64_t) (long long) blocks[n].number * (mix64(base | 0xFFFFFFFFULL) | 1);
      if (buf && mamr_dropin_fetch(n, var, buf)) {
         fprintf(stderr, "ref_hooks: fetch failed\n");
         exit(-1);
      }
      for (i = 0; i < nx2; i++)
         for (j = 0; j < ny2; j++)
            for (k = 0; k < nz2; k++, c++) {
               double v = buf ? buf[c] : blocks[n].array[var][i][j][k];
               uint64_t bits;
               memcpy(&bits, &v, sizeof(bits));
               h += bits * (mix64(base | c) | 1);
            }
   }
   free(buf);
   return h;
}

/* MAMR_REF_HASH_STRIDE=n: cell hashes only for every n-th group of
 * num_vars check_sum calls (the others log hash 0), for long runs. */
static long hash_stride(void)
{
   static long stride = -1;
   if (stride < 0) {
      const char *p = getenv("MAMR_REF_HASH_STRIDE");
      stride = (p && atol(p) > 0) ? atol(p) : 1;
   }
   return stride;
}

double __wrap_check_sum(int var)
{
   double s = __real_check_sum(var);
   FILE *fp = hook_log();
   if (fp) {
      uint64_t bits, h = 0;
      memcpy(&bits, &s, sizeof(bits));
      if ((cs_calls / num_vars) % hash_stride() == 0)
         h = var_cell_hash(var);
      fprintf(fp, "cs %ld %d %016llx %016llx\n", cs_calls, var,
              (unsigned long long) bits, (unsigned long long) h);
   }
   cs_calls++;
   return s;
}

void __wrap_refine(int ts)
{
   FILE *fp;
   __real_refine(ts);
   fp = hook_log();
   if (fp) {
      int in, l, a, b, dump = getenv("MAMR_REF_MESH_DUMP") != NULL;
      uint64_t h = 1469598103934665603ULL;
      for (in = 0; in < sorted_index[num_refine+1]; in++) {
         int n = sorted_list[in].n;
         block *bp = &blocks[n];
         int rec[1 + 1 + 6 + 24 + 3];
         long long number = (long long) bp->number;
         rec[0] = n;
         rec[1] = bp->level;
         for (l = 0; l < 6; l++) {
            rec[2 + l] = bp->nei_level[l];
            for (a = 0; a < 2; a++)
               for (b = 0; b < 2; b++)
                  rec[8 + l*4 + a*2 + b] = bp->nei[l][a][b];
         }
         rec[32] = bp->cen[0];
         rec[33] = bp->cen[1];
         rec[34] = bp->cen[2];
         h = fnv_bytes(h, &number, sizeof(number));
         h = fnv_bytes(h, rec, sizeof(rec));
         if (dump) {
            fprintf(fp, "blk %lld", number);
            for (l = 0; l < 35; l++)
               fprintf(fp, " %d", rec[l]);
            fprintf(fp, "\n");
         }
      }
      fprintf(fp, "mesh %d %d %016llx\n", ts, sorted_index[num_refine+1],
              (unsigned long long) h);
      fflush(fp);
   }
}

static long env_long(const char *name, long dflt)
{
   const char *p = getenv(name);
   return (p && *p) ? atol(p) : dflt;
}

static void put_f64(FILE *fp, double x)
{
   uint64_t b;
   memcpy(&b, &x, sizeof(b));
   fprintf(fp, " %016llx", (unsigned long long) b);
}

void __wrap_split_blocks(void)
{
   static FILE *mfp;
   static int opened;
   static long calls, dumped;
   if (!opened) {
      const char *p = getenv("MAMR_MARK_DUMP");
      opened = 1;
      if (p && *p && !(mfp = fopen(p, "w"))) {
         fprintf(stderr, "ref_hooks: cannot open %s\n", p);
         exit(-1);
      }
   }
   if (mfp && calls % env_long("MAMR_MARK_DUMP_EVERY", 1) == 0 &&
       dumped < env_long("MAMR_MARK_DUMP_MAX", 1L << 30)) {
      int in, o, l, d, k, nb = sorted_index[num_refine+1];
      fprintf(mfp, "step %ld %d %d %d %d %d %d %d %d %d %d %d %d\n", calls,
              nb, max_active_parent, num_refine, refine_ghost,
              uniform_refine, mesh_size[0], mesh_size[1], mesh_size[2],
              x_block_size, y_block_size, z_block_size, num_objects);
      for (o = 0; o < num_objects; o++) {
         fprintf(mfp, "o %d", objects[o].type);
         for (d = 0; d < 3; d++)
            put_f64(mfp, objects[o].cen[d]);
         for (d = 0; d < 3; d++)
            put_f64(mfp, objects[o].size[d]);
         fprintf(mfp, "\n");
      }
      for (in = 0; in < nb; in++) {
         int n = sorted_list[in].n;
         block *bp = &blocks[n];
         fprintf(mfp, "b %d %d %d %d %d %d", n, bp->level, (int) bp->parent,
                 bp->cen[0], bp->cen[1], bp->cen[2]);
         for (l = 0; l < 6; l++)
            fprintf(mfp, " %d", bp->nei_level[l]);
         for (l = 0; l < 6; l++)
            fprintf(mfp, " %d", bp->nei[l][0][0]);
         fprintf(mfp, " %d\n", bp->refine);
      }
      for (k = 0; k < max_active_parent; k++) {
         parent *pp = &parents[k];
         fprintf(mfp, "p %d %d", k, pp->number >= 0);
         for (o = 0; o < 8; o++)
            fprintf(mfp, " %d", (int) pp->child[o]);
         fprintf(mfp, " %d\n", pp->refine);
      }
      fflush(mfp);
      dumped++;
   }
   calls++;
   __real_split_blocks();
}
