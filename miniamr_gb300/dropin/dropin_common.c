/*
 * Context, upload and mesh synchronisation for the drop-in translation
 * units.  The reference allocates host arrays for every slot
 * (ref/main.c:429-450) and init() fills the initial blocks
 * (ref/init.c:484-495); the first call into the hot path after that copies
 * the active blocks into the device pool, which is authoritative from then
 * on.  The mesh (sorted_list order plus each block's neighbour table) is
 * rebuilt from the reference's globals on every hot-path call and re-sent
 * only when it differs from what the device holds.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>

#include "block.h"
#include "comm.h"
#include "proto.h"
#include "dropin.h"

static mamr_ctx *ctx;
static int uploaded;
static int mesh_dirty = 1;
static mamr_block *desc, *sent;
static int n_desc, n_sent, cap_desc;

/* Cache of the whole active pool for mamr_dropin_fetch(). */
static double *fetch_buf;
static int32_t *fetch_slot_pos;
static long fetch_generation = -1, generation;

void mamr_dropin_check(int rc, const char *where)
{
   if (rc != MAMR_OK) {
      printf("ERROR: %s: %s (status %d)\n", where, mamr_last_error(), rc);
      exit(-1);
   }
}

mamr_ctx *mamr_dropin_ctx(void)
{
   if (!ctx) {
      mamr_config cfg;
      const char *dt = getenv("MAMR_DTYPE");
      memset(&cfg, 0, sizeof(cfg));
      cfg.nx = x_block_size;
      cfg.ny = y_block_size;
      cfg.nz = z_block_size;
      cfg.num_vars = num_vars;
      cfg.max_blocks = max_num_blocks;
      cfg.stencil = stencil;
      cfg.code = code;
      cfg.permute = permute;
      cfg.dtype = (dt && !strcmp(dt, "fp32")) ? MAMR_FP32 : MAMR_FP64;
      if (num_pes != 1) {
         printf("ERROR: the GB300 back end runs one rank (num_pes %d)\n",
                num_pes);
         exit(-1);
      }
      mamr_dropin_check(mamr_create(&cfg, &ctx), "mamr_create");
      /* --stencil 0: the coefficients init() drew (ref/init.c:418-423) */
      if (stencil == 0)
         mamr_dropin_check(mamr_set_work_params(ctx, a1, a0, mat),
                           "mamr_set_work_params");
   }
   return ctx;
}

void mamr_dropin_mesh_changed(void)
{
   mesh_dirty = 1;
   generation++;
}

static void upload_initial(void)
{
   int nx2 = x_block_size + 2, ny2 = y_block_size + 2, nz2 = z_block_size + 2;
   int nact = sorted_index[num_refine+1], in, v, i, j;
   size_t bv = (size_t) nx2 * ny2 * nz2, off;
   int32_t *slots = (int32_t *) malloc(sizeof(int32_t) * (nact ? nact : 1));
   double *buf = (double *) malloc(sizeof(double) * bv * num_vars *
                                   (nact ? nact : 1));
   if (!slots || !buf) {
      printf("ERROR: drop-in upload: out of host memory\n");
      exit(-1);
   }
   for (in = 0; in < nact; in++) {
      int n = sorted_list[in].n;
      slots[in] = n;
      for (v = 0; v < num_vars; v++)
         for (i = 0; i < nx2; i++)
            for (j = 0; j < ny2; j++) {
               off = (((size_t) in * num_vars + v) * nx2 + i) * ny2 + j;
               memcpy(buf + off * nz2, blocks[n].array[v][i][j],
                      sizeof(double) * nz2);
            }
   }
   mamr_dropin_check(mamr_upload_blocks(ctx, slots, nact, buf),
                     "mamr_upload_blocks");
   free(slots);
   free(buf);
}

static void build_desc(void)
{
   int nact = sorted_index[num_refine+1], in, l, a, b;
   if (nact > cap_desc) {
      cap_desc = nact + nact / 2 + 16;
      desc = (mamr_block *) realloc(desc, sizeof(mamr_block) * cap_desc);
      sent = (mamr_block *) realloc(sent, sizeof(mamr_block) * cap_desc);
      if (!desc || !sent) {
         printf("ERROR: drop-in mesh: out of host memory\n");
         exit(-1);
      }
   }
   for (in = 0; in < nact; in++) {
      int n = sorted_list[in].n;
      block *bp = &blocks[n];
      mamr_block *d = &desc[in];
      d->slot = n;
      d->level = bp->level;
      for (l = 0; l < 6; l++) {
         d->nei_level[l] = bp->nei_level[l];
         for (a = 0; a < 2; a++)
            for (b = 0; b < 2; b++)
               d->nei[l][a][b] = bp->nei[l][a][b];
      }
   }
   n_desc = nact;
}

void mamr_dropin_sync_data(void)
{
   mamr_dropin_ctx();
   if (!uploaded) {
      upload_initial();
      uploaded = 1;
   }
   generation++;
}

void mamr_dropin_sync_state(void)
{
   mamr_dropin_sync_data();
   build_desc();
   if (mesh_dirty || n_desc != n_sent ||
       memcmp(desc, sent, sizeof(mamr_block) * n_desc)) {
      mamr_dropin_check(mamr_set_mesh(ctx, desc, n_desc), "mamr_set_mesh");
      memcpy(sent, desc, sizeof(mamr_block) * n_desc);
      n_sent = n_desc;
      mesh_dirty = 0;
   }
   generation++;
}

int mamr_dropin_fetch(int slot, int var, double *out)
{
   size_t bv = (size_t) (x_block_size + 2) * (y_block_size + 2) *
               (z_block_size + 2);
   if (!ctx || slot < 0 || slot >= max_num_blocks || var < 0 ||
       var >= num_vars)
      return -1;
   if (fetch_generation != generation) {
      int nact = sorted_index[num_refine+1], in;
      int32_t *slots = (int32_t *) malloc(sizeof(int32_t) * (nact ? nact : 1));
      free(fetch_buf);
      fetch_buf = (double *) malloc(sizeof(double) * bv * num_vars *
                                    (nact ? nact : 1));
      if (!fetch_slot_pos)
         fetch_slot_pos = (int32_t *) malloc(sizeof(int32_t) *
                                             max_num_blocks);
      if (!slots || !fetch_buf || !fetch_slot_pos)
         return -1;
      for (in = 0; in < max_num_blocks; in++)
         fetch_slot_pos[in] = -1;
      for (in = 0; in < nact; in++) {
         slots[in] = sorted_list[in].n;
         fetch_slot_pos[slots[in]] = in;
      }
      if (mamr_download_blocks(ctx, slots, nact, fetch_buf) != MAMR_OK) {
         free(slots);
         return -1;
      }
      free(slots);
      fetch_generation = generation;
   }
   if (fetch_slot_pos[slot] < 0)
      return -1;
   memcpy(out, fetch_buf + ((size_t) fetch_slot_pos[slot] * num_vars + var) *
               bv, sizeof(double) * bv);
   return 0;
}
