/*
 * amr_oracle.c -- CPU restatement of miniAMR's per-timestep hot path behind
 * the mamr_* C ABI (include/miniamr_gb300.h).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is
 * compared against; it is never linked into or called by the product path.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  Parity of this restatement with the reference itself is pinned by
 * running the reference's own driver over these functions
 * (oracle/_ref/miniamr_hybrid_oracle vs oracle/_ref/miniamr_ref:
 * tests/golden/make_golden.py, tests/test_host_cpu.py) and by the committed
 * golden logs (tests/test_oracle_golden.py).
 *
 * Every routine is a sequential restatement of the reference code it cites
 * (paths are inside the miniAMR repository).  Cells are held as doubles in
 * a dense [slot][var][nx+2][ny+2][nz+2] array.  In FP32 mode every stored
 * value is a float and every arithmetic result is rounded to float right
 * after the double operation (RF below); double rounding is exact for
 * +, -, *, / of floats because 53 >= 2*24+2.
 */
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "miniamr_gb300.h"
#include "work_formulas.h"
#define MAMR_MFN static inline
#include "mark_geometry.h"

struct mamr_ctx {
   mamr_config cfg;
   int X, Y, Z;            /* nx+2, ny+2, nz+2 */
   size_t bv;              /* cells per block-variable */
   int fp32;
   double *pool;           /* max_blocks * num_vars * bv */
   mamr_block *mesh;
   int32_t n_mesh;
   int32_t *slot_pos;      /* slot -> position in mesh, -1 if inactive */
   int64_t launches;       /* stays 0: the oracle launches nothing */
   mamr_work_par work;     /* --stencil 0 coefficients */
   int work_set;
};

static __thread char err_buf[256];

static int fail(int code, const char *fmt, ...)
{
   va_list ap;
   va_start(ap, fmt);
   vsnprintf(err_buf, sizeof(err_buf), fmt, ap);
   va_end(ap);
   return code;
}

const char *mamr_last_error(void) { return err_buf; }

/* How the AMR driver (miniamr_gb300/csrc/amr_driver.cpp, linked into this
 * library too) records its own failures. */
int mamr_driver_fail(int code, const char *msg)
{
   return fail(code, "%s", msg);
}

/* Round to the pool's precision. */
static inline double RF(const mamr_ctx *c, double x)
{
   return c->fp32 ? (double) (float) x : x;
}

static inline double *blk(const mamr_ctx *c, int slot, int var)
{
   return c->pool + ((size_t) slot * c->cfg.num_vars + var) * c->bv;
}

#define AT(p, i, j, k) (p)[((size_t) (i) * c->Y + (j)) * c->Z + (k)]

/* Per-cell formulas of the variable-work stencils (--stencil 0), shared
 * with the GB300 kernels; this file supplies the dense-layout accessor
 * and the loops (ref/stencil.c:147-983). */
typedef struct {
   const struct mamr_ctx *c;
   int slot;
} oracle_wview;
#define MAMR_WFN static inline
#define MAMR_WVIEW oracle_wview
#define MAMR_AT(w, v, i, j, k) \
   (((w)->c->pool + ((size_t) (w)->slot * (w)->c->cfg.num_vars + (v)) * \
     (w)->c->bv)[((size_t) (i) * (w)->c->Y + (j)) * (w)->c->Z + (k)])
#include "work_formulas.h"

int mamr_create(const mamr_config *cfg, mamr_ctx **out)
{
   mamr_ctx *c;
   int r;
   if (!cfg || !out)
      return fail(MAMR_EINVAL, "null argument");
   if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2 || cfg->nx % 2 ||
       cfg->ny % 2 || cfg->nz % 2)
      return fail(MAMR_EINVAL, "block sizes must be even and >= 2");
   if (cfg->num_vars < 1 || cfg->max_blocks < 1)
      return fail(MAMR_EINVAL, "num_vars and max_blocks must be >= 1");
   if (cfg->stencil != 0 && cfg->stencil != 7 && cfg->stencil != 27)
      return fail(MAMR_EUNSUP, "stencil %d not supported", cfg->stencil);
   if (cfg->stencil == 0 && cfg->dtype != MAMR_FP64)
      return fail(MAMR_EUNSUP, "stencil 0 runs on FP64 pools only");
   if (cfg->stencil == 0 &&
       (cfg->num_vars < 8 || cfg->num_vars / 4 > MAMR_WORK_MAX_MAT))
      return fail(MAMR_EINVAL, "stencil 0 needs 8 <= num_vars <= %d",
                  4 * MAMR_WORK_MAX_MAT + 3);
   if (cfg->code < 0 || cfg->code > 2)
      return fail(MAMR_EUNSUP, "code %d not supported", cfg->code);
   if (cfg->dtype != MAMR_FP64 && cfg->dtype != MAMR_FP32)
      return fail(MAMR_EINVAL, "bad dtype");
   for (r = 0; r < 7; r++)
      if (cfg->reserved[r])
         return fail(MAMR_EINVAL, "reserved fields must be zero");
   c = (mamr_ctx *) calloc(1, sizeof(*c));
   if (!c)
      return fail(MAMR_ENOMEM, "host allocation");
   c->cfg = *cfg;
   c->X = cfg->nx + 2;
   c->Y = cfg->ny + 2;
   c->Z = cfg->nz + 2;
   c->bv = (size_t) c->X * c->Y * c->Z;
   c->fp32 = cfg->dtype == MAMR_FP32;
   /* zero-filled, never cleared: ref/main.c:429-450 fresh heap */
   c->pool = (double *) calloc((size_t) cfg->max_blocks * cfg->num_vars *
                               c->bv, sizeof(double));
   if (!c->pool) {
      free(c);
      return fail(MAMR_ENOMEM, "host pool allocation");
   }
   *out = c;
   return MAMR_OK;
}

int mamr_destroy(mamr_ctx *c)
{
   if (!c)
      return MAMR_OK;
   free(c->pool);
   free(c->mesh);
   free(c->slot_pos);
   free(c);
   return MAMR_OK;
}

int mamr_stream(mamr_ctx *c, void **stream)
{
   if (!c || !stream)
      return fail(MAMR_EINVAL, "null argument");
   *stream = NULL;
   return MAMR_OK;
}

int mamr_sync(mamr_ctx *c)
{
   return c ? MAMR_OK : fail(MAMR_EINVAL, "null context");
}

int mamr_launch_count(mamr_ctx *c, int64_t *count)
{
   if (!c || !count)
      return fail(MAMR_EINVAL, "null argument");
   *count = c->launches;
   return MAMR_OK;
}

/* The oracle has no launch shapes: the setting is accepted and ignored,
 * and no choice is ever reported. */
int mamr_set_tuning(mamr_ctx *c, int32_t choice)
{
   (void) choice;
   return c ? MAMR_OK : fail(MAMR_EINVAL, "null context");
}

int mamr_get_tuning(const mamr_ctx *c, int32_t *choice,
                    int32_t *n_candidates, int32_t *shape)
{
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (choice)
      *choice = -1;
   if (n_candidates)
      *n_candidates = 0;
   if (shape)
      for (int q = 0; q < 5; q++)
         shape[q] = 0;
   return MAMR_OK;
}

static int check_slot(const mamr_ctx *c, int32_t s)
{
   return s >= 0 && s < c->cfg.max_blocks;
}

int mamr_upload_blocks(mamr_ctx *c, const int32_t *slots, int32_t n,
                       const double *host)
{
   int32_t b;
   int v;
   size_t q;
   if (!c || (n && (!slots || !host)) || n < 0)
      return fail(MAMR_EINVAL, "bad upload arguments");
   for (b = 0; b < n; b++)
      if (!check_slot(c, slots[b]))
         return fail(MAMR_EINVAL, "slot %d out of range", slots[b]);
   for (b = 0; b < n; b++)
      for (v = 0; v < c->cfg.num_vars; v++) {
         double *d = blk(c, slots[b], v);
         const double *s = host + ((size_t) b * c->cfg.num_vars + v) * c->bv;
         for (q = 0; q < c->bv; q++)
            d[q] = RF(c, s[q]);
      }
   return MAMR_OK;
}

int mamr_download_blocks(mamr_ctx *c, const int32_t *slots, int32_t n,
                         double *host)
{
   int32_t b;
   int v;
   if (!c || (n && (!slots || !host)) || n < 0)
      return fail(MAMR_EINVAL, "bad download arguments");
   for (b = 0; b < n; b++)
      if (!check_slot(c, slots[b]))
         return fail(MAMR_EINVAL, "slot %d out of range", slots[b]);
   for (b = 0; b < n; b++)
      for (v = 0; v < c->cfg.num_vars; v++)
         memcpy(host + ((size_t) b * c->cfg.num_vars + v) * c->bv,
                blk(c, slots[b], v), c->bv * sizeof(double));
   return MAMR_OK;
}

int mamr_set_mesh(mamr_ctx *c, const mamr_block *blocks, int32_t n)
{
   int32_t b;
   int l, i, j;
   mamr_block *m;
   if (!c || n < 0 || (n && !blocks))
      return fail(MAMR_EINVAL, "bad mesh arguments");
   for (b = 0; b < n; b++) {
      const mamr_block *bp = &blocks[b];
      if (!check_slot(c, bp->slot))
         return fail(MAMR_EINVAL, "block %d: slot %d out of range", b,
                     bp->slot);
      for (l = 0; l < 6; l++) {
         int nl = bp->nei_level[l];
         if (nl == -2)
            continue;
         if (nl != bp->level && nl != bp->level + 1 && nl != bp->level - 1)
            return fail(MAMR_EMESH, "misconnected block (slot %d face %d)",
                        bp->slot, l);
         for (i = 0; i < 2; i++)
            for (j = 0; j < 2; j++)
               if ((nl == bp->level + 1 || (i == 0 && j == 0)) &&
                   !check_slot(c, bp->nei[l][i][j]))
                  return fail(MAMR_EMESH,
                              "misconnected block (slot %d face %d nei %d)",
                              bp->slot, l, bp->nei[l][i][j]);
      }
   }
   /* every listed neighbour must be active (the library checks the same) */
   {
      unsigned char *act = (unsigned char *) calloc((size_t) c->cfg.max_blocks,
                                                    1);
      int bad = -1;
      if (!act)
         return fail(MAMR_ENOMEM, "host allocation");
      for (b = 0; b < n; b++)
         act[blocks[b].slot] = 1;
      for (b = 0; b < n && bad < 0; b++)
         for (l = 0; l < 6; l++) {
            const mamr_block *bp = &blocks[b];
            const int nl = bp->nei_level[l];
            if (nl == -2)
               continue;
            for (i = 0; i < 2; i++)
               for (j = 0; j < 2; j++)
                  if ((nl == bp->level + 1 || (i == 0 && j == 0)) &&
                      !act[bp->nei[l][i][j]])
                     bad = bp->nei[l][i][j];
         }
      free(act);
      if (bad >= 0)
         return fail(MAMR_EMESH, "neighbour slot %d not active", bad);
   }
   m = (mamr_block *) malloc(sizeof(mamr_block) * (n ? n : 1));
   if (!m)
      return fail(MAMR_ENOMEM, "host allocation");
   if (!c->slot_pos) {
      c->slot_pos = (int32_t *) malloc(sizeof(int32_t) * c->cfg.max_blocks);
      if (!c->slot_pos) {
         free(m);
         return fail(MAMR_ENOMEM, "host allocation");
      }
   }
   memcpy(m, blocks, sizeof(mamr_block) * n);
   free(c->mesh);
   c->mesh = m;
   c->n_mesh = n;
   for (b = 0; b < c->cfg.max_blocks; b++)
      c->slot_pos[b] = -1;
   for (b = 0; b < n; b++)
      c->slot_pos[m[b].slot] = b;
   return MAMR_OK;
}

/* ref/comm.c:1465-1534 (code 0): same-level exchange across face l between
 * blocks n and n1, variables [start, start+num). */
static void on_proc_comm(mamr_ctx *c, int n, int n1, int l, int start,
                         int num)
{
   int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz, m, i, j, k;
   int is, ie, js, je, lo, hi;
   /* l even: bp = n, bp1 = n1; l odd: swapped */
   lo = (l % 2 == 0) ? n : n1;   /* bp  */
   hi = (l % 2 == 0) ? n1 : n;   /* bp1 */
   for (m = start; m < start + num; m++) {
      double *bp = blk(c, lo, m), *bp1 = blk(c, hi, m);
      /* code 1/2 (ref/comm.c:1535-1579): every plane whole */
      const int all = c->cfg.code != 0;
      if (l / 2 == 0) {
         js = all ? 0 : 1; je = all ? ny + 1 : ny;
         for (j = js; j <= je; j++)
            for (k = js ? 1 : 0; k <= (all ? nz + 1 : nz); k++) {
               AT(bp1, nx + 1, j, k) = AT(bp, 1, j, k);
               AT(bp, 0, j, k) = AT(bp1, nx, j, k);
            }
      } else if (l / 2 == 1) {
         if (c->cfg.stencil == 7 && !all) { is = 1; ie = nx; }
         else { is = 0; ie = nx + 1; }
         for (i = is; i <= ie; i++)
            for (k = all ? 0 : 1; k <= (all ? nz + 1 : nz); k++) {
               AT(bp1, i, ny + 1, k) = AT(bp, i, 1, k);
               AT(bp, i, 0, k) = AT(bp1, i, ny, k);
            }
      } else {
         if (c->cfg.stencil == 7 && !all) { is = 1; ie = nx; js = 1; je = ny; }
         else { is = 0; ie = nx + 1; js = 0; je = ny + 1; }
         for (i = is; i <= ie; i++)
            for (j = js; j <= je; j++) {
               AT(bp1, i, j, nz + 1) = AT(bp, i, j, 1);
               AT(bp, i, j, 0) = AT(bp1, i, j, nz);
            }
      }
   }
}

/* Cell (nc, a, b) of a face normal to dir: tangential (a, b) are (j, k)
 * for x faces, (i, k) for y faces, (i, j) for z faces. */
static double *face_at(const mamr_ctx *c, double *p, int dir, int nc, int a,
                       int b)
{
   if (dir == 0)
      return &AT(p, nc, a, b);
   if (dir == 1)
      return &AT(p, a, nc, b);
   return &AT(p, a, b, nc);
}

/* ref/comm.c:1689-1907 (code 1/2: ghosts transferred whole), one
 * direction-generic form of the reference's three branches.  Block n is
 * coarse, n1 fine, (iq, jq) the quarter of n's face l: the fine ghost
 * plane gets coarse/4 over its whole (na+2) x (nb+2) extent (tangential
 * index A maps to coarse offset + A=0 -> 0, A=na+1 -> na/2+1, else
 * (A+1)/2); the coarse ghost plane gets the quarter's 2x2 sums, the pair
 * sums of the fine ghost row and column on the jq and iq sides, and one
 * corner copied. */
static void comm_diff_all(mamr_ctx *c, int n, int n1, int l, int iq, int jq,
                          int start, int num)
{
   const int dir = l / 2;
   const int nn = dir == 0 ? c->cfg.nx : (dir == 1 ? c->cfg.ny : c->cfg.nz);
   const int na = dir == 0 ? c->cfg.ny : c->cfg.nx;
   const int nb = dir == 2 ? c->cfg.ny : c->cfg.nz;
   const int ha = na / 2, hb = nb / 2, oa = jq * ha, ob = iq * hb;
   const int c0 = (l % 2 == 0) ? 0 : nn + 1, c1 = (l % 2 == 0) ? 1 : nn;
   const int f2 = (l % 2 == 0) ? nn + 1 : 0, f3 = (l % 2 == 0) ? nn : 1;
   const int ae = jq ? na + 1 : 0, be = iq ? nb + 1 : 0;  /* edge sides */
   int m, A, B, a, b;
   for (m = start; m < start + num; m++) {
      double *C = blk(c, n, m), *F = blk(c, n1, m);
      for (A = 0; A <= na + 1; A++)
         for (B = 0; B <= nb + 1; B++) {
            int ca = A == 0 ? oa : (A == na + 1 ? ha + 1 + oa : (A + 1) / 2 + oa);
            int cb = B == 0 ? ob : (B == nb + 1 ? hb + 1 + ob : (B + 1) / 2 + ob);
            *face_at(c, F, dir, f2, A, B) =
               RF(c, *face_at(c, C, dir, c1, ca, cb) / 4.0);
         }
      *face_at(c, C, dir, c0, ae, be) = *face_at(c, F, dir, f3, ae, be);
      for (b = 1; b <= hb; b++)
         *face_at(c, C, dir, c0, ae, b + ob) =
            RF(c, *face_at(c, F, dir, f3, ae, 2*b - 1) +
                  *face_at(c, F, dir, f3, ae, 2*b));
      for (a = 1; a <= ha; a++) {
         *face_at(c, C, dir, c0, a + oa, be) =
            RF(c, *face_at(c, F, dir, f3, 2*a - 1, be) +
                  *face_at(c, F, dir, f3, 2*a, be));
         for (b = 1; b <= hb; b++)
            *face_at(c, C, dir, c0, a + oa, b + ob) =
               RF(c, RF(c, RF(c, *face_at(c, F, dir, f3, 2*a - 1, 2*b - 1) +
                                 *face_at(c, F, dir, f3, 2*a - 1, 2*b)) +
                          *face_at(c, F, dir, f3, 2*a, 2*b - 1)) +
                     *face_at(c, F, dir, f3, 2*a, 2*b));
      }
   }
}

/* ref/comm.c:1585-1688 (code 0): block n (coarse) and n1 (fine) across
 * face l of n, quarter (iq, jq) of n's face.  Fine ghosts get coarse/4,
 * the coarse ghost gets the left-to-right sum of the 2x2 fine cells. */
static void on_proc_comm_diff(mamr_ctx *c, int n, int n1, int l, int iq,
                              int jq, int start, int num)
{
   int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz;
   int xh = nx / 2, yh = ny / 2, zh = nz / 2, m, i, j, k;
   int a0, a1, a2, a3, o1, o2;
   if (c->cfg.code != 0) {
      comm_diff_all(c, n, n1, l, iq, jq, start, num);
      return;
   }
   for (m = start; m < start + num; m++) {
      double *bp = blk(c, n, m), *bp1 = blk(c, n1, m);
      if (l / 2 == 0) {
         if (l == 0) { a0 = 0; a1 = 1; a2 = nx + 1; a3 = nx; }
         else { a0 = nx + 1; a1 = nx; a2 = 0; a3 = 1; }
         o1 = jq * yh;   /* j offset */
         o2 = iq * zh;   /* k offset */
         for (j = 1; j <= yh; j++)
            for (k = 1; k <= zh; k++) {
               double q = RF(c, AT(bp, a1, j + o1, k + o2) / 4.0);
               AT(bp1, a2, 2*j - 1, 2*k - 1) = q;
               AT(bp1, a2, 2*j - 1, 2*k) = q;
               AT(bp1, a2, 2*j, 2*k - 1) = q;
               AT(bp1, a2, 2*j, 2*k) = q;
               AT(bp, a0, j + o1, k + o2) =
                  RF(c, RF(c, RF(c, AT(bp1, a3, 2*j - 1, 2*k - 1) +
                                    AT(bp1, a3, 2*j - 1, 2*k)) +
                             AT(bp1, a3, 2*j, 2*k - 1)) +
                        AT(bp1, a3, 2*j, 2*k));
            }
      } else if (l / 2 == 1) {
         if (l == 2) { a0 = 0; a1 = 1; a2 = ny + 1; a3 = ny; }
         else { a0 = ny + 1; a1 = ny; a2 = 0; a3 = 1; }
         o1 = jq * xh;   /* i offset */
         o2 = iq * zh;   /* k offset */
         for (i = 1; i <= xh; i++)
            for (k = 1; k <= zh; k++) {
               double q = RF(c, AT(bp, i + o1, a1, k + o2) / 4.0);
               AT(bp1, 2*i - 1, a2, 2*k - 1) = q;
               AT(bp1, 2*i - 1, a2, 2*k) = q;
               AT(bp1, 2*i, a2, 2*k - 1) = q;
               AT(bp1, 2*i, a2, 2*k) = q;
               AT(bp, i + o1, a0, k + o2) =
                  RF(c, RF(c, RF(c, AT(bp1, 2*i - 1, a3, 2*k - 1) +
                                    AT(bp1, 2*i - 1, a3, 2*k)) +
                             AT(bp1, 2*i, a3, 2*k - 1)) +
                        AT(bp1, 2*i, a3, 2*k));
            }
      } else {
         if (l == 4) { a0 = 0; a1 = 1; a2 = nz + 1; a3 = nz; }
         else { a0 = nz + 1; a1 = nz; a2 = 0; a3 = 1; }
         o1 = jq * xh;   /* i offset */
         o2 = iq * yh;   /* j offset */
         for (i = 1; i <= xh; i++)
            for (j = 1; j <= yh; j++) {
               double q = RF(c, AT(bp, i + o1, j + o2, a1) / 4.0);
               AT(bp1, 2*i - 1, 2*j - 1, a2) = q;
               AT(bp1, 2*i - 1, 2*j, a2) = q;
               AT(bp1, 2*i, 2*j - 1, a2) = q;
               AT(bp1, 2*i, 2*j, a2) = q;
               AT(bp, i + o1, j + o2, a0) =
                  RF(c, RF(c, RF(c, AT(bp1, 2*i - 1, 2*j - 1, a3) +
                                    AT(bp1, 2*i - 1, 2*j, a3)) +
                             AT(bp1, 2*i, 2*j - 1, a3)) +
                        AT(bp1, 2*i, 2*j, a3));
            }
      }
   }
}

/* ref/comm.c:1911-1965: reflective copy of the plane next to face l into
 * its ghost plane; interior tangential range when code==0 && stencil==7,
 * full 0..n+1 otherwise. */
static void apply_bc(mamr_ctx *c, int l, int n, int start, int num)
{
   int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz, var, i, j, k, t, f;
   int full = !(c->cfg.code == 0 && c->cfg.stencil == 7);
   int lo0 = full ? 0 : 1;
   for (var = start; var < start + num; var++) {
      double *bp = blk(c, n, var);
      if (l / 2 == 0) {
         t = (l == 1) ? nx + 1 : 0;
         f = (l == 1) ? nx : 1;
         for (j = lo0; j <= (full ? ny + 1 : ny); j++)
            for (k = lo0; k <= (full ? nz + 1 : nz); k++)
               AT(bp, t, j, k) = AT(bp, f, j, k);
      } else if (l / 2 == 1) {
         t = (l == 3) ? ny + 1 : 0;
         f = (l == 3) ? ny : 1;
         for (i = lo0; i <= (full ? nx + 1 : nx); i++)
            for (k = lo0; k <= (full ? nz + 1 : nz); k++)
               AT(bp, i, t, k) = AT(bp, i, f, k);
      } else {
         t = (l == 5) ? nz + 1 : 0;
         f = (l == 5) ? nz : 1;
         for (i = lo0; i <= (full ? nx + 1 : nx); i++)
            for (j = lo0; j <= (full ? ny + 1 : ny); j++)
               AT(bp, i, j, t) = AT(bp, i, j, f);
      }
   }
}

static const int permutations[6][3] = { {0, 1, 2}, {1, 2, 0}, {2, 0, 1},
                                        {0, 2, 1}, {1, 0, 2}, {2, 1, 0} };

/* ref/comm.c:42-56,162-203: the on-rank part of comm() on one rank.
 * Within one direction every ghost cell is written by exactly one face
 * exchange and only planes that direction does not write are read, so the
 * blocks of a direction may be visited in any order or concurrently
 * (the reference's OpenMP variant threads this loop, openmp/comm.c:166). */
static int comm_block(mamr_ctx *c, int in, int dir, int start, int num)
{
   const mamr_block *bp = &c->mesh[in];
   int n = bp->slot, l, i, j, k, m;
   for (l = dir * 2; l < dir * 2 + 2; l++) {
      if (bp->nei_level[l] == bp->level) {
         if ((m = bp->nei[l][0][0]) > n)
            on_proc_comm(c, n, m, l, start, num);
      } else if (bp->nei_level[l] == bp->level + 1) {
         for (i = 0; i < 2; i++)
            for (j = 0; j < 2; j++)
               if ((m = bp->nei[l][i][j]) > n)
                  on_proc_comm_diff(c, n, m, l, i, j, start, num);
      } else if (bp->nei_level[l] == bp->level - 1) {
         if ((m = bp->nei[l][0][0]) > n) {
            /* blocks[m]: the coarse neighbour's record */
            const mamr_block *mb = c->slot_pos[m] >= 0 ?
                                   &c->mesh[c->slot_pos[m]] : NULL;
            if (!mb)
               return MAMR_EMESH;
            k = dir * 2 + 1 - l % 2;
            for (i = 0; i < 2; i++)
               for (j = 0; j < 2; j++)
                  if (mb->nei[k][i][j] == n)
                     on_proc_comm_diff(c, m, n, k, i, j, start, num);
         }
      } else if (bp->nei_level[l] == -2) {
         apply_bc(c, l, n, start, num);
      } else {
         return MAMR_EMESH;
      }
   }
   return MAMR_OK;
}

int mamr_comm(mamr_ctx *c, int32_t start, int32_t num, int32_t stage)
{
   int o, dir, in, bad = 0;
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (start < 0 || num < 0 || start + num > c->cfg.num_vars)
      return fail(MAMR_EINVAL, "variable range out of bounds");
   for (o = 0; o < 3; o++) {
      dir = c->cfg.permute ? permutations[stage % 6][o] : o;
#pragma omp parallel for schedule(dynamic, 4) reduction(|:bad)
      for (in = 0; in < c->n_mesh; in++)
         bad |= comm_block(c, in, dir, start, num) != MAMR_OK;
      if (bad)
         return fail(MAMR_EMESH, "misconnected block");
   }
   return MAMR_OK;
}

/* Rounds to the pool's precision where f32 is a compile-time constant (the
 * stencil and checksum loops below are instantiated once per precision, so
 * the FP64 loops carry no test and vectorise along k). */
#define RND(f32, x) ((f32) ? (double) (float) (x) : (x))
#define ORACLE_INLINE static inline __attribute__((always_inline))

/* ref/stencil.c:82-101: the 7-point average of interior plane i into out
 * (rows of nz values, row j at (j-1)*nz), in the reference's term order. */
ORACLE_INLINE void stencil7_plane(const mamr_ctx *c, const double *a, int i,
                                  double *out, const int f32)
{
   const int ny = c->cfg.ny, nz = c->cfg.nz;
   const ptrdiff_t sy = c->Z, sx = (ptrdiff_t) c->Y * c->Z;
   int j, k;
   for (j = 1; j <= ny; j++) {
      const double *p = a + i * sx + j * sy;
      double *o = out + (size_t) (j - 1) * nz - 1;
      for (k = 1; k <= nz; k++) {
         double s = RND(f32, p[k - sx] + p[k - sy]);
         s = RND(f32, s + p[k - 1]);
         s = RND(f32, s + p[k]);
         s = RND(f32, s + p[k + 1]);
         s = RND(f32, s + p[k + sy]);
         s = RND(f32, s + p[k + sx]);
         o[k] = RND(f32, s / 7.0);
      }
   }
}

/* The 9-term sum of ref/stencil.c:108-134 for every interior (j, k) of
 * plane p (sb, sm or sf of the cells whose i-1, i or i+1 plane it is),
 * left to right over (j-1, k-1) .. (j+1, k+1). */
ORACLE_INLINE void plane_sums9(const mamr_ctx *c, const double *a, int p,
                               double *out, const int f32)
{
   const int ny = c->cfg.ny, nz = c->cfg.nz;
   const ptrdiff_t sy = c->Z, sx = (ptrdiff_t) c->Y * c->Z;
   int j, k;
   for (j = 1; j <= ny; j++) {
      const double *r0 = a + p * sx + (j - 1) * sy, *r1 = r0 + sy,
                   *r2 = r1 + sy;
      double *o = out + (size_t) (j - 1) * nz - 1;
      for (k = 1; k <= nz; k++) {
         double t = RND(f32, r0[k - 1] + r0[k]);
         t = RND(f32, t + r0[k + 1]);
         t = RND(f32, t + r1[k - 1]);
         t = RND(f32, t + r1[k]);
         t = RND(f32, t + r1[k + 1]);
         t = RND(f32, t + r2[k - 1]);
         t = RND(f32, t + r2[k]);
         o[k] = RND(f32, t + r2[k + 1]);
      }
   }
}

/* Copies rows of nz values (row j at (j-1)*nz) into interior plane i. */
static void store_plane(const mamr_ctx *c, double *a, int i, const double *in)
{
   const int ny = c->cfg.ny, nz = c->cfg.nz;
   int j;
   for (j = 1; j <= ny; j++)
      memcpy(&AT(a, i, j, 1), in + (size_t) (j - 1) * nz,
             sizeof(double) * nz);
}

/* ref/stencil.c:76-145 (stencil_calc), Jacobi update of one block-variable.
 * Each output plane is written back as soon as no later plane reads its
 * old values (the reference's work array holds the whole block): 7-point,
 * plane i-1 after plane i is computed; 27-point, plane i as soon as the
 * sums of plane i+1 exist -- each 9-term plane sum is formed once and used
 * by the three cells that need it, the same additions in the same order.
 * scratch holds 3 * ny * nz doubles. */
ORACLE_INLINE void stencil_block_t(const mamr_ctx *c, int st, double *a,
                                   double *scratch, const int f32)
{
   const int nx = c->cfg.nx;
   const size_t pl = (size_t) c->cfg.ny * c->cfg.nz;
   int i;
   size_t q;
   if (st == 7) {
      double *buf[2] = {scratch, scratch + pl};
      for (i = 1; i <= nx; i++) {
         stencil7_plane(c, a, i, buf[i & 1], f32);
         if (i > 1)
            store_plane(c, a, i - 1, buf[(i - 1) & 1]);
      }
      store_plane(c, a, nx, buf[nx & 1]);
      return;
   }
   double *s0 = scratch, *s1 = scratch + pl, *s2 = scratch + 2 * pl, *t;
   plane_sums9(c, a, 0, s0, f32);
   plane_sums9(c, a, 1, s1, f32);
   for (i = 1; i <= nx; i++) {
      plane_sums9(c, a, i + 1, s2, f32);
      /* plane i's old values are no longer read: overwrite them */
      for (q = 0; q < pl; q++)
         s0[q] = RND(f32, RND(f32, RND(f32, s0[q] + s1[q]) + s2[q]) / 27.0);
      store_plane(c, a, i, s0);
      t = s0; s0 = s1; s1 = s2; s2 = t;
   }
}

static void stencil_block(mamr_ctx *c, int st, double *a, double *scratch)
{
   if (c->fp32)
      stencil_block_t(c, st, a, scratch, 1);
   else
      stencil_block_t(c, st, a, scratch, 0);
}

/* ref/stencil.c:76-145 (stencil_calc), Jacobi update of every active
 * block's interior for one variable; blocks are independent (threaded over
 * blocks as in openmp/stencil.c:84,107). */
/* The variable-work branch of stencil_driver (ref/stencil.c:51-71) for
 * one block: the kernel of calc_stage % 6 in the reference's loop order,
 * then stencil_check. */
static void work_block(mamr_ctx *c, int slot, int var, int calc_stage,
                       double *work)
{
   int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz, i, j, k;
   oracle_wview w;
   double *a = blk(c, slot, var);
   w.c = c;
   w.slot = slot;
   switch (calc_stage % 6) {
   case 0:
      for (i = 1; i <= nx; i++)
         for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++)
               AT(a, i, j, k) = mamr_w_stencil0(&w, var, i, j, k, &c->work);
      break;
   case 1:
   case 2:
   case 3:
      /* stencil_x/y/z update in place as the i, j, k loops advance */
      for (i = 1; i <= nx; i++)
         for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++)
               AT(a, i, j, k) = mamr_w_line(&w, var, calc_stage % 6 - 1, i,
                                            j, k, &c->work);
      break;
   default:
      for (i = 1; i <= nx; i++)
         for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++)
               AT(work, i, j, k) =
                  calc_stage % 6 == 4
                     ? mamr_w_seven(&w, var, i, j, k, &c->work)
                     : mamr_w_twentyseven(&w, var, i, j, k, &c->work);
      for (i = 1; i <= nx; i++)
         for (j = 1; j <= ny; j++)
            for (k = 1; k <= nz; k++)
               AT(a, i, j, k) = AT(work, i, j, k);
      break;
   }
   for (i = 1; i <= nx; i++)
      for (j = 1; j <= ny; j++)
         for (k = 1; k <= nz; k++)
            AT(a, i, j, k) = mamr_w_check(AT(a, i, j, k), &c->work);
}

int mamr_set_work_params(mamr_ctx *c, double a1, const double *a0,
                         int32_t n_a0)
{
   int q;
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (c->cfg.stencil != 0)
      return fail(MAMR_EINVAL, "work parameters belong to stencil 0");
   if (!a0 || n_a0 != c->cfg.num_vars / 4)
      return fail(MAMR_EINVAL, "a0 must hold num_vars/4 = %d values",
                  c->cfg.num_vars / 4);
   c->work.mat = n_a0;
   c->work.a1 = a1;
   for (q = 0; q < n_a0; q++)
      c->work.a0[q] = a0[q];
   c->work_set = 1;
   return MAMR_OK;
}

int mamr_stencil(mamr_ctx *c, int32_t var, int32_t calc_stage)
{
   int bad = 0, st, varwork;
   if (!c)
      return fail(MAMR_EINVAL, "null context");
   if (var < 0 || var >= c->cfg.num_vars)
      return fail(MAMR_EINVAL, "variable out of range");
   if (calc_stage < 0)
      return fail(MAMR_EINVAL, "negative calc_stage");
   /* stencil_driver (ref/stencil.c:43-74) */
   st = c->cfg.stencil ? c->cfg.stencil : 7;
   varwork = c->cfg.stencil == 0 && var != 0 && var < 4 * (c->cfg.num_vars / 4);
   if (varwork && !c->work_set)
      return fail(MAMR_EINVAL, "stencil 0 needs mamr_set_work_params before "
                  "the first stencil");
#pragma omp parallel reduction(|:bad)
   {
      /* the variable-work kernels' block-sized work array, or the plain
         stencil's three planes */
      double *work = (double *) malloc(sizeof(double) *
                                       (c->bv > 3 * (size_t) c->cfg.ny *
                                                    c->cfg.nz
                                           ? c->bv
                                           : 3 * (size_t) c->cfg.ny *
                                                c->cfg.nz));
      int in;
      if (!work)
         bad = 1;
#pragma omp for schedule(dynamic, 4)
      for (in = 0; in < c->n_mesh; in++)
         if (work) {
            if (varwork)
               work_block(c, c->mesh[in].slot, var, calc_stage, work);
            else
               stencil_block(c, st, blk(c, c->mesh[in].slot, var), work);
         }
      free(work);
   }
   if (bad)
      return fail(MAMR_ENOMEM, "host allocation");
   return MAMR_OK;
}

/* FP32 checksum unit: each cell truncated toward zero to a multiple of
 * 2^-52, accumulated exactly in 128 bits.  Returns 0 on success, -1 when a
 * cell is outside the exact window v == 0 or 2^-52 <= |v| < 2^10 (too
 * large or not finite for the accumulator, or too small to register). */
static int fixed_cell(double v, int64_t *out)
{
   const double a = fabs(v);
   if (!(a < 1024.0 && (a >= 0x1p-52 || a == 0.0))) {
      *out = 0;
      return -1;
   }
   *out = (int64_t) (v * 0x1p52);
   return 0;
}

/* Neumaier-compensated FP64 step: adds x to the running sum s with its
 * correction c; once the sum is not finite the correction is left alone,
 * so an infinite cell gives an infinite sum as plain summation does. */
static void neumaier(double *s, double *c, double x)
{
   const double t = *s + x;
   if (isfinite(t)) {
      if (fabs(*s) >= fabs(x))
         *c += (*s - t) + x;
      else
         *c += (x - t) + *s;
   }
   *s = t;
}

/* The FP32 checksum of a variable with a cell outside the fixed-point
 * window: the reference's order (ref/check_sum.c:44-53) in FP64 with
 * Neumaier compensation -- each block serially (k fastest) into s + c,
 * then the block values serially in sorted order, S + C. */
static int fp32_fallback_sum(const mamr_ctx *c, int var, double *sum)
{
   double S = 0.0, C = 0.0, *bs = (double *) malloc(sizeof(double) *
                                                    (c->n_mesh ? c->n_mesh
                                                               : 1));
   int in;
   if (!bs)
      return fail(MAMR_ENOMEM, "host allocation");
#pragma omp parallel for schedule(dynamic, 8)
   for (in = 0; in < c->n_mesh; in++) {
      const double *a = blk(c, c->mesh[in].slot, var);
      double s = 0.0, cc = 0.0;
      int i, j, k;
      for (i = 1; i <= c->cfg.nx; i++)
         for (j = 1; j <= c->cfg.ny; j++)
            for (k = 1; k <= c->cfg.nz; k++)
               neumaier(&s, &cc, AT(a, i, j, k));
      bs[in] = s + cc;
   }
   for (in = 0; in < c->n_mesh; in++)
      neumaier(&S, &C, bs[in]);
   free(bs);
   *sum = S + C;
   return MAMR_OK;
}

static double fixed128_to_double(__int128 acc)
{
   return (double) acc * 0x1p-52;
}

/* ref/check_sum.c:36-65.  Block sums may be formed concurrently; they are
 * added serially in sorted_list order. */
int mamr_check_sum(mamr_ctx *c, int32_t var, double *sum)
{
   int in, bad = 0;
   if (!c || !sum)
      return fail(MAMR_EINVAL, "null argument");
   if (var < 0 || var >= c->cfg.num_vars)
      return fail(MAMR_EINVAL, "variable out of range");
   if (!c->fp32) {
      double s = 0.0, *bs = (double *) malloc(sizeof(double) *
                                              (c->n_mesh ? c->n_mesh : 1));
      if (!bs)
         return fail(MAMR_ENOMEM, "host allocation");
      /* four blocks' serial sums side by side (independent chains in
         flight; each block's additions in the reference's order) */
#pragma omp parallel for schedule(dynamic, 2)
      for (in = 0; in < c->n_mesh; in += 4) {
         const double *a[4];
         double t[4] = {0.0, 0.0, 0.0, 0.0};
         int i, j, k, q, m = c->n_mesh - in < 4 ? c->n_mesh - in : 4;
         for (q = 0; q < 4; q++)
            a[q] = blk(c, c->mesh[in + (q < m ? q : 0)].slot, var);
         for (i = 1; i <= c->cfg.nx; i++)
            for (j = 1; j <= c->cfg.ny; j++) {
               const size_t r = ((size_t) i * c->Y + j) * c->Z;
               for (k = 1; k <= c->cfg.nz; k++) {
                  t[0] += a[0][r + k];
                  t[1] += a[1][r + k];
                  t[2] += a[2][r + k];
                  t[3] += a[3][r + k];
               }
            }
         for (q = 0; q < m; q++)
            bs[in + q] = t[q];
      }
      for (in = 0; in < c->n_mesh; in++)
         s += bs[in];
      free(bs);
      *sum = s;
   } else {
      __int128 acc = 0, *bs = (__int128 *) malloc(sizeof(__int128) *
                                                 (c->n_mesh ? c->n_mesh : 1));
      if (!bs)
         return fail(MAMR_ENOMEM, "host allocation");
#pragma omp parallel for schedule(dynamic, 8) reduction(|:bad)
      for (in = 0; in < c->n_mesh; in++) {
         const double *a = blk(c, c->mesh[in].slot, var);
         __int128 t = 0;
         int i, j, k;
         for (i = 1; i <= c->cfg.nx; i++)
            for (j = 1; j <= c->cfg.ny; j++)
               for (k = 1; k <= c->cfg.nz; k++) {
                  int64_t q;
                  if (fixed_cell(AT(a, i, j, k), &q))
                     bad = 1;
                  t += q;
               }
         bs[in] = t;
      }
      for (in = 0; in < c->n_mesh; in++)
         acc += bs[in];
      free(bs);
      if (bad)
         return fp32_fallback_sum(c, var, sum);
      *sum = fixed128_to_double(acc);
   }
   return MAMR_OK;
}

/* ref/block.c:158-173: each child octant's interior is its parent's
 * matching half-block, each parent cell replicated 2x2x2 and divided by 8
 * (exact).  Child ghost cells keep the slot's previous contents. */
int mamr_split(mamr_ctx *c, const mamr_split_job *jobs, int32_t n)
{
   int32_t t;
   int o, v, i, j, k, i2, j2, k2;
   if (!c || n < 0 || (n && !jobs))
      return fail(MAMR_EINVAL, "bad split arguments");
   for (t = 0; t < n; t++) {
      if (!check_slot(c, jobs[t].parent))
         return fail(MAMR_EINVAL, "split parent slot out of range");
      for (o = 0; o < 8; o++)
         if (!check_slot(c, jobs[t].child[o]))
            return fail(MAMR_EINVAL, "split child slot out of range");
   }
   for (t = 0; t < n; t++)
      for (o = 0; o < 8; o++) {
         int i1 = (o % 2) * (c->cfg.nx / 2), j1 = ((o / 2) % 2) * (c->cfg.ny / 2),
             k1 = (o / 4) * (c->cfg.nz / 2);
         for (v = 0; v < c->cfg.num_vars; v++) {
            const double *p = blk(c, jobs[t].parent, v);
            double *ch = blk(c, jobs[t].child[o], v);
            for (i2 = i = 1; i <= c->cfg.nx / 2; i++, i2 += 2)
               for (j2 = j = 1; j <= c->cfg.ny / 2; j++, j2 += 2)
                  for (k2 = k = 1; k <= c->cfg.nz / 2; k++, k2 += 2) {
                     double q = RF(c, AT(p, i + i1, j + j1, k + k1) / 8.0);
                     AT(ch, i2, j2, k2) = q;
                     AT(ch, i2 + 1, j2, k2) = q;
                     AT(ch, i2, j2 + 1, k2) = q;
                     AT(ch, i2 + 1, j2 + 1, k2) = q;
                     AT(ch, i2, j2, k2 + 1) = q;
                     AT(ch, i2 + 1, j2, k2 + 1) = q;
                     AT(ch, i2, j2 + 1, k2 + 1) = q;
                     AT(ch, i2 + 1, j2 + 1, k2 + 1) = q;
                  }
         }
      }
   return MAMR_OK;
}

/* Neumaier-compensated FP64 sum of the 8 children of one coarse cell, in
 * the reference's term order; used for FP32 pools. */
static double sum8_compensated(const double *t)
{
   double s = t[0], comp = 0.0;
   int q;
   for (q = 1; q < 8; q++) {
      double u = s + t[q];
      if (fabs(s) >= fabs(t[q]))
         comp += (s - u) + t[q];
      else
         comp += (t[q] - u) + s;
      s = u;
   }
   return s + comp;
}

/* ref/block.c:411-431: each coarse interior cell is the left-to-right sum
 * of its 8 children (no division: cell values are extensive).  The target's
 * ghost cells keep the slot's previous contents. */
int mamr_consolidate(mamr_ctx *c, const mamr_consolidate_job *jobs,
                     int32_t n)
{
   int32_t t;
   int o, v, i, j, k, i2, j2, k2;
   if (!c || n < 0 || (n && !jobs))
      return fail(MAMR_EINVAL, "bad consolidate arguments");
   for (t = 0; t < n; t++) {
      if (!check_slot(c, jobs[t].target))
         return fail(MAMR_EINVAL, "consolidate target slot out of range");
      for (o = 0; o < 8; o++)
         if (!check_slot(c, jobs[t].child[o]))
            return fail(MAMR_EINVAL, "consolidate child slot out of range");
   }
   for (t = 0; t < n; t++)
      for (o = 0; o < 8; o++) {
         int i1 = (o % 2) * (c->cfg.nx / 2), j1 = ((o / 2) % 2) * (c->cfg.ny / 2),
             k1 = (o / 4) * (c->cfg.nz / 2);
         for (v = 0; v < c->cfg.num_vars; v++) {
            double *p = blk(c, jobs[t].target, v);
            const double *ch = blk(c, jobs[t].child[o], v);
            for (i2 = i = 1; i <= c->cfg.nx / 2; i++, i2 += 2)
               for (j2 = j = 1; j <= c->cfg.ny / 2; j++, j2 += 2)
                  for (k2 = k = 1; k <= c->cfg.nz / 2; k++, k2 += 2) {
                     double t8[8] = {
                        AT(ch, i2, j2, k2), AT(ch, i2 + 1, j2, k2),
                        AT(ch, i2, j2 + 1, k2), AT(ch, i2 + 1, j2 + 1, k2),
                        AT(ch, i2, j2, k2 + 1), AT(ch, i2 + 1, j2, k2 + 1),
                        AT(ch, i2, j2 + 1, k2 + 1),
                        AT(ch, i2 + 1, j2 + 1, k2 + 1) };
                     double s;
                     if (c->fp32)
                        s = (double) (float) sum8_compensated(t8);
                     else {
                        int q;
                        s = t8[0];
                        for (q = 1; q < 8; q++)
                           s += t8[q];
                     }
                     AT(p, i + i1, j + j1, k + k1) = s;
                  }
         }
      }
   return MAMR_OK;
}

/* ref/driver.c:73-108 with comm_vars = num_vars (one comm per stage). */
int mamr_run_timesteps(mamr_ctx *c, int32_t num_ts, int32_t stages_per_ts,
                       int32_t checksum_freq, int32_t first_stage,
                       int32_t flags, double *sums, int32_t *n_sums)
{
   int ts, stage, var, r, cnt = 0, gstage = first_stage;
   (void) flags;
   if (!c || num_ts < 0 || stages_per_ts < 1 || checksum_freq < 0)
      return fail(MAMR_EINVAL, "bad run arguments");
   for (ts = 0; ts < num_ts; ts++)
      for (stage = 0; stage < stages_per_ts; stage++, gstage++) {
         int do_cs = checksum_freq && !(stage % checksum_freq);
         if ((r = mamr_comm(c, 0, c->cfg.num_vars, gstage)))
            return r;
         for (var = 0; var < c->cfg.num_vars; var++) {
            if ((r = mamr_stencil(c, var, gstage)))
               return r;
            if (do_cs) {
               double s;
               if ((r = mamr_check_sum(c, var, &s)))
                  return r;
               if (sums)
                  sums[(size_t) cnt * c->cfg.num_vars + var] = s;
            }
         }
         if (do_cs)
            cnt++;
      }
   if (n_sums)
      *n_sums = cnt;
   return MAMR_OK;
}

/* ref/init.c:484-495 on one rank: zero every cell, then the interior from
 * the unseeded rand() stream (seed 1), reproduced with a private random_r
 * state. */
int mamr_initial_values(const mamr_config *cfg, int32_t n_blocks, double *out)
{
   char state[128];
   struct random_data rd;
   int32_t b;
   int v, i, j, k, X, Y, Z;
   size_t bv;
   if (!cfg || n_blocks < 0 || (n_blocks && !out) || cfg->nx < 1 ||
       cfg->ny < 1 || cfg->nz < 1 || cfg->num_vars < 1)
      return fail(MAMR_EINVAL, "bad initial-value arguments");
   memset(&rd, 0, sizeof(rd));
   memset(state, 0, sizeof(state));
   if (initstate_r(1u, state, sizeof(state), &rd))
      return fail(MAMR_EINVAL, "initstate_r failed");
   X = cfg->nx + 2; Y = cfg->ny + 2; Z = cfg->nz + 2;
   bv = (size_t) X * Y * Z;
   /* stencil 0: init() draws a1 and a0[] first (ref/init.c:418-423) */
   if (cfg->stencil == 0)
      for (i = 0; i < 1 + cfg->num_vars / 4; i++) {
         int32_t r;
         random_r(&rd, &r);
      }
   for (b = 0; b < n_blocks; b++)
      for (v = 0; v < cfg->num_vars; v++) {
         double *a = out + ((size_t) b * cfg->num_vars + v) * bv;
         memset(a, 0, sizeof(double) * bv);
         for (i = 1; i <= cfg->nx; i++)
            for (j = 1; j <= cfg->ny; j++)
               for (k = 1; k <= cfg->nz; k++) {
                  int32_t r;
                  random_r(&rd, &r);
                  a[((size_t) i * Y + j) * Z + k] =
                     ((double) r) / ((double) RAND_MAX);
               }
      }
   return MAMR_OK;
}

/* ref/init.c:418-423: a1, then a0[0 .. num_vars/4), from the seed-1 rand()
 * stream before any cell value. */
int mamr_work_coefficients(int32_t num_vars, double *a1, double *a0)
{
   char state[128];
   struct random_data rd;
   int32_t r;
   int i;
   if (num_vars < 1 || !a1 || (num_vars >= 4 && !a0))
      return fail(MAMR_EINVAL, "bad coefficient arguments");
   memset(&rd, 0, sizeof(rd));
   memset(state, 0, sizeof(state));
   if (initstate_r(1u, state, sizeof(state), &rd))
      return fail(MAMR_EINVAL, "initstate_r failed");
   random_r(&rd, &r);
   *a1 = ((double) r) / ((double) RAND_MAX);
   for (i = 0; i < num_vars / 4; i++) {
      random_r(&rd, &r);
      a0[i] = ((double) r) / ((double) RAND_MAX);
   }
   return MAMR_OK;
}

/* ---- refinement marking ------------------------------------------------- */

/* Raises *x to v (flags only rise: -1 < 0 < 1); counts the change. */
static void mark_raise(int32_t *x, int32_t v, int *changed)
{
   if (*x < v) {
      *x = v;
      *changed = 1;
   }
}

/* reset_all + check_objects (or the uniform assignment) + refine_level on
 * one rank (ref/refine.c:500-527, ref/move.c:65-623, ref/refine.c:68-74,
 * 325-496), as the least fixed point of their rules, applied in passes
 * over all blocks until none changes:
 *   initial   a block: 1 if an object meets it (0 at the maximum level),
 *             else 0 if, with refine_ghost, one meets its parent's extent,
 *             else 0 at level 0, else -1 (uniform: 1 below the maximum
 *             level, 0 at it); a parent: 0 if a child is itself a parent,
 *             else -1;
 *   family    a block at 1 -- or at 0, except the initial zeros of the
 *             uniform assignment, whose families the reference never
 *             touches -- raises its parent to 0; a parent at 0 raises its
 *             children to 0 (ref/move.c:124-135, refine.c:348-359);
 *   refine    a block at 1 raises same-level neighbours to 0 and coarser
 *             ones to 1 (refine.c:360-396);
 *   keep      a block with a finer neighbour rises to 0 (refine.c:397-415);
 *             a block at 0 raises coarser neighbours to 0
 *             (refine.c:437-462). */
int mamr_mark_refine(mamr_ctx *c, const mamr_mark_params *p,
                     const mamr_object *objs, int32_t n_objs,
                     const mamr_mark_block *mb, int32_t nb,
                     const mamr_mark_parent *pa, int32_t np,
                     int32_t *block_refine, int32_t *parent_refine)
{
   const int32_t cap = c ? c->cfg.max_blocks : 0;
   unsigned char *listed;
   int32_t *ref, *pref, i, k;
   const char *msg;
   int changed, uni, bsize[3], passes = 0;
   if (!c || (nb && !block_refine) || (np && !parent_refine))
      return fail(MAMR_EINVAL, "mark_refine: bad arguments");
   listed = (unsigned char *) calloc((size_t) cap + 1, 1);
   ref = (int32_t *) malloc(sizeof(int32_t) * ((size_t) cap + 1));
   pref = (int32_t *) malloc(sizeof(int32_t) * ((size_t) np + 1));
   if (!listed || !ref || !pref) {
      free(listed); free(ref); free(pref);
      return fail(MAMR_ENOMEM, "mark_refine: out of host memory");
   }
   if ((msg = mamr_mark_validate(p, objs, n_objs, mb, nb, pa, np, cap,
                                 listed))) {
      free(listed); free(ref); free(pref);
      return fail(MAMR_EINVAL, "%s", msg);
   }
   uni = p->uniform_refine != 0;
   bsize[0] = c->cfg.nx; bsize[1] = c->cfg.ny; bsize[2] = c->cfg.nz;
   for (i = 0; i < np; i++) {
      pref[i] = -1;
      for (k = 0; k < 8; k++)
         if (pa[i].child[k] < 0)
            pref[i] = 0;
   }
   for (i = 0; i < nb; i++) {
      const mamr_mark_block *b = &mb[i];
      int r;
      if (uni) {
         r = b->level < p->num_refine ? 1 : 0;
      } else {
         r = mamr_mg_block_state(b->cen, b->level, p, bsize, objs, n_objs);
         if (r == 1 && b->level == p->num_refine)
            r = 0;
         if (r == -1 && b->level == 0)
            r = 0;
      }
      ref[b->slot] = r;
   }
   do {
      changed = 0;
      for (i = 0; i < nb; i++) {
         const mamr_mark_block *b = &mb[i];
         const int32_t v = ref[b->slot];
         int l;
         if ((v == 1 || (v == 0 && !uni)) && b->parent >= 0)
            mark_raise(&pref[b->parent], 0, &changed);
         for (l = 0; l < 6; l++) {
            const int nl = b->nei_level[l];
            if (nl == b->level + 1)
               mark_raise(&ref[b->slot], 0, &changed);
            else if (v == 1 && nl == b->level)
               mark_raise(&ref[b->nei[l]], 0, &changed);
            else if (v >= 0 && nl == b->level - 1)
               mark_raise(&ref[b->nei[l]], v, &changed);
         }
      }
      for (i = 0; i < np; i++)
         if (pa[i].active && pref[i] >= 0)
            for (k = 0; k < 8; k++) {
               const int32_t ch = pa[i].child[k];
               if (ch >= 0 && listed[ch])
                  mark_raise(&ref[ch], 0, &changed);
            }
      /* the caller's pass cap, as the device applies it */
      if (changed && p->max_passes > 0 && ++passes >= p->max_passes) {
         free(listed); free(ref); free(pref);
         return fail(MAMR_EDEVICE, "refinement marking did not settle");
      }
   } while (changed);
   for (i = 0; i < nb; i++)
      block_refine[i] = ref[mb[i].slot];
   for (i = 0; i < np; i++)
      if (pa[i].active)
         parent_refine[i] = pref[i];
   free(listed); free(ref); free(pref);
   return MAMR_OK;
}

/* Test helper, no counterpart in the ABI: the FNV-1a hash oracle/ref_hooks.c
 * takes of the reference's mesh after each refine() -- per block in
 * sorted_list order its number (8 bytes) and then slot, level,
 * nei_level[6], nei[6][2][2] and cen[3] as 35 int32 values. */
uint64_t mamr_oracle_mesh_hash(const mamr_block *b, const int64_t *numbers,
                               const int32_t *cen, int32_t n)
{
   uint64_t h = 1469598103934665603ULL;
   int32_t q, l, a, d;
   for (q = 0; q < n; q++) {
      int32_t rec[35];
      const unsigned char *c;
      size_t i;
      rec[0] = b[q].slot;
      rec[1] = b[q].level;
      for (l = 0; l < 6; l++) {
         rec[2 + l] = b[q].nei_level[l];
         for (a = 0; a < 2; a++)
            for (d = 0; d < 2; d++)
               rec[8 + l*4 + a*2 + d] = b[q].nei[l][a][d];
      }
      rec[32] = cen[3*q];
      rec[33] = cen[3*q + 1];
      rec[34] = cen[3*q + 2];
      c = (const unsigned char *) &numbers[q];
      for (i = 0; i < sizeof(int64_t); i++)
         h = (h ^ c[i]) * 1099511628211ULL;
      c = (const unsigned char *) rec;
      for (i = 0; i < sizeof(rec); i++)
         h = (h ^ c[i]) * 1099511628211ULL;
   }
   return h;
}
