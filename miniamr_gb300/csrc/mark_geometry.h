/*
 * mark_geometry.h -- the block/object intersection test of miniAMR's
 * refinement marking (ref/move.c:65-141 check_objects, :143-623
 * check_block), restated as plain C shared by the GB300 kernels
 * (miniamr_gb300/csrc/mark_kernels.cu) and the CPU oracle
 * (oracle/amr_oracle.c).
 *
 * Each includer defines MAMR_MFN, the qualifiers of the functions
 * (static inline, or static __device__ __forceinline__), after the
 * mamr_object / mamr_mark_params types (include/miniamr_gb300.h).  Every
 * comparison and every FP64 expression keeps the reference's form and
 * operand order -- a corner term is ((x - c)/s) * ((x - c)/s), sums run
 * over x, y, z left to right from 0.0 (adding the first term to 0.0 is
 * exact), no contraction (-ffp-contract=off / -fmad=false) -- so the
 * decisions are bit-identical to the reference's.
 */
#ifndef MAMR_MARK_GEOMETRY_H
#define MAMR_MARK_GEOMETRY_H

#if defined(MAMR_MFN)

/* Squared scaled distance of coordinate x from centre c along one axis. */
MAMR_MFN double mamr_mg_sq(double x, double c, double s)
{
   const double q = (x - c) / s;
   return q * q;
}

/* Where centre c lies along one axis of the block [lo, hi]: 1 inside (then
 * *v = 0 for the lower half, 1 for the upper, when `half`; 0 otherwise),
 * 0 outside (*v = 0 below the block, 1 above it). */
MAMR_MFN int mamr_mg_side(double c, double lo, double hi, int half, int *v)
{
   if (c < lo) {
      *v = 0;
      return 0;
   }
   if (c > hi) {
      *v = 1;
      return 0;
   }
   *v = half ? (c < (lo + hi) / 2.0 ? 0 : 1) : 0;
   return 1;
}

/* The block overlaps the object's slab along axis d. */
MAMR_MFN int mamr_mg_overlap(const double cor[3][2], const mamr_object *o,
                             int d)
{
   return cor[d][1] > (o->cen[d] - o->size[d]) &&
          cor[d][0] < (o->cen[d] + o->size[d]);
}

/* The block holds exactly one of the slab's two planes along axis d. */
MAMR_MFN int mamr_mg_straddle(const double cor[3][2], const mamr_object *o,
                              int d)
{
   return (cor[d][0] < (o->cen[d] - o->size[d]) &&
           cor[d][1] < (o->cen[d] + o->size[d])) ||
          (cor[d][0] > (o->cen[d] - o->size[d]) &&
           cor[d][1] > (o->cen[d] + o->size[d]));
}

/* Nearest-corner test over the axes in mask `axes` whose centre lies
 * outside the block: none -> true; one axis d -> |cor[d][v] - c| < s;
 * two or three -> the sum of their squared scaled distances < 1. */
MAMR_MFN int mamr_mg_near(const double cor[3][2], const mamr_object *o,
                          const int in[3], const int v[3], int axes)
{
   int d, n_out = 0, one = 0;
   double sum = 0.0;
   for (d = 0; d < 3; d++)
      if ((axes >> d & 1) && !in[d]) {
         n_out++;
         one = d;
      }
   if (n_out == 0)
      return 1;
   if (n_out == 1)
      return fabs(cor[one][v[one]] - o->cen[one]) < o->size[one];
   for (d = 0; d < 3; d++)
      if ((axes >> d & 1) && !in[d])
         sum = sum + mamr_mg_sq(cor[d][v[d]], o->cen[d], o->size[d]);
   return sum < 1.0;
}

/* Farthest-corner term: sum over the axes in `axes` of the squared scaled
 * distance of the block's far side (1 - v). */
MAMR_MFN double mamr_mg_far(const double cor[3][2], const mamr_object *o,
                            const int v[3], int axes)
{
   int d;
   double sum = 0.0;
   for (d = 0; d < 3; d++)
      if (axes >> d & 1)
         sum = sum + mamr_mg_sq(cor[d][1 - v[d]], o->cen[d], o->size[d]);
   return sum;
}

/* One object against the block [cor[d][0], cor[d][1]]^3
 * (ref/move.c:152-618). */
MAMR_MFN int mamr_mg_object(const double cor[3][2], const mamr_object *o)
{
   const int t = o->type;
   int in[3] = {0, 0, 0}, v[3] = {0, 0, 0}, d, hit = 0;
   if (t == 0) {                       /* surface of a box */
      if (!mamr_mg_overlap(cor, o, 0))
         return 0;
      if (mamr_mg_straddle(cor, o, 0))
         return mamr_mg_overlap(cor, o, 1) && mamr_mg_overlap(cor, o, 2);
      if (mamr_mg_overlap(cor, o, 1))
         return mamr_mg_straddle(cor, o, 1) && mamr_mg_overlap(cor, o, 2);
      return mamr_mg_overlap(cor, o, 2) && mamr_mg_straddle(cor, o, 2);
   }
   if (t == 1)                         /* solid box */
      return mamr_mg_overlap(cor, o, 0) && mamr_mg_overlap(cor, o, 1) &&
             mamr_mg_overlap(cor, o, 2);
   if (t >= 2 && t <= 15) {
      /* spheroid or half of one: even = surface, odd = solid; 4..15 keep
       * the half on one side of the centre plane x, y or z */
      const int surface = !(t % 2);
      for (d = 0; d < 3; d++)
         in[d] = mamr_mg_side(o->cen[d], cor[d][0], cor[d][1], surface,
                              &v[d]);
      if (surface)
         hit = mamr_mg_near(cor, o, in, v, 7) &&
               mamr_mg_far(cor, o, v, 7) > 1.0;
      else
         hit = mamr_mg_near(cor, o, in, v, 7);
      if (hit && t >= 4) {
         const int axis = (t - 4) / 4, upper = ((t - 4) / 2) % 2;
         /* lower halves drop blocks wholly below the centre plane,
          * upper halves blocks wholly above it */
         if (!upper ? cor[axis][1] < o->cen[axis]
                    : cor[axis][0] > o->cen[axis])
            hit = 0;
      }
      return hit;
   }
   if (t >= 20 && t <= 25) {
      /* cylinder along axis ca = (t - 20) / 2: even = surface, odd =
       * solid; c1, c2 the other axes in cyclic order */
      const int ca = (t - 20) / 2, c1 = (ca + 1) % 3, c2 = (ca + 2) % 3;
      const int axes = 1 << c1 | 1 << c2, surface = !(t % 2);
      if (!mamr_mg_overlap(cor, o, ca))
         return 0;
      in[c1] = mamr_mg_side(o->cen[c1], cor[c1][0], cor[c1][1], surface,
                            &v[c1]);
      in[c2] = mamr_mg_side(o->cen[c2], cor[c2][0], cor[c2][1], surface,
                            &v[c2]);
      /* two-term sums: the reference's c1 + c2 order and the x, y, z
       * order give the same bits (IEEE addition commutes).  The surface
       * test checks the end planes along x whatever the axis, as the
       * reference does. */
      if (!surface || mamr_mg_straddle(cor, o, 0))
         return mamr_mg_near(cor, o, in, v, axes);
      return mamr_mg_near(cor, o, in, v, axes) &&
             mamr_mg_far(cor, o, v, axes) > 1.0;
   }
   return 0;                           /* undefined type: no intersection */
}

/* check_block (ref/move.c:143-623): some object, all of whose sizes are
 * non-negative, meets the block. */
MAMR_MFN int mamr_mg_check(const double cor[3][2], const mamr_object *objs,
                           int n_objs)
{
   int o;
   for (o = 0; o < n_objs; o++) {
      const mamr_object *op = &objs[o];
      if (op->size[0] < 0.0 || op->size[1] < 0.0 || op->size[2] < 0.0)
         continue;
      if (mamr_mg_object(cor, op))
         return 1;
   }
   return 0;
}

/* The refine state check_objects gives one block before any rule that
 * involves other blocks (ref/move.c:81-122): 1 when an object meets the
 * block's extent, 0 when, with refine_ghost, one meets its parent's wider
 * extent, -1 otherwise.  bsize = cells per block along x, y, z. */
MAMR_MFN int mamr_mg_block_state(const int cen[3], int level,
                                 const mamr_mark_params *p,
                                 const int bsize[3],
                                 const mamr_object *objs, int n_objs)
{
   const int sz = 1 << (p->num_refine - level);     /* half block size */
   double cor[3][2];
   int d;
   for (d = 0; d < 3; d++) {
      cor[d][0] = ((double) (cen[d] - sz)) / ((double) p->mesh_size[d]);
      cor[d][1] = ((double) (cen[d] + sz)) / ((double) p->mesh_size[d]);
   }
   if (p->refine_ghost)
      for (d = 0; d < 3; d++) {
         const double e = 2.0 * (((double) sz) / ((double) bsize[d])) /
                          ((double) p->mesh_size[d]);
         cor[d][0] -= e;
         cor[d][1] += e;
      }
   if (mamr_mg_check(cor, objs, n_objs))
      return 1;
   if (p->refine_ghost && level) {
      const int szp = 1 << (p->num_refine - level + 1);   /* parent's */
      for (d = 0; d < 3; d++) {
         const double e = (((double) szp) / ((double) bsize[d])) /
                          ((double) p->mesh_size[d]);
         cor[d][0] -= e;
         cor[d][1] += e;
      }
      if (mamr_mg_check(cor, objs, n_objs))
         return 0;
   }
   return -1;
}

#endif /* MAMR_MFN */

/* Host-side argument check shared by both implementations of
 * mamr_mark_refine: returns 0, or a message for MAMR_EINVAL.  is_listed
 * (max_blocks entries, zeroed by the caller) is left marking the listed
 * slots. */
static inline const char *mamr_mark_validate(
   const mamr_mark_params *p, const mamr_object *objs, int32_t n_objs,
   const mamr_mark_block *mb, int32_t nb, const mamr_mark_parent *pa,
   int32_t np, int32_t max_blocks, unsigned char *is_listed)
{
   int32_t i, l, k;
   if (!p || n_objs < 0 || nb < 0 || np < 0 || (n_objs && !objs) ||
       (nb && !mb) || (np && !pa))
      return "mark_refine: bad arguments";
   if (p->num_refine < 0 || p->num_refine > 29 || p->mesh_size[0] <= 0 ||
       p->mesh_size[1] <= 0 || p->mesh_size[2] <= 0)
      return "mark_refine: bad parameters";
   if (p->max_passes < 0)
      return "mark_refine: negative pass cap";
   for (k = 0; k < 9; k++)
      if (p->reserved[k])
         return "mark_refine: reserved parameters must be zero";
   for (i = 0; i < nb; i++) {
      const mamr_mark_block *b = &mb[i];
      if (b->slot < 0 || b->slot >= max_blocks || is_listed[b->slot])
         return "mark_refine: block slot out of range or listed twice";
      if (b->level < 0 || b->level > p->num_refine || b->parent < -1 ||
          b->parent >= np)
         return "mark_refine: block level or parent out of range";
      is_listed[b->slot] = 1;
   }
   for (i = 0; i < nb; i++)
      for (l = 0; l < 6; l++) {
         const int nl = mb[i].nei_level[l], n = mb[i].nei[l];
         if ((nl == mb[i].level || nl == mb[i].level - 1) &&
             (n < 0 || n >= max_blocks || !is_listed[n]))
            return "mark_refine: neighbour is not a listed block";
      }
   for (i = 0; i < np; i++)
      if (pa[i].active)
         for (k = 0; k < 8; k++) {
            const int c = pa[i].child[k];
            if (c >= max_blocks || (c < 0 && -1 - c >= np))
               return "mark_refine: parent's child out of range";
         }
   return 0;
}

#endif /* MAMR_MARK_GEOMETRY_H */
