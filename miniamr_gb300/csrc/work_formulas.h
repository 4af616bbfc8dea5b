/*
 * work_formulas.h -- per-cell formulas of miniAMR's variable-work stencils
 * (--stencil 0; ref/stencil.c:43-74 dispatch, :147-983 kernels).
 *
 * Plain C shared by the GB300 kernels (miniamr_gb300/csrc/work_kernels.cu)
 * and the CPU oracle (oracle/amr_oracle.c).  Each includer first defines
 *   MAMR_WFN               the qualifiers of the functions that take a view
 *                          (static inline, or a template over the view
 *                          type with __device__)
 *   MAMR_WFN0              optional, those of the one that does not
 *                          (defaults to MAMR_WFN)
 *   MAMR_WVIEW             the type of a block view
 *   MAMR_AT(w, v, i, j, k) the value of variable v at cell (i, j, k)
 * and owns the loops and the stores: these functions only evaluate one
 * cell.  Expressions keep the reference's operand order and
 * parenthesisation term by term (products rounded separately: no
 * contraction, -ffp-contract=off / -fmad=false), so that the results are
 * bit-identical to the reference's.
 */
#ifndef MAMR_WORK_FORMULAS_H
#define MAMR_WORK_FORMULAS_H

/* mat = num_vars/4, a1 and a0[0..mat) (ref/init.c:418-423). */
#define MAMR_WORK_MAX_MAT 64
typedef struct {
   int mat;
   double a1;
   double a0[MAMR_WORK_MAX_MAT];
} mamr_work_par;

#endif /* MAMR_WORK_FORMULAS_H */

#if defined(MAMR_WFN) && defined(MAMR_AT) && !defined(MAMR_WORK_FNS_DONE)
#define MAMR_WORK_FNS_DONE

#define MAMR_A(v, i, j, k) MAMR_AT(w, (v), (i), (j), (k))
#ifndef MAMR_WFN0
#define MAMR_WFN0 MAMR_WFN
#endif

/* stencil_0 (ref/stencil.c:147-226): the new value of cell (i, j, k) of
 * var; reads only that cell's variables. */
MAMR_WFN double mamr_w_stencil0(const MAMR_WVIEW *w, int var, int i, int j,
                                int k, const mamr_work_par *P)
{
   const int mat = P->mat;
   const double a1 = P->a1;
   if (var == 1) {
      double x = MAMR_A(1, i, j, k);
      for (int v = mat; v < 2 * mat; v++)
         x += MAMR_A(v, i, j, k) * MAMR_A(0, i, j, k);
      return x;
   }
   const double x = MAMR_A(var, i, j, k);
   if (var < mat)
      return x + x * (MAMR_A(0, i, j, k) + MAMR_A(1, i, j, k) - a1 * x);
   if (var < 2 * mat)
      return x * (MAMR_A(0, i, j, k) + x + a1 * MAMR_A(var + mat, i, j, k) +
                  (1.0 - a1) * MAMR_A(var + 2 * mat, i, j, k)) /
             MAMR_A(1, i, j, k);
   if (var < 3 * mat)
      return x + MAMR_A(var - mat, i, j, k) *
                    (a1 * MAMR_A(0, i, j, k) + P->a0[var - 2 * mat] * x +
                     (1.0 - a1) * MAMR_A(var + mat, i, j, k)) /
                    MAMR_A(1, i, j, k);
   return x + MAMR_A(var - 2 * mat, i, j, k) *
                 (a1 * MAMR_A(0, i, j, k) + P->a0[var - 3 * mat] * x +
                  (1.0 - P->a0[var - 3 * mat]) * MAMR_A(var - mat, i, j, k) +
                  (1.0 - a1) * MAMR_A(var - 2 * mat, i, j, k)) /
                 (MAMR_A(1, i, j, k) * MAMR_A(1, i, j, k));
}

/* stencil_x / _y / _z (ref/stencil.c:228-370, 372-514, 516-659): the new
 * value of cell (i, j, k) of var for the sweep along `axis` (0 x, 1 y,
 * 2 z).  The reference updates in place while its loops advance, so the
 * neighbour at -1 along the axis already holds its new value: the caller
 * walks each line in increasing order and stores every result before the
 * next cell. */
MAMR_WFN double mamr_w_line(const MAMR_WVIEW *w, int var, int axis, int i,
                            int j, int k, const mamr_work_par *P)
{
   const int mat = P->mat;
   const double a1 = P->a1;
   const int di = axis == 0, dj = axis == 1, dk = axis == 2;
   if (var == 1) {
      double x = MAMR_A(1, i, j, k);
      for (int v = 2; v < mat + 2; v++)
         x += MAMR_A(v, i, j, k) * MAMR_A(0, i, j, k);
      x /= (a1 + x);
      return x;
   }
   const double x = MAMR_A(var, i, j, k);
   if (var < mat)
      return x + x * (MAMR_A(0, i, j, k) + MAMR_A(1, i, j, k) - a1 * x) /
                    (P->a0[var] + MAMR_A(1, i, j, k));
   /* the variable whose differences pick the branch, and the two extra
    * terms of the denominator */
   int dv;
   double t0, t1;
   const double am = MAMR_A(var, i - di, j - dj, k - dk);
   const double ap = MAMR_A(var, i + di, j + dj, k + dk);
   if (var < 2 * mat) {
      dv = var;
   } else if (var < 3 * mat) {
      dv = var - mat;
   } else {
      dv = var - 2 * mat;
   }
   const double c = MAMR_A(dv, i, j, k);
   const double tmp1 = fabs(c - MAMR_A(dv, i - di, j - dj, k - dk));
   const double tmp2 = fabs(c - MAMR_A(dv, i + di, j + dj, k + dk));
   const double d = tmp1 > tmp2 ? tmp1 - tmp2 : tmp2 - tmp1;
   const double num = tmp1 * am + d * (x + MAMR_A(1, i, j, k)) + tmp2 * ap;
   double den;
   if (var < 2 * mat) {
      den = a1 + P->a0[var - mat] + am + x + ap + MAMR_A(0, i, j, k) +
            MAMR_A(1, i, j, k);
   } else if (var < 3 * mat) {
      t0 = MAMR_A(var - mat, i, j, k);
      t1 = MAMR_A(var + mat, i, j, k);
      den = a1 + P->a0[var - 2 * mat] + t0 + t1 + am + x + ap;
   } else {
      t0 = MAMR_A(var - mat, i, j, k);
      t1 = MAMR_A(var - 2 * mat, i, j, k);
      den = a1 + P->a0[var - 3 * mat] + t0 + t1 + am + x + ap;
   }
   return num / den;
}

/* stencil_7 (ref/stencil.c:661-784): the work value of cell (i, j, k);
 * the partner variable of each neighbour depends on its axis and on the
 * class of var.  The reference stores work values only after the whole
 * block, so every read is of the values before the call. */
MAMR_WFN double mamr_w_seven(const MAMR_WVIEW *w, int var, int i, int j,
                             int k, const mamr_work_par *P)
{
   const int mat = P->mat;
   int bx, by, bz;            /* partners along x, y, z */
   if (var < mat) {
      bx = var + mat; by = var + 2 * mat; bz = var + 3 * mat;
   } else if (var < 2 * mat) {
      bx = var + mat; by = var + 2 * mat; bz = var - mat;
   } else if (var < 3 * mat) {
      bx = var + mat; by = var - 2 * mat; bz = var - mat;
   } else {
      bx = var - 3 * mat; by = var - 2 * mat; bz = var - mat;
   }
   const double c = MAMR_A(var, i, j, k);
   return (MAMR_A(var, i - 1, j, k) * MAMR_A(bx, i - 1, j, k) +
           MAMR_A(var, i, j - 1, k) * MAMR_A(by, i, j - 1, k) +
           MAMR_A(var, i, j, k - 1) * MAMR_A(bz, i, j, k - 1) +
           c * c +
           MAMR_A(var, i, j, k + 1) * MAMR_A(bz, i, j, k + 1) +
           MAMR_A(var, i, j + 1, k) * MAMR_A(by, i, j + 1, k) +
           MAMR_A(var, i + 1, j, k) * MAMR_A(bx, i + 1, j, k)) /
          7.0 * (P->a1 + c);
}

/* stencil_27 (ref/stencil.c:786-957): the work value of cell (i, j, k):
 * the 27 neighbours in i, j, k order, each taken from the variable of its
 * offset class (corner, edge, face, centre) for the class of var, over
 * a1 + 27. */
MAMR_WFN double mamr_w_twentyseven(const MAMR_WVIEW *w, int var, int i,
                                   int j, int k, const mamr_work_par *P)
{
   const int mat = P->mat;
   int vc[4];                 /* by number of nonzero offsets 0..3 */
   vc[0] = var;
   if (var < mat) {
      vc[1] = var + mat; vc[2] = var + 2 * mat; vc[3] = var + 3 * mat;
   } else if (var < 2 * mat) {
      vc[1] = var + mat; vc[2] = var + 2 * mat; vc[3] = var - mat;
   } else if (var < 3 * mat) {
      vc[1] = var + mat; vc[2] = var - 2 * mat; vc[3] = var - mat;
   } else {
      vc[1] = var - 3 * mat; vc[2] = var - 2 * mat; vc[3] = var - mat;
   }
   double s = 0.0;
   int first = 1;
   for (int di = -1; di <= 1; di++)
      for (int dj = -1; dj <= 1; dj++)
         for (int dk = -1; dk <= 1; dk++) {
            const int cls = (di != 0) + (dj != 0) + (dk != 0);
            const double v = MAMR_A(vc[cls], i + di, j + dj, k + dk);
            if (first) {
               s = v;
               first = 0;
            } else {
               s = s + v;
            }
         }
   return s / (P->a1 + 27.0);
}

/* stencil_check (ref/stencil.c:959-983) on one value. */
MAMR_WFN0 double mamr_w_check(double x, const mamr_work_par *P)
{
   x = fabs(x);
   if (x >= 1.0)
      x /= (P->a1 + P->a0[0] + x);
   else if (x < 0.1)
      x *= 10.0 - P->a1;
   return x;
}

#undef MAMR_A
#endif
