/*
 * Drop-in replacement of the reference's move.c.
 *
 * move() (ref/move.c:37-63, called from ref/driver.c:112) advances the
 * refinement objects on the host, as the reference does.  check_objects()
 * (ref/move.c:65-141, called from ref/refine.c:78 after reset_all())
 * hands the whole marking of the step -- the object tests and the rules of
 * refine_level() -- to mamr_mark_refine() and writes the flags back into
 * blocks[].refine and parents[].refine.  Those flags are the fixed point
 * refine_level() (ref/refine.c:325-496) converges to, so when the
 * reference's refine_level() runs next it finds nothing to change.
 * check_block() keeps its prototype (ref/proto.h:86) for link
 * compatibility; nothing calls it.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>

#include "block.h"
#include "comm.h"
#include "proto.h"
#include "dropin.h"

/* One axis of one object: position and size advance by delta; with
 * bounce 1 the centre reflects off the faces of the unit cube and the
 * motion reverses.  The reference's bounce-2 branch (ref/move.c:51-59)
 * hangs off the inner if-chain of the bounce-1 branch (C's dangling else)
 * and can never run, so any other bounce value only moves the object. */
static void advance(object *op, int d, double delta)
{
   op->cen[d] += delta * op->move[d];
   op->size[d] += delta * op->inc[d];
   if (op->bounce != 1)
      return;
   if (op->cen[d] >= 1.0) {
      op->cen[d] = 2.0 - op->cen[d];
      op->move[d] = -op->move[d];
   } else if (op->cen[d] <= 0.0) {
      op->cen[d] = 0.0 - op->cen[d];
      op->move[d] = -op->move[d];
   }
}

void move(double delta)
{
   int o, d;
   for (o = 0; o < num_objects; o++)
      for (d = 0; d < 3; d++)
         advance(&objects[o], d, delta);
}

static mamr_object *objs;
static mamr_mark_block *mb;
static mamr_mark_parent *pa;
static int32_t *bref, *pref;
static int cap_objs, cap_mb, cap_pa;

static void *grow(void *p, int *cap, int want, size_t elem)
{
   if (want <= *cap)
      return p;
   *cap = want + want / 4 + 16;
   p = realloc(p, (size_t) *cap * elem);
   if (!p) {
      printf("ERROR: check_objects: out of host memory\n");
      exit(-1);
   }
   return p;
}

void check_objects(void)
{
   const int nb = sorted_index[num_refine+1], np = max_active_parent;
   mamr_mark_params prm;
   int o, in, d, l, k;

   objs = (mamr_object *) grow(objs, &cap_objs, num_objects,
                               sizeof(mamr_object));
   mb = (mamr_mark_block *) grow(mb, &cap_mb, nb, sizeof(mamr_mark_block));
   bref = (int32_t *) realloc(bref, sizeof(int32_t) * (size_t) (cap_mb + 1));
   pa = (mamr_mark_parent *) grow(pa, &cap_pa, np, sizeof(mamr_mark_parent));
   pref = (int32_t *) realloc(pref, sizeof(int32_t) * (size_t) (cap_pa + 1));
   if (!bref || !pref) {
      printf("ERROR: check_objects: out of host memory\n");
      exit(-1);
   }
   memset(&prm, 0, sizeof(prm));
   prm.num_refine = num_refine;
   prm.refine_ghost = refine_ghost;
   prm.uniform_refine = 0;
   for (d = 0; d < 3; d++)
      prm.mesh_size[d] = mesh_size[d];
   for (o = 0; o < num_objects; o++) {
      objs[o].type = objects[o].type;
      objs[o].reserved = 0;
      for (d = 0; d < 3; d++) {
         objs[o].cen[d] = objects[o].cen[d];
         objs[o].size[d] = objects[o].size[d];
      }
   }
   for (in = 0; in < nb; in++) {
      const int n = sorted_list[in].n;
      const block *bp = &blocks[n];
      mb[in].slot = n;
      mb[in].level = bp->level;
      mb[in].parent = (int32_t) bp->parent;
      for (d = 0; d < 3; d++)
         mb[in].cen[d] = bp->cen[d];
      for (l = 0; l < 6; l++) {
         mb[in].nei_level[l] = bp->nei_level[l];
         mb[in].nei[l] = bp->nei[l][0][0];
      }
   }
   for (k = 0; k < np; k++) {
      pa[k].active = parents[k].number >= 0;
      for (o = 0; o < 8; o++)
         pa[k].child[o] = (int32_t) parents[k].child[o];
   }
   mamr_dropin_check(mamr_mark_refine(mamr_dropin_ctx(), &prm, objs,
                                      num_objects, mb, nb, pa, np, bref,
                                      pref),
                     "mamr_mark_refine");
   for (in = 0; in < nb; in++)
      blocks[sorted_list[in].n].refine = bref[in];
   for (k = 0; k < np; k++)
      if (parents[k].number >= 0)
         parents[k].refine = pref[k];
}

int check_block(double cor[3][2])
{
   (void) cor;
   printf("ERROR: check_block: the marking runs in mamr_mark_refine\n");
   exit(-1);
   return 0;
}
