/*
 * Shared state of the drop-in replacements for the reference's comm.c,
 * stencil.c, check_sum.c and block.c.  These translation units are compiled
 * against the reference's own headers (block.h, comm.h, timer.h, proto.h)
 * and linked with its remaining sources; they keep every symbol those
 * sources call and forward the cell-data work to the mamr_* C ABI.
 *
 * Error convention: like the reference, a failure prints one line and
 * exits with status -1 (ref/block.c:71-75, ref/comm.c:198-201).
 */
#ifndef MAMR_DROPIN_H
#define MAMR_DROPIN_H

#include "miniamr_gb300.h"

/* The context behind the reference's globals; created on first use from
 * x/y/z_block_size, num_vars, max_num_blocks, stencil, code, permute and
 * the MAMR_DTYPE environment variable ("fp64" default, or "fp32"). */
mamr_ctx *mamr_dropin_ctx(void);

/* Makes the device state current: creates the context, uploads the host
 * arrays that init() filled (once), and re-sends the mesh when the active
 * blocks' connectivity changed since the last call. */
void mamr_dropin_sync_state(void);

/* Creates the context and uploads init()'s host arrays (once), without
 * touching the mesh: what split/consolidate need. */
void mamr_dropin_sync_data(void);

/* Marks the mesh as changed (split/consolidate). */
void mamr_dropin_mesh_changed(void);

/* Prints "ERROR: <where>: <library message>" and exits on a failed call. */
void mamr_dropin_check(int rc, const char *where);

/* Copies one block-variable (ghosts included, [i][j][k] dense doubles) out
 * of the device pool; 0 on success.  Used by verification hooks. */
int mamr_dropin_fetch(int slot, int var, double *out);

#endif
