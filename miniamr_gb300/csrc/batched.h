// Batched (fused ghost + stencil + checksum) path: per-context state.
#pragma once

#include "mamr_internal.h"

namespace mamr {

struct BatchedState;

void batched_destroy(BatchedState *b);
void batched_mesh_changed(BatchedState *b);

}  // namespace mamr
