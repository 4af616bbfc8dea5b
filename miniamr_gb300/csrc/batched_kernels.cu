#include "batched.h"

namespace mamr {

struct BatchedState {
   int dummy;
};

void batched_destroy(BatchedState *b) { delete b; }
void batched_mesh_changed(BatchedState *b) { (void) b; }

}  // namespace mamr
