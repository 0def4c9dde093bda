// push_t32.cu -- the particle push kernels for 32 x 32-cell tiles (push.cuh),
// compiled beside particles.cu (16 x 16) and push_t8.cu (8 x 8).
#include "push.cuh"

namespace iskra {
ISKRA_PUSH_TILE_TU(5, t32)
}  // namespace iskra
