// push_t8.cu -- the particle push kernels for 8 x 8-cell tiles (push.cuh),
// compiled beside particles.cu (16 x 16) and push_t32.cu (32 x 32).
#include "push.cuh"

namespace iskra {
ISKRA_PUSH_TILE_TU(3, t8)
}  // namespace iskra
