// noalloc.cu -- density deposit that allocates no device memory.
//
// Some callers cannot allocate: a host framework that reserves all device
// memory up front and forbids later cudaMalloc, or code that runs while
// another library holds the stream in capture, where an allocation would
// break the capture.  iskra_density_noalloc serves them: the caller passes
// device pointers for the particle positions and the output density, and the
// int64 fixed-point accumulator that the deposit needs lives in the
// file-scope array below.  That array is part of the library image: every
// GPU that loads the library holds it (kNoAllocMaxNodes * 8 bytes = 8 MiB)
// until the process exits.
#include <atomic>
#include <cmath>

#include "internal.cuh"

namespace iskra {

constexpr int kNoAllocMaxNodes = 1 << 20;  // grids up to 1024 x 1024 nodes
constexpr int kNoAllocMaxDevices = 64;

// Shared by every call: it keeps the last call's contents, so each call
// clears it before depositing; calls that overlap on the GPU race on it.
static __device__ __align__(256) unsigned long long g_noalloc_acc[kNoAllocMaxNodes];

// Device address of g_noalloc_acc per device, looked up once with that device
// current (in host code the symbol itself is only a host-side stand-in).
// Host threads may call concurrently: each entry is published atomically (two
// threads racing on the first call both look up the same address).  The
// cached address belongs to the device's primary context: it assumes that
// context outlives every call (no cudaDeviceReset between calls).
static std::atomic<unsigned long long *> g_acc_addr[kNoAllocMaxDevices];

__global__ void __launch_bounds__(256) k_noalloc_deposit(const double *__restrict__ x, long long np, long long ld,
                                                         double dx, double dy, int nx, int ny, int shift,
                                                         unsigned long long *__restrict__ acc,
                                                         int *__restrict__ bad) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np;
       p += (long long)gridDim.x * blockDim.x) {
    // same cell / 2^-24 offset quantisation as the species upload
    const double fx = x[p] / dx, fy = x[p + ld] / dy;
    const double ix = floor(fx), jy = floor(fy);
    long long i0 = (long long)ix, j0 = (long long)jy;
    long long ux = llrint((fx - ix) * 16777216.0), uy = llrint((fy - jy) * 16777216.0);
    if (ux >= 16777216LL) {
      if (i0 + 1 <= nx - 2) { i0 += 1; ux = 0; } else { ux = 16777215LL; }
    }
    if (uy >= 16777216LL) {
      if (j0 + 1 <= ny - 2) { j0 += 1; uy = 0; } else { uy = 16777215LL; }
    }
    if (!(fx == fx) || !(fy == fy) || i0 < 0 || j0 < 0 || i0 > nx - 2 || j0 > ny - 2) {
      atomicOr(bad, 1);
      continue;
    }
    const unsigned long long gx = (1ull << 24) - (unsigned long long)ux;
    const unsigned long long gy = (1ull << 24) - (unsigned long long)uy;
    unsigned long long w[4] = {gx * gy, (unsigned long long)ux * gy, gx * (unsigned long long)uy,
                               (unsigned long long)ux * (unsigned long long)uy};
    if (shift) {
      const unsigned long long half = 1ull << (shift - 1);
      for (int k = 0; k < 4; k++) w[k] = (w[k] + half) >> shift;
    }
    const long long n0 = i0 + (long long)nx * j0;
    atomicAdd(acc + n0, w[0]);
    atomicAdd(acc + n0 + 1, w[1]);
    atomicAdd(acc + n0 + nx, w[2]);
    atomicAdd(acc + n0 + nx + 1, w[3]);
  }
}

// n = acc * w0 * 2^(shift-48) / cell_volume (RegularGrids.jl:26-38)
__global__ void k_noalloc_finalize(const unsigned long long *__restrict__ acc, int nx, int ny, double scale,
                                   double V0, int4 per, double *__restrict__ n_out) {
  const int nn = nx * ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int i = k % nx, j = k / nx;
    double V = V0;
    if (i == 0 && !per.x) V *= 0.5;
    if (i == nx - 1 && !per.y) V *= 0.5;
    if (j == 0 && !per.z) V *= 0.5;
    if (j == ny - 1 && !per.w) V *= 0.5;
    n_out[k] = (double)acc[k] * scale / V;
  }
}

}  // namespace iskra

using namespace iskra;

extern "C" int iskra_density_noalloc(const iskra_grid_t *grid, const double *x, int64_t np, int64_t ld, double w0,
                                     double *n_out, int *flag, uint64_t stream) {
  if (!grid || (!x && np > 0) || !n_out || !flag || np < 0 || ld < np || !(w0 > 0)) return ISKRA_EINVAL;
  if (grid->nx < 2 || grid->ny < 2 || !(grid->dx > 0) || !(grid->dy > 0)) return ISKRA_EINVAL;
  // particle_cell ignores the origin (ParticleInCell.jl:28-35): like
  // iskra_ctx_create, only the zero origin is accepted
  if (grid->ox != 0.0 || grid->oy != 0.0) return ISKRA_EINVAL;
  const long long nn = (long long)grid->nx * grid->ny;
  if (nn > kNoAllocMaxNodes) return ISKRA_EINVAL;  // grid larger than the static accumulator
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ISKRA_ECUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return ISKRA_EINVAL;
  unsigned long long *acc = g_acc_addr[dev].load(std::memory_order_acquire);
  if (!acc) {
    // one-time set-up for this device (before any stream capture)
    unsigned long long *ptr = nullptr;
    if (cudaGetSymbolAddress((void **)&ptr, g_noalloc_acc) != cudaSuccess || !ptr) return ISKRA_ECUDA;
    g_acc_addr[dev].store(ptr, std::memory_order_release);
    acc = ptr;
  }
  cudaStream_t st = (cudaStream_t)(uintptr_t)stream;
  if (cudaMemsetAsync(acc, 0, (size_t)nn * sizeof(unsigned long long), st) != cudaSuccess) return ISKRA_ECUDA;
  if (cudaMemsetAsync(flag, 0, sizeof(int), st) != cudaSuccess) return ISKRA_ECUDA;
  int bits = 0;
  while ((1LL << bits) < np + 1) bits++;
  const int shift = 48 + bits > 63 ? 48 + bits - 63 : 0;
  if (np > 0) {
    long long blocks = (np + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_noalloc_deposit<<<(unsigned)blocks, 256, 0, st>>>(x, np, ld, grid->dx, grid->dy, grid->nx, grid->ny, shift,
                                                        acc, flag);
  }
  const int4 per = make_int4(grid->bc[0] != 0, grid->bc[1] != 0, grid->bc[2] != 0, grid->bc[3] != 0);
  long long fb = (nn + 255) / 256;
  if (fb > 1024) fb = 1024;
  k_noalloc_finalize<<<(unsigned)fb, 256, 0, st>>>(acc, grid->nx, grid->ny, w0 * ldexp(1.0, shift - 48),
                                                   grid->dx * grid->dy, per, n_out);
  return cudaGetLastError() == cudaSuccess ? ISKRA_OK : ISKRA_ECUDA;
}
