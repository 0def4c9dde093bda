// lws.cu -- learned warm start of the CG Poisson solve.
//
// A 4-level convolutional encoder-decoder (32 channels, bias-free 3x3
// convolutions with zero padding, ReLU, 2x2 average pooling, nearest-neighbour
// upsampling with additive skips) maps the first residual of a solve,
// r = b - A ϕ_prev (the scaled residual of the CG pass) divided by its RMS s,
// to the correction (ϕ - ϕ_prev) / s.  A solve in "use" mode adds
// s net(r / s) to ϕ on the free rows before CG starts; CG is always iterated
// to the same tolerance, so the physics is unchanged and only the iteration
// count falls.  In "harvest" mode each CG solve records its (r / s,
// (ϕ - ϕ_prev) / s) pair; iskra_lws_train fits the network to the recorded
// pairs (Adam on the mean squared error) with the kernels below.  A
// bias-free ReLU network is positively homogeneous, net(s r) = s net(r), so
// the normalisation by s only keeps BF16 values in range.
//
// Layers (H x W image = ny x nx nodes, levels 0..3 at H >> l x W >> l):
//   a0 = relu(conv_1->32(x))             level 0
//   a1 = relu(conv(pool(a0)))            level 1
//   a2 = relu(conv(pool(a1)))            level 2
//   a3 = relu(conv(pool(a2)))            level 3 (bottleneck)
//   a4 = relu(conv(up(a3) + a2))         level 2
//   a5 = relu(conv(up(a4) + a1))         level 1
//   a6 = relu(conv(up(a5) + a0))         level 0
//   y  = conv_32->1(a6)                  level 0, FP32
// Activations and their gradients are BF16 NHWC (32 channels innermost),
// weights BF16 copies of FP32 masters, and every sum accumulates in FP32.
// The 32->32 convolutions -- forward, input gradient (the same kernel with
// the weights flipped in space and transposed in channels) and weight
// gradient -- run on the tensor cores (mma.sync m16n8k16, BF16 x BF16 ->
// FP32); the 1->32 and 32->1 end layers, pooling, upsampling and the
// elementwise gradient combinations run on the FP32 pipes.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "internal.cuh"

namespace iskra {

typedef __nv_bfloat16 bf16;

namespace {

constexpr int kCh = 32;          // channels
constexpr int kPs = 40;          // shared-memory pixel stride (bf16): 80 B rows keep ldmatrix conflict-free
constexpr int kTy = 8, kTx = 16; // output tile of the tensor-core convolutions (128 pixels)
constexpr int kPatch = (kTy + 2) * (kTx + 2);
constexpr int kLayers = 8;
constexpr int kW1 = 9 * kCh;          // parameters of the 1->32 and 32->1 layers
constexpr int kW32 = 9 * kCh * kCh;   // parameters of a 32->32 layer
constexpr int kParams = 2 * kW1 + 6 * kW32;

__host__ __device__ constexpr int layer_off(int l) { return l == 0 ? 0 : (l <= 7 ? kW1 + (l - 1) * kW32 : kParams); }

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(unsigned addr, unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned addr, unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
// c += a b: a 16x16 (row), b 16x8 (col), BF16 inputs, FP32 accumulators
__device__ __forceinline__ void mma_bf16(float c[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float bf(bf16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float round_bf(float v) { return __bfloat162float(__float2bfloat16(v)); }

// the (kTy + 2) x (kTx + 2) pixels around the output tile whose first pixel is
// (y0 + 1, x0 + 1), 32 channels each, zero outside the H x W image
__device__ __forceinline__ void load_patch(bf16 (*patch)[kPs], const bf16 *__restrict__ in, int H, int W, int y0,
                                           int x0) {
  for (int t = threadIdx.x; t < kPatch * 4; t += blockDim.x) {
    const int q = t & 3, pix = t >> 2;
    const int y = y0 + pix / (kTx + 2), x = x0 + pix % (kTx + 2);
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (y >= 0 && y < H && x >= 0 && x < W) v = *reinterpret_cast<const uint4 *>(in + ((size_t)y * W + x) * kCh + q * 8);
    *reinterpret_cast<uint4 *>(&patch[pix][q * 8]) = v;
  }
}

// out[p][n] = act(Σ_tap Σ_k in[p + off(tap)][k] w[tap][n][k]) over an H x W
// image (off(tap) = (tap / 3 - 1, tap % 3 - 1), zero padding).  One block per
// 8 x 16 output tile, four warps of two 16-pixel rows each; per tap and
// 16-channel slice a warp issues 2 x 4 mma (rows x output-channel octets).
template <bool RELU>
__global__ void __launch_bounds__(128) k_conv32(const bf16 *__restrict__ in, const bf16 *__restrict__ w,
                                                bf16 *__restrict__ out, int H, int W) {
  __shared__ __align__(16) bf16 patch[kPatch][kPs];
  __shared__ __align__(16) bf16 wsm[9 * kCh][kPs];
  const int tx = blockIdx.x, ty = blockIdx.y;
  load_patch(patch, in, H, W, ty * kTy - 1, tx * kTx - 1);
  for (int t = threadIdx.x; t < 9 * kCh * 4; t += blockDim.x) {
    const int q = t & 3, row = t >> 2;
    *reinterpret_cast<uint4 *>(&wsm[row][q * 8]) = *reinterpret_cast<const uint4 *>(w + row * kCh + q * 8);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float acc[2][4][4];
#pragma unroll
  for (int mi = 0; mi < 2; mi++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[mi][ni][q] = 0.f;
  for (int tap = 0; tap < 9; tap++) {
    const int dy = tap / 3, dx = tap % 3;  // patch offsets of the tap
#pragma unroll
    for (int kc = 0; kc < 2; kc++) {
      unsigned b[4][2];
#pragma unroll
      for (int np = 0; np < 2; np++) {
        const int n = np * 16 + (lane & 7) + 8 * (lane >> 4);
        const int k = kc * 16 + 8 * ((lane >> 3) & 1);
        ldsm_x4(smem_u32(&wsm[tap * kCh + n][k]), b[2 * np][0], b[2 * np][1], b[2 * np + 1][0], b[2 * np + 1][1]);
      }
#pragma unroll
      for (int mi = 0; mi < 2; mi++) {
        const int r = warp * 2 + mi;
        const int c = (lane & 7) + 8 * ((lane >> 3) & 1);
        const int k = kc * 16 + 8 * (lane >> 4);
        unsigned a0, a1, a2, a3;
        ldsm_x4(smem_u32(&patch[(r + dy) * (kTx + 2) + c + dx][k]), a0, a1, a2, a3);
#pragma unroll
        for (int ni = 0; ni < 4; ni++) mma_bf16(acc[mi][ni], a0, a1, a2, a3, b[ni][0], b[ni][1]);
      }
    }
  }
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int mi = 0; mi < 2; mi++) {
    const int y = ty * kTy + warp * 2 + mi;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int x = tx * kTx + gid + 8 * h;
      if (y >= H || x >= W) continue;
#pragma unroll
      for (int ni = 0; ni < 4; ni++) {
        float v0 = acc[mi][ni][2 * h], v1 = acc[mi][ni][2 * h + 1];
        if (RELU) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        *reinterpret_cast<__nv_bfloat162 *>(out + ((size_t)y * W + x) * kCh + ni * 8 + 2 * tig) =
            __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

// ---- the same convolution on the 5th-generation tensor cores (tcgen05) ----
//
// Implicit GEMM per 16 x 8-pixel output tile: D (128 pixels x 32 output
// channels, FP32 in tensor memory) = Σ over 9 taps x 2 K-slices of
// A (128 pixels x 16 input channels) B (16 x 32), 18 tcgen05.mma of
// M128 N32 K16 (BF16 x BF16 -> FP32) issued by one thread.  Both operands sit
// in shared memory in the canonical K-major layout without swizzle: "core
// matrices" of 8 rows x 16 bytes (8 channels), 128 contiguous bytes.
//   A: the tile's (16 + 2) x (8 + 2)-pixel patch stored as four planes, one
//      per channel octet, of 180 pixels x 16 bytes.  The tap (dy, dx) view is
//      the plane address shifted by dy * 10 + dx pixels: its 8-row core
//      matrices are the tile's pixel rows (8 consecutive pixels, 16 B apart),
//      successive rows 10 pixels (160 B) apart (stride offset), successive
//      octets one plane (2880 B) apart (leading offset).
//   B: w[tap][n][k] as (tap, octet, n) chunks of 16 bytes: core matrices of
//      8 output channels 128 B apart, octets 512 B apart.
// Blocks are persistent (a fixed number per SM, weights staged once): the
// patch of the next tile streams in by cp.async while the current tile's
// accumulators (two 32-column TMEM buffers) are read back with tcgen05.ld,
// activated, rounded to BF16 and stored.  Waits on the MMA completion
// barrier are bounded; a wait that gives up raises DERR_TIMEOUT and the block
// stops after its MMAs drain.
constexpr int kTcTy = 16, kTcTx = 8;                         // output tile: M = 128 pixels
constexpr int kTcPw = kTcTx + 2, kTcPix = (kTcTy + 2) * kTcPw;  // patch: 18 x 10 pixels
constexpr int kTcPlane = kTcPix * 16;                         // bytes per channel-octet plane
constexpr int kTcPatch = 4 * kTcPlane;                        // 11520 B
constexpr int kTcWBytes = 9 * 4 * kCh * 16;                   // 18432 B
constexpr int kTcSmem = kTcWBytes + 2 * kTcPatch;             // 41472 B
constexpr int kTcBlocksPerSm = 4;                             // 4 x 64 TMEM columns of 512
constexpr unsigned kTcSpins = 1u << 22;                       // polls of the MMA barrier before DERR_TIMEOUT
// instruction descriptor (kind::f16): D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24
constexpr unsigned kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(kCh >> 3) << 17) | ((128u >> 4) << 24);

// shared-memory matrix descriptor: start, leading and stride byte offsets
// (16-byte units), descriptor version 1 (bit 46), no swizzle, base offset 0
__device__ __forceinline__ unsigned long long tc_sdesc(unsigned saddr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((saddr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(unsigned d_tmem, unsigned long long a, unsigned long long b, unsigned acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kTcIdesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned long long *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool tc_wait(unsigned long long *bar, unsigned parity) {
  const unsigned b = smem_u32(bar);
  for (unsigned it = 0; it < kTcSpins; it++) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(b), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// 32 FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld32(unsigned taddr, unsigned (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void cp_async16(unsigned dst, const void *src, unsigned bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}

template <bool RELU>
__global__ void __launch_bounds__(128) k_conv32_tc(const bf16 *__restrict__ in, const bf16 *__restrict__ w,
                                                   bf16 *__restrict__ out, int H, int W, int *err) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  __shared__ __align__(8) unsigned long long bar[2];
  __shared__ unsigned tmem_base;
  __shared__ int stop;
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned sW = smem_u32(tc_smem), sP = sW + kTcWBytes;
  const int ntx = (W + kTcTx - 1) / kTcTx, ntiles = ntx * ((H + kTcTy - 1) / kTcTy);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[1])) : "memory");
    stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int c = tid; c < 9 * kCh * 4; c += blockDim.x) {
    const int o = c & 3, row = c >> 2;  // row = tap * 32 + n
    *reinterpret_cast<uint4 *>(tc_smem + (row >> 5) * 2048 + o * 512 + (row & 31) * 16) =
        *reinterpret_cast<const uint4 *>(w + row * kCh + o * 8);
  }
  auto load_patch_tc = [&](int t, int b) {
    const int y0 = (t / ntx) * kTcTy - 1, x0 = (t % ntx) * kTcTx - 1;
    const unsigned dst = sP + b * kTcPatch;
    for (int c = tid; c < kTcPix * 4; c += blockDim.x) {
      const int o = c & 3, q = c >> 2;
      const int y = y0 + q / kTcPw, x = x0 + q % kTcPw;
      const bool ok = y >= 0 && y < H && x >= 0 && x < W;
      cp_async16(dst + o * kTcPlane + q * 16, ok ? in + ((size_t)y * W + x) * kCh + o * 8 : in, ok ? 16u : 0u);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  auto issue = [&](int b) {
    tc_fence_after();
    const unsigned pa = sP + b * kTcPatch, d = tmem_base + b * kCh;
#pragma unroll
    for (int tap = 0; tap < 9; tap++) {
      const int dy = tap / 3, dx = tap % 3;
#pragma unroll
      for (int kc = 0; kc < 2; kc++) {
        const unsigned long long a = tc_sdesc(pa + kc * 2 * kTcPlane + (dy * kTcPw + dx) * 16, kTcPlane, kTcPw * 16);
        const unsigned long long bd = tc_sdesc(sW + tap * 2048 + kc * 1024, 512, 128);
        tc_mma(d, a, bd, (tap | kc) ? 1u : 0u);
      }
    }
    tc_commit(&bar[b]);
  };
  int t = blockIdx.x;
  if (t < ntiles) load_patch_tc(t, 0);
  asm volatile("cp.async.wait_all;" ::: "memory");
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && t < ntiles) issue(0);
  unsigned phase = 0;  // bit b: parity of the next completion of bar[b]
  int b = 0;
  for (; t < ntiles; t += gridDim.x, b ^= 1) {
    const int tn = t + gridDim.x;
    if (tn < ntiles) load_patch_tc(tn, b ^ 1);
    const bool ok = tc_wait(&bar[b], (phase >> b) & 1u);
    if (ok) phase ^= 1u << b;
    tc_fence_after();
    if (ok) {
      unsigned r[32];
      tc_ld32(tmem_base + b * kCh + ((unsigned)(warp * 32) << 16), r);
      const int m = tid;  // TMEM lane = GEMM row = tile pixel
      const int y = (t / ntx) * kTcTy + (m >> 3), x = (t % ntx) * kTcTx + (m & 7);
      if (y < H && x < W) {
        uint4 *dst = reinterpret_cast<uint4 *>(out + ((size_t)y * W + x) * kCh);
#pragma unroll
        for (int q = 0; q < 4; q++) {
          unsigned v[4];
#pragma unroll
          for (int e = 0; e < 4; e++) {
            float v0 = __uint_as_float(r[8 * q + 2 * e]), v1 = __uint_as_float(r[8 * q + 2 * e + 1]);
            if (RELU) {
              v0 = fmaxf(v0, 0.f);
              v1 = fmaxf(v1, 0.f);
            }
            __nv_bfloat162 p2 = __floats2bfloat162_rn(v0, v1);
            v[e] = *reinterpret_cast<unsigned *>(&p2);
          }
          dst[q] = make_uint4(v[0], v[1], v[2], v[3]);
        }
      }
    } else {
      atomicOr(err, DERR_TIMEOUT);
      stop = 1;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (stop) break;
    if (tid == 0 && tn < ntiles) issue(b ^ 1);
  }
  if (stop && tid == 0) tc_wait(&bar[b], (phase >> b) & 1u);  // the MMAs in flight drain before TMEM is freed
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem_base) : "memory");
  }
}

// The same convolution with the patches brought in by the tensor memory
// accelerator: one 3-D tiled bulk-tensor load per channel octet (box 8
// channels x 10 x 18 pixels of the NHWC activation, zeros outside the image
// -- the load starts at pixel (-1, -1) of the tile, its channel coordinate is
// a multiple of 8 BF16 = 16 bytes) writes exactly one octet plane of the
// patch (pixel q = y 10 + x, 16 bytes each), completing on the buffer's
// mbarrier.  One thread issues the loads and the MMAs; the others only read
// the accumulators back.  Planes are 2944 bytes apart (128-byte aligned).
constexpr int kTmaPlane = 2944;
constexpr int kTmaPatch = 4 * kTmaPlane;
constexpr int kTmaSmem = kTcWBytes + 2 * kTmaPatch + 128;  // + room to align the base to 128 bytes
constexpr unsigned kTmaBytes = 4u * kTcPix * 16u;         // bytes a patch load delivers

__device__ __forceinline__ void tma_patch(const CUtensorMap *map, unsigned dst, int c, int x, int y, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

template <bool RELU>
__global__ void __launch_bounds__(128) k_conv32_tma(const __grid_constant__ CUtensorMap map,
                                                    const bf16 *__restrict__ w, bf16 *__restrict__ out, int H, int W,
                                                    int *err) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  __shared__ __align__(8) unsigned long long ld_bar[2], mma_bar[2];
  __shared__ unsigned tmem_base;
  __shared__ int stop;
  const int tid = threadIdx.x, warp = tid >> 5;
  const unsigned base = (smem_u32(tc_smem) + 127u) & ~127u;
  unsigned char *gbase = tc_smem + (base - smem_u32(tc_smem));
  const unsigned sW = base, sP = base + kTcWBytes;
  const int ntx = (W + kTcTx - 1) / kTcTx, ntiles = ntx * ((H + kTcTy - 1) / kTcTy);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(&tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int d = 0; d < 2; d++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&ld_bar[d])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mma_bar[d])) : "memory");
    }
    stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<unsigned long long>(&map)) : "memory");
  }
  for (int c = tid; c < 9 * kCh * 4; c += blockDim.x) {
    const int o = c & 3, row = c >> 2;  // row = tap * 32 + n
    *reinterpret_cast<uint4 *>(gbase + (row >> 5) * 2048 + o * 512 + (row & 31) * 16) =
        *reinterpret_cast<const uint4 *>(w + row * kCh + o * 8);
  }
  fence_async_smem();  // the weights (generic stores) are read by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = tmem_base;
  auto load = [&](int t, int b) {
    const int y0 = (t / ntx) * kTcTy - 1, x0 = (t % ntx) * kTcTx - 1;
    const unsigned bar = smem_u32(&ld_bar[b]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(kTmaBytes) : "memory");
#pragma unroll
    for (int o = 0; o < 4; o++) tma_patch(&map, sP + b * kTmaPatch + o * kTmaPlane, 8 * o, x0, y0, bar);
  };
  auto issue = [&](int b) {
    tc_fence_after();
    const unsigned pa = sP + b * kTmaPatch, d = tmem + b * kCh;
#pragma unroll
    for (int tap = 0; tap < 9; tap++) {
      const int dy = tap / 3, dx = tap % 3;
#pragma unroll
      for (int kc = 0; kc < 2; kc++) {
        const unsigned long long a = tc_sdesc(pa + kc * 2 * kTmaPlane + (dy * kTcPw + dx) * 16, kTmaPlane, kTcPw * 16);
        const unsigned long long bd = tc_sdesc(sW + tap * 2048 + kc * 1024, 512, 128);
        tc_mma(d, a, bd, (tap | kc) ? 1u : 0u);
      }
    }
    tc_commit(&mma_bar[b]);
  };
  int t = blockIdx.x;
  unsigned ldp = 0, mmp = 0;  // bit b: parity of the next completion of buffer b's barriers
  unsigned ldpend = 0;        // thread 0: bit b, a load into buffer b not yet waited for
  bool mma_pending = false;   // thread 0: an issued MMA group not yet waited for
  if (tid == 0 && t < ntiles) {
    load(t, 0);
    ldpend |= 1u;
  }
  int b = 0;
  for (; t < ntiles; t += gridDim.x, b ^= 1) {
    const int tn = t + gridDim.x;
    if (tid == 0) {
      // buffer b ^ 1 is free: the MMAs that read it (tile t - G) completed in the previous iteration
      if (tn < ntiles) {
        load(tn, b ^ 1);
        ldpend |= 1u << (b ^ 1);
      }
      if (tc_wait(&ld_bar[b], (ldp >> b) & 1u)) {
        ldp ^= 1u << b;
        ldpend &= ~(1u << b);
        issue(b);
        mma_pending = true;
      } else {
        atomicOr(err, DERR_TIMEOUT);
        stop = 1;
      }
    }
    __syncthreads();
    if (stop) break;
    const bool ok = tc_wait(&mma_bar[b], (mmp >> b) & 1u);
    if (ok) mmp ^= 1u << b;
    tc_fence_after();
    if (ok) {
      unsigned r[32];
      tc_ld32(tmem + b * kCh + ((unsigned)(warp * 32) << 16), r);
      const int m = tid;  // TMEM lane = GEMM row = tile pixel
      const int y = (t / ntx) * kTcTy + (m >> 3), x = (t % ntx) * kTcTx + (m & 7);
      if (y < H && x < W) {
        uint4 *dst = reinterpret_cast<uint4 *>(out + ((size_t)y * W + x) * kCh);
#pragma unroll
        for (int q = 0; q < 4; q++) {
          unsigned v[4];
#pragma unroll
          for (int e = 0; e < 4; e++) {
            float v0 = __uint_as_float(r[8 * q + 2 * e]), v1 = __uint_as_float(r[8 * q + 2 * e + 1]);
            if (RELU) {
              v0 = fmaxf(v0, 0.f);
              v1 = fmaxf(v1, 0.f);
            }
            __nv_bfloat162 p2 = __floats2bfloat162_rn(v0, v1);
            v[e] = *reinterpret_cast<unsigned *>(&p2);
          }
          dst[q] = make_uint4(v[0], v[1], v[2], v[3]);
        }
      }
    } else {
      atomicOr(err, DERR_TIMEOUT);
      stop = 1;
    }
    tc_fence_before();
    __syncthreads();
    if (tid == 0 && ok) mma_pending = false;
    if (stop) break;
  }
  if (tid == 0 && stop) {
    // bounded drains: the MMAs and the loads still in flight finish before
    // TMEM and the block's shared memory are given up
    if (mma_pending) tc_wait(&mma_bar[b], (mmp >> b) & 1u);
    for (int x = 0; x < 2; x++)
      if (ldpend & (1u << x)) tc_wait(&ld_bar[x], (ldp >> x) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
  }
}

// dw[tap][co][ci] += Σ_p dz[p][co] in[p + off(tap)][ci]: nine warps, one per
// tap, each a 32 x 32 FP32 tile (co x ci) over the K = pixel dimension in
// steps of one 16-pixel tile row; operands are read transposed from the
// pixel-major tiles (ldmatrix .trans).  Blocks stride over the image's tiles
// and add their sums to dw once.
__global__ void __launch_bounds__(288) k_conv32_dw(const bf16 *__restrict__ in, const bf16 *__restrict__ dz,
                                                   float *__restrict__ dw, int H, int W) {
  __shared__ __align__(16) bf16 patch[kPatch][kPs];
  __shared__ __align__(16) bf16 dzs[kTy * kTx][kPs];
  const int lane = threadIdx.x & 31, tap = threadIdx.x >> 5;
  const int dy = tap / 3, dx = tap % 3;
  const int ntx = (W + kTx - 1) / kTx, nty = (H + kTy - 1) / kTy;
  float acc[2][4][4];
#pragma unroll
  for (int mi = 0; mi < 2; mi++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[mi][ni][q] = 0.f;
  for (int t = blockIdx.x; t < ntx * nty; t += gridDim.x) {
    const int tx = t % ntx, ty = t / ntx;
    __syncthreads();  // the previous tile's operands are no longer read
    load_patch(patch, in, H, W, ty * kTy - 1, tx * kTx - 1);
    for (int u = threadIdx.x; u < kTy * kTx * 4; u += blockDim.x) {
      const int q = u & 3, pix = u >> 2;
      const int y = ty * kTy + pix / kTx, x = tx * kTx + pix % kTx;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (y < H && x < W) v = *reinterpret_cast<const uint4 *>(dz + ((size_t)y * W + x) * kCh + q * 8);
      *reinterpret_cast<uint4 *>(&dzs[pix][q * 8]) = v;
    }
    __syncthreads();
    const int i = lane >> 3, j = lane & 7;
    for (int r = 0; r < kTy; r++) {
      unsigned a[2][4];
#pragma unroll
      for (int mi = 0; mi < 2; mi++) {
        // matrices (co lo, p lo), (co hi, p lo), (co lo, p hi), (co hi, p hi)
        const int p = r * kTx + j + 8 * (i >> 1);
        ldsm_x4_t(smem_u32(&dzs[p][mi * 16 + 8 * (i & 1)]), a[mi][0], a[mi][1], a[mi][2], a[mi][3]);
      }
#pragma unroll
      for (int np = 0; np < 2; np++) {
        // matrices (p lo, ci 0-7), (p hi, ci 0-7), (p lo, ci 8-15), (p hi, ci 8-15) of the pair
        const int c = j + 8 * (i & 1);
        unsigned b0, b1, b2, b3;
        ldsm_x4_t(smem_u32(&patch[(r + dy) * (kTx + 2) + c + dx][np * 16 + 8 * (i >> 1)]), b0, b1, b2, b3);
#pragma unroll
        for (int mi = 0; mi < 2; mi++) {
          mma_bf16(acc[mi][2 * np], a[mi][0], a[mi][1], a[mi][2], a[mi][3], b0, b1);
          mma_bf16(acc[mi][2 * np + 1], a[mi][0], a[mi][1], a[mi][2], a[mi][3], b2, b3);
        }
      }
    }
  }
  const int gid = lane >> 2, tig = lane & 3;
  float *d = dw + tap * kCh * kCh;
#pragma unroll
  for (int mi = 0; mi < 2; mi++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int co = mi * 16 + gid + 8 * (q >> 1), ci = ni * 8 + 2 * tig + (q & 1);
        atomicAdd(d + co * kCh + ci, acc[mi][ni][q]);
      }
}

// a0[p][c] = relu(Σ_tap x[p + off(tap)] w0[tap][c]), x rounded to BF16.
// Four threads per pixel, one per channel octet, each holding its 9 x 8
// weights in registers; the quad's x loads coincide (one transaction).
__global__ void __launch_bounds__(256) k_enc0(const float *__restrict__ x, const bf16 *__restrict__ w0,
                                              bf16 *__restrict__ a0, int H, int W) {
  const int o = threadIdx.x & 3;
  float wr[9][8];
#pragma unroll
  for (int tap = 0; tap < 9; tap++)
#pragma unroll
    for (int u = 0; u < 8; u++) wr[tap][u] = bf(w0[tap * kCh + o * 8 + u]);
  const int P = H * W;  // at most 2^30 nodes
  const int per_block = blockDim.x >> 2;
  for (int p = blockIdx.x * per_block + (threadIdx.x >> 2); p < P; p += gridDim.x * per_block) {
    const int y = p / W, xx = p - y * W;
    float v[9];
#pragma unroll
    for (int tap = 0; tap < 9; tap++) {  // unconditional loads of the clamped pixel, zeroed outside
      const int yy = y + tap / 3 - 1, xq = xx + tap % 3 - 1;
      const int yc = min(max(yy, 0), H - 1), xc = min(max(xq, 0), W - 1);
      const float t = __ldg(x + (size_t)yc * W + xc);
      v[tap] = (yy == yc && xq == xc) ? t : 0.f;
    }
    unsigned out[4];
#pragma unroll
    for (int u = 0; u < 8; u += 2) {
      float s0 = 0.f, s1 = 0.f;
#pragma unroll
      for (int tap = 0; tap < 9; tap++) {
        s0 = fmaf(v[tap], wr[tap][u], s0);
        s1 = fmaf(v[tap], wr[tap][u + 1], s1);
      }
      __nv_bfloat162 h2 = __floats2bfloat162_rn(fmaxf(s0, 0.f), fmaxf(s1, 0.f));
      out[u / 2] = *reinterpret_cast<unsigned *>(&h2);
    }
    *reinterpret_cast<uint4 *>(a0 + (size_t)p * kCh + o * 8) = make_uint4(out[0], out[1], out[2], out[3]);
  }
}

// dw0[tap][c] += Σ_p x[p + off(tap)] dz[p][c]: thread (tap, c) of 288
__global__ void __launch_bounds__(288) k_enc0_dw(const float *__restrict__ x, const bf16 *__restrict__ dz,
                                                 float *__restrict__ dw, int H, int W) {
  const int tap = threadIdx.x / kCh, c = threadIdx.x % kCh;
  const int oy = tap / 3 - 1, ox = tap % 3 - 1;
  const int P = H * W;
  float s = 0.f;
  for (int p = blockIdx.x; p < P; p += gridDim.x) {
    const int y = p / W + oy, xx = p % W + ox;
    if (y < 0 || y >= H || xx < 0 || xx >= W) continue;
    s = fmaf(x[y * W + xx], bf(dz[(size_t)p * kCh + c]), s);
  }
  atomicAdd(dw + tap * kCh + c, s);
}

// y[p] = Σ_tap Σ_c a[p + off(tap)][c] w7[tap][c] (FP32 output).  Four
// threads per pixel, one per channel octet (its 9 x 8 weights in registers,
// one 16-byte load per tap), summed across the quad with two shuffles; the
// block's pixel range advances uniformly so every lane reaches the shuffles.
__global__ void __launch_bounds__(256) k_head(const bf16 *__restrict__ a, const bf16 *__restrict__ w7,
                                              float *__restrict__ y, int H, int W) {
  const int o = threadIdx.x & 3;
  float wr[9][8];
#pragma unroll
  for (int tap = 0; tap < 9; tap++)
#pragma unroll
    for (int u = 0; u < 8; u++) wr[tap][u] = bf(w7[tap * kCh + o * 8 + u]);
  const int P = H * W;  // at most 2^30 nodes
  const int per_block = blockDim.x >> 2;
  for (int base = blockIdx.x * per_block; base < P; base += gridDim.x * per_block) {
    const int p = base + (threadIdx.x >> 2);
    float s = 0.f;
    if (p < P) {
      const int yy0 = p / W, xx0 = p - yy0 * W;
      uint4 v[9];
#pragma unroll
      for (int tap = 0; tap < 9; tap++) {
        // unconditional loads from the clamped pixel (all nine in flight at
        // once), zeroed outside the image
        const int yy = yy0 + tap / 3 - 1, xq = xx0 + tap % 3 - 1;
        const int yc = min(max(yy, 0), H - 1), xc = min(max(xq, 0), W - 1);
        const uint4 t = __ldg(reinterpret_cast<const uint4 *>(a + ((size_t)yc * W + xc) * kCh + o * 8));
        v[tap] = (yy == yc && xq == xc) ? t : make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int tap = 0; tap < 9; tap++) {
        const bf16 *e = reinterpret_cast<const bf16 *>(&v[tap]);
#pragma unroll
        for (int u = 0; u < 8; u++) s = fmaf(bf(e[u]), wr[tap][u], s);
      }
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (p < P && o == 0) y[p] = s;
  }
}

// dz6[p][c] = (Σ_tap dy[p - off(tap)] w7[tap][c]) (a6[p][c] > 0)
__global__ void k_head_dx(const float *__restrict__ dy, const bf16 *__restrict__ w7, const bf16 *__restrict__ a,
                          bf16 *__restrict__ dz, int H, int W) {
  __shared__ float ws[kW1];
  for (int t = threadIdx.x; t < kW1; t += blockDim.x) ws[t] = bf(w7[t]);
  __syncthreads();
  const int P = H * W;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int y = p / W, x = p - y * W;
    float g[9];
#pragma unroll
    for (int tap = 0; tap < 9; tap++) {
      const int yy = y - (tap / 3 - 1), xq = x - (tap % 3 - 1);
      g[tap] = (yy >= 0 && yy < H && xq >= 0 && xq < W) ? dy[yy * W + xq] : 0.f;
    }
    const uint4 *src = reinterpret_cast<const uint4 *>(a + (size_t)p * kCh);
    uint4 *dst = reinterpret_cast<uint4 *>(dz + (size_t)p * kCh);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint4 av = src[q];
      const bf16 *ae = reinterpret_cast<const bf16 *>(&av);
      __nv_bfloat162 o[4];
#pragma unroll
      for (int u = 0; u < 8; u += 2) {
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
          s0 = fmaf(g[tap], ws[tap * kCh + q * 8 + u], s0);
          s1 = fmaf(g[tap], ws[tap * kCh + q * 8 + u + 1], s1);
        }
        o[u / 2] = __floats2bfloat162_rn(bf(ae[u]) > 0.f ? s0 : 0.f, bf(ae[u + 1]) > 0.f ? s1 : 0.f);
      }
      dst[q] = *reinterpret_cast<const uint4 *>(o);
    }
  }
}

// dw7[tap][c] += Σ_p a[p + off(tap)][c] dy[p]: thread (tap, c) of 288
__global__ void __launch_bounds__(288) k_head_dw(const bf16 *__restrict__ a, const float *__restrict__ dy,
                                                 float *__restrict__ dw, int H, int W) {
  const int tap = threadIdx.x / kCh, c = threadIdx.x % kCh;
  const int oy = tap / 3 - 1, ox = tap % 3 - 1;
  const int P = H * W;
  float s = 0.f;
  for (int p = blockIdx.x; p < P; p += gridDim.x) {
    const int y = p / W + oy, xx = p % W + ox;
    if (y < 0 || y >= H || xx < 0 || xx >= W) continue;
    s = fmaf(bf(a[((size_t)y * W + xx) * kCh + c]), dy[p], s);
  }
  atomicAdd(dw + tap * kCh + c, s);
}

// 8-channel chunks: thread per (pixel, chunk) of the output image
__device__ __forceinline__ void unpack8(const uint4 &v, float f[8]) {
  const bf16 *e = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
  for (int u = 0; u < 8; u++) f[u] = bf(e[u]);
}
__device__ __forceinline__ uint4 pack8(const float f[8]) {
  __nv_bfloat162 o[4];
#pragma unroll
  for (int u = 0; u < 4; u++) o[u] = __floats2bfloat162_rn(f[2 * u], f[2 * u + 1]);
  return *reinterpret_cast<const uint4 *>(o);
}
__device__ __forceinline__ uint4 ld8(const bf16 *base, size_t pix, int q) {
  return reinterpret_cast<const uint4 *>(base + pix * kCh)[q];
}

// out (H/2 x W/2) = 2x2 average of in (H x W)
__global__ void k_pool(const bf16 *__restrict__ in, bf16 *__restrict__ out, int H, int W) {
  const int h = H / 2, w = W / 2, n = h * w * 4;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = t & 3, p = t >> 2, y = p / w, x = p - y * w;
    float s[8] = {}, f[8];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      unpack8(ld8(in, (size_t)(2 * y + (u >> 1)) * W + 2 * x + (u & 1), q), f);
#pragma unroll
      for (int e = 0; e < 8; e++) s[e] += f[e];
    }
#pragma unroll
    for (int e = 0; e < 8; e++) s[e] *= 0.25f;
    reinterpret_cast<uint4 *>(out + (size_t)p * kCh)[q] = pack8(s);
  }
}

// u (H x W) = up(a) + skip, a at H/2 x W/2
__global__ void k_up_add(const bf16 *__restrict__ a, const bf16 *__restrict__ skip, bf16 *__restrict__ u, int H,
                         int W) {
  const int n = H * W * 4, w = W / 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = t & 3, p = t >> 2, y = p / W, x = p - y * W;
    float f[8], g[8];
    unpack8(ld8(a, (size_t)(y / 2) * w + x / 2, q), f);
    unpack8(ld8(skip, p, q), g);
#pragma unroll
    for (int e = 0; e < 8; e++) f[e] += g[e];
    reinterpret_cast<uint4 *>(u + (size_t)p * kCh)[q] = pack8(f);
  }
}

// dz (h x w) = (Σ over the 2x2 children of du (2h x 2w)) (a > 0)
__global__ void k_up_bwd_mask(const bf16 *__restrict__ du, const bf16 *__restrict__ a, bf16 *__restrict__ dz, int h,
                              int w) {
  const int n = h * w * 4, W = 2 * w;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = t & 3, p = t >> 2, y = p / w, x = p - y * w;
    float s[8] = {}, f[8], m[8];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      unpack8(ld8(du, (size_t)(2 * y + (u >> 1)) * W + 2 * x + (u & 1), q), f);
#pragma unroll
      for (int e = 0; e < 8; e++) s[e] += f[e];
    }
    unpack8(ld8(a, p, q), m);
#pragma unroll
    for (int e = 0; e < 8; e++) s[e] = m[e] > 0.f ? s[e] : 0.f;
    reinterpret_cast<uint4 *>(dz + (size_t)p * kCh)[q] = pack8(s);
  }
}

// dz (H x W) = (dp(y/2, x/2) / 4 + ds) (a > 0), dp at H/2 x W/2
__global__ void k_pool_bwd_mask(const bf16 *__restrict__ dp, const bf16 *__restrict__ ds, const bf16 *__restrict__ a,
                                bf16 *__restrict__ dz, int H, int W) {
  const int n = H * W * 4, w = W / 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = t & 3, p = t >> 2, y = p / W, x = p - y * W;
    float f[8], g[8], m[8];
    unpack8(ld8(dp, (size_t)(y / 2) * w + x / 2, q), f);
    unpack8(ld8(ds, p, q), g);
    unpack8(ld8(a, p, q), m);
#pragma unroll
    for (int e = 0; e < 8; e++) f[e] = m[e] > 0.f ? 0.25f * f[e] + g[e] : 0.f;
    reinterpret_cast<uint4 *>(dz + (size_t)p * kCh)[q] = pack8(f);
  }
}

// loss += Σ (y - c t)^2 / P, dy = 2 (y - c t) / P
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ tgt, float c, float *__restrict__ dy,
                      int P, double *__restrict__ loss) {
  __shared__ float sh[32];
  float s = 0.f;
  const float inv = 1.f / (float)P;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const float d = y[p] - c * tgt[p];
    s = fmaf(d, d, s);
    dy[p] = 2.f * d * inv;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(loss, (double)s * inv);
  }
}

// 5-point stencil 4 e - (west + east + south + north), zero outside: the
// shape of the solver's operator, used to measure errors in residual space
__device__ __forceinline__ float stencil5(const float *e, int p, int y, int x, int H, int W) {
  float v = 4.f * e[p];
  if (x > 0) v -= e[p - 1];
  if (x < W - 1) v -= e[p + 1];
  if (y > 0) v -= e[p - W];
  if (y < H - 1) v -= e[p + W];
  return v;
}

// error e = y - c t of the predicted correction
__global__ void k_err(const float *__restrict__ y, const float *__restrict__ tgt, float c, float *__restrict__ e,
                      int P) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) e[p] = y[p] - c * tgt[p];
}
// its energy norm under the 5-point stencil S: loss += e.Se / P, dy = 2 Se / P
__global__ void k_energy(const float *__restrict__ e, float *__restrict__ dy, int H, int W,
                         double *__restrict__ loss) {
  __shared__ float sh[32];
  const int P = H * W;
  const float f = 2.f / (float)P;
  float s = 0.f;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int y = p / W, x = p - y * W;
    const float v = stencil5(e, p, y, x, H, W);
    if (dy) dy[p] = f * v;
    s = fmaf(e[p], v, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(loss, (double)s / P);
  }
}

// BF16 copies of the FP32 masters: wb as stored ([tap][co][ci] for the
// 32->32 layers), wt flipped in space and transposed in channels
// (wt[8 - tap][ci][co]) for the input-gradient convolutions
__global__ void k_weights_bf16(const float *__restrict__ w, bf16 *__restrict__ wb, bf16 *__restrict__ wt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
    const bf16 v = __float2bfloat16(w[i]);
    wb[i] = v;
    if (i >= kW1 && i < kW1 + 6 * kW32) {
      const int l = (i - kW1) / kW32, r = (i - kW1) % kW32;
      const int tap = r / (kCh * kCh), co = (r / kCh) % kCh, ci = r % kCh;
      wt[kW1 + l * kW32 + ((8 - tap) * kCh + ci) * kCh + co] = v;
    }
  }
}

// Adam (FP32 masters, bias-corrected moments)
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

// network input: x = bf16(r / s) of the scaled residual (and a copy into the
// harvested pair when rec != nullptr)
// s = RMS of the first residual (from ss = Σ r²), its inverse and the scale of
// the network's output, on the device (no host round trip inside the solve)
__global__ void k_lws_scale(LwsScal *ls, int P, double gain) {
  const double s = sqrt(ls->ss / P);
  const bool ok = s > 0 && isfinite(s);
  ls->inv_s = ok ? 1.0 / s : 0.0;
  ls->scale = ok ? s * gain : 0.0;
}

__global__ void k_lws_input(const double *__restrict__ r, const LwsScal *__restrict__ ls, float *__restrict__ x,
                            float *__restrict__ rec, int P) {
  const double inv_s = ls->inv_s;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const float v = round_bf((float)(r[p] * inv_s));
    x[p] = v;
    if (rec) rec[p] = v;
  }
}

// sum of squares (FP64 accumulation)
template <typename T>
__global__ void k_sumsq(const T *__restrict__ a, int n, double *__restrict__ out) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const double v = (double)a[p];
    s += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(out, s);
  }
}

// one pass of the binomial filter [1 2 1]/4 x [1 2 1]/4 (edge values repeated)
__global__ void k_smooth(const float *__restrict__ in, float *__restrict__ out, int H, int W) {
  const int P = H * W;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const int y = p / W, x = p - y * W;
    const int ym = max(y - 1, 0), yp = min(y + 1, H - 1), xm = max(x - 1, 0), xp = min(x + 1, W - 1);
    auto row = [&](int yy) { return in[yy * W + xm] + 2.f * in[yy * W + x] + in[yy * W + xp]; };
    out[p] = (row(ym) + 2.f * row(y) + row(yp)) * 0.0625f;
  }
}

// harvested target (ϕ - ϕ_prev) / s
__global__ void k_lws_target(const double *__restrict__ phi, const double *__restrict__ prev,
                             const LwsScal *__restrict__ ls, float *__restrict__ t, int P) {
  const double inv_s = ls->inv_s;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x)
    t[p] = (float)((phi[p] - prev[p]) * inv_s);
}

}  // namespace

struct Lws {
  int H = 0, W = 0;
  int h[4] = {}, w[4] = {};
  int capacity = 0, count = 0, next = 0;
  bool harvest = false, use = false;
  int smooth = 4;                              // binomial passes over the prediction before it is applied
  bool energy_loss = true;                     // train on the energy norm of the error
  long long adam_t = 0;
  float *w32 = nullptr, *g32 = nullptr, *m = nullptr, *v = nullptr;
  bf16 *wb = nullptr, *wt = nullptr;
  float *x = nullptr, *y = nullptr, *dy = nullptr;
  float *te = nullptr;                         // error of the prediction (energy-norm loss)
  bf16 *a[7] = {}, *p[4] = {}, *u[3] = {};   // p[1..3]; u[l] at level l
  bf16 *dz[7] = {}, *du[3] = {}, *dp[4] = {};
  float *din = nullptr, *dout = nullptr;       // harvested pairs: capacity x P each
  double *prev = nullptr;                      // ϕ before the solve (harvest)
  double *loss = nullptr;                      // device accumulator
  int slot = -1;                               // pair being harvested by the running solve
  double gain = 0.0;                           // network output x gain = correction / s (0: not set)
  long long solves = 0;
  LwsScal *scal = nullptr;                     // device: s of the running solve, warm-start statistics
  std::vector<std::pair<const void *, CUtensorMap>> maps;  // TMA maps of the 32 -> 32 convolutions' inputs
  std::vector<void *> allocs;
};

namespace {

int lws_alloc(Ctx *c, Lws *L, void **p, size_t bytes) {
  ISKRA_CUDA(c, cudaMalloc(p, bytes));
  L->allocs.push_back(*p);
  ISKRA_CUDA(c, cudaMemset(*p, 0, bytes));
  return ISKRA_OK;
}

void lws_free(Lws *L) {
  for (void *p : L->allocs) cudaFree(p);
  delete L;
}

int blocks_for(Ctx *c, long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  long long cap = (long long)c->num_sms * 8;
  return (int)std::max(1LL, std::min(b, cap));
}

dim3 conv_grid(int H, int W) { return dim3((W + kTx - 1) / kTx, (H + kTy - 1) / kTy); }

#define LWS_TRY(call)        \
  do {                       \
    const int rc_ = (call);  \
    if (rc_) return rc_;     \
  } while (0)

// out = act(conv(in, w)) for one 32 -> 32 layer: tcgen05 kernel, or the
// mma.sync kernel when the context selected it (ISKRA_CONV_MMA_SYNC=1, kept
// for measurement)
int conv32(Ctx *c, bool relu, const bf16 *in, const bf16 *w, bf16 *out, int H, int W) {
  cudaStream_t st = c->stream;
  static const bool legacy = [] {
    const char *e = std::getenv("ISKRA_CONV_MMA_SYNC");
    return e && e[0] == '1';
  }();
  if (legacy) {
    if (relu) k_conv32<true><<<conv_grid(H, W), 128, 0, st>>>(in, w, out, H, W);
    else k_conv32<false><<<conv_grid(H, W), 128, 0, st>>>(in, w, out, H, W);
    ISKRA_CUDA(c, cudaGetLastError());
    return ISKRA_OK;
  }
  static bool attr = false;
  if (!attr) {
    ISKRA_CUDA(c, cudaFuncSetAttribute(k_conv32_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    ISKRA_CUDA(c, cudaFuncSetAttribute(k_conv32_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    ISKRA_CUDA(c, cudaFuncSetAttribute(k_conv32_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmaSmem));
    ISKRA_CUDA(c, cudaFuncSetAttribute(k_conv32_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmaSmem));
    attr = true;
  }
  const int tiles = ((W + kTcTx - 1) / kTcTx) * ((H + kTcTy - 1) / kTcTy);
  const int grid = std::min(tiles, kTcBlocksPerSm * c->num_sms);
  const CUtensorMap *map = nullptr;
  for (const auto &m : c->lws->maps)
    if (m.first == in) map = &m.second;
  if (map) {
    if (relu) k_conv32_tma<true><<<grid, 128, kTmaSmem, st>>>(*map, w, out, H, W, c->d_err);
    else k_conv32_tma<false><<<grid, 128, kTmaSmem, st>>>(*map, w, out, H, W, c->d_err);
  } else if (relu) {
    k_conv32_tc<true><<<grid, 128, kTcSmem, st>>>(in, w, out, H, W, c->d_err);
  } else {
    k_conv32_tc<false><<<grid, 128, kTcSmem, st>>>(in, w, out, H, W, c->d_err);
  }
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// TMA tensor map of a 32-channel BF16 NHWC activation (H x W): boxes of 8
// channels x 10 x 18 pixels, zeros outside.  False when the driver cannot
// encode it (the convolution then stages its patches with cp.async).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

static bool activation_map(CUtensorMap *m, const bf16 *ptr, int H, int W) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn || W < kTcPw || H < kTcTy + 2) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)kCh, (cuuint64_t)W, (cuuint64_t)H};
  const cuuint64_t strides[2] = {(cuuint64_t)kCh * sizeof(bf16), (cuuint64_t)W * kCh * sizeof(bf16)};
  const cuuint32_t box[3] = {8, (cuuint32_t)kTcPw, (cuuint32_t)(kTcTy + 2)}, es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16 *>(ptr), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// maps of every input of a 32 -> 32 convolution (forward: pooled inputs and
// upsampled sums; backward: the output gradients)
static void make_maps(Lws *L) {
  L->maps.clear();
  auto add = [&](const bf16 *p, int l) {
    CUtensorMap m;
    if (activation_map(&m, p, L->h[l], L->w[l])) L->maps.emplace_back(p, m);
  };
  for (int l = 1; l <= 3; l++) add(L->p[l], l);
  for (int l = 0; l <= 2; l++) add(L->u[l], l);
  for (int l = 0; l <= 2; l++) add(L->dz[6 - l], l);
  for (int l = 1; l <= 3; l++) add(L->dz[l], l);
}

int lws_forward(Ctx *c, Lws *L) {
  cudaStream_t st = c->stream;
  const int T = 256;
  const bf16 *wb = L->wb;
  const int *h = L->h, *w = L->w;
  k_enc0<<<blocks_for(c, (long long)h[0] * w[0], T), T, 0, st>>>(L->x, wb + layer_off(0), L->a[0], h[0], w[0]);
  for (int l = 1; l <= 3; l++) {
    k_pool<<<blocks_for(c, (long long)h[l] * w[l] * 4, T), T, 0, st>>>(L->a[l - 1], L->p[l], h[l - 1], w[l - 1]);
    LWS_TRY(conv32(c, true, L->p[l], wb + layer_off(l), L->a[l], h[l], w[l]));
  }
  // decoder: a4 at level 2, a5 at level 1, a6 at level 0
  for (int l = 2; l >= 0; l--) {
    const int li = 6 - l;  // layer 4, 5, 6
    k_up_add<<<blocks_for(c, (long long)h[l] * w[l] * 4, T), T, 0, st>>>(L->a[li - 1], L->a[l], L->u[l], h[l], w[l]);
    LWS_TRY(conv32(c, true, L->u[l], wb + layer_off(li), L->a[li], h[l], w[l]));
  }
  k_head<<<blocks_for(c, (long long)h[0] * w[0], T), T, 0, st>>>(L->a[6], wb + layer_off(7), L->y, h[0], w[0]);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// loss and gradients (into g32, zeroed here) for target tscale t: the mean
// squared error of the output (energy = false) or the energy norm of the
// error under the 5-point stencil, the norm CG minimises (energy = true)
int lws_backward(Ctx *c, Lws *L, const float *t, float tscale, bool energy = false) {
  cudaStream_t st = c->stream;
  const int T = 256;
  const int *h = L->h, *w = L->w;
  const int P0 = h[0] * w[0];
  // weight-gradient blocks: at most two per SM, at most one per tile of the level
  auto dwb = [&](int l) {
    return std::max(1, std::min(2 * c->num_sms, ((w[l] + kTx - 1) / kTx) * ((h[l] + kTy - 1) / kTy)));
  };
  ISKRA_CUDA(c, cudaMemsetAsync(L->g32, 0, kParams * sizeof(float), st));
  if (energy) {
    k_err<<<blocks_for(c, P0, T), T, 0, st>>>(L->y, t, tscale, L->te, P0);
    k_energy<<<blocks_for(c, P0, T), T, 0, st>>>(L->te, L->dy, h[0], w[0], L->loss);
  } else {
    k_mse<<<blocks_for(c, P0, T), T, 0, st>>>(L->y, t, tscale, L->dy, P0, L->loss);
  }
  k_head_dx<<<blocks_for(c, P0, T), T, 0, st>>>(L->dy, L->wb + layer_off(7), L->a[6], L->dz[6], h[0], w[0]);
  k_head_dw<<<std::min(P0, 4 * c->num_sms), 288, 0, st>>>(L->a[6], L->dy, L->g32 + layer_off(7), h[0], w[0]);
  // decoder layers 6, 5, 4 (levels 0, 1, 2): input u[l], output gradient dz[li]
  for (int l = 0; l <= 2; l++) {
    const int li = 6 - l;
    LWS_TRY(conv32(c, false, L->dz[li], L->wt + layer_off(li), L->du[l], h[l], w[l]));
    k_conv32_dw<<<dwb(l), 288, 0, st>>>(L->u[l], L->dz[li], L->g32 + layer_off(li), h[l], w[l]);
    // the upsampled input came from layer li - 1 one level down
    k_up_bwd_mask<<<blocks_for(c, (long long)h[l + 1] * w[l + 1] * 4, T), T, 0, st>>>(
        L->du[l], L->a[li - 1], L->dz[li - 1], h[l + 1], w[l + 1]);
  }
  // encoder layers 3, 2, 1: input p[l], then the pooled layer l - 1 gets its
  // pooling gradient plus the skip gradient du[l - 1]
  for (int l = 3; l >= 1; l--) {
    LWS_TRY(conv32(c, false, L->dz[l], L->wt + layer_off(l), L->dp[l], h[l], w[l]));
    k_conv32_dw<<<dwb(l), 288, 0, st>>>(L->p[l], L->dz[l], L->g32 + layer_off(l), h[l], w[l]);
    k_pool_bwd_mask<<<blocks_for(c, (long long)h[l - 1] * w[l - 1] * 4, T), T, 0, st>>>(
        L->dp[l], L->du[l - 1], L->a[l - 1], L->dz[l - 1], h[l - 1], w[l - 1]);
  }
  k_enc0_dw<<<std::min(P0, 4 * c->num_sms), 288, 0, st>>>(L->x, L->dz[0], L->g32 + layer_off(0), h[0], w[0]);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

int lws_sync_weights(Ctx *c, Lws *L) {
  k_weights_bf16<<<blocks_for(c, kParams, 256), 256, 0, c->stream>>>(L->w32, L->wb, L->wt);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// The corrections are many orders smaller than the unit-RMS residual input:
// the network learns them over a fixed gain, their RMS over the pairs
// harvested when it is first trained.
int lws_set_gain(Ctx *c, Lws *L) {
  if (L->gain > 0 || L->count == 0) return ISKRA_OK;
  const size_t P = (size_t)L->H * L->W;
  ISKRA_CUDA(c, cudaMemsetAsync(L->loss, 0, sizeof(double), c->stream));
  for (int k = 0; k < L->count; k++)
    k_sumsq<float><<<blocks_for(c, (long long)P, 256), 256, 0, c->stream>>>(L->dout + k * P, (int)P, L->loss);
  double ss = 0.0;
  ISKRA_CUDA(c, cudaMemcpyAsync(&ss, L->loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  const double g = std::sqrt(ss / ((double)P * L->count));
  L->gain = (g > 0 && std::isfinite(g)) ? g : 1.0;
  return ISKRA_OK;
}

Lws *get_lws(iskra_ctx *h);

}  // namespace

// ---- hooks of the CG solve (poisson.cu) ----

bool lws_active(Ctx *c) { return c->lws && (c->lws->harvest || c->lws->use); }

// After the first residual of a CG solve: r the scaled residual (the
// network's input, normalised by its RMS s).  Records the input of a
// harvested pair and, in use mode, runs the network: *y (device) times
// *scale is the predicted correction of ϕ (*y = nullptr otherwise).  The
// solver applies it along an exact line search in its energy norm.
bool lws_harvesting(Ctx *c) { return c->lws && c->lws->harvest; }

LwsScal *lws_scal(Ctx *c) { return c->lws ? c->lws->scal : nullptr; }

int lws_begin(Ctx *c, const double *r, const float **y, const double **scale) {
  Lws *L = c->lws;
  *y = nullptr;
  *scale = nullptr;
  L->slot = -1;
  const int P = L->H * L->W;
  const int T = 256;
  ISKRA_CUDA(c, cudaMemsetAsync(&L->scal->ss, 0, sizeof(double), c->stream));
  k_sumsq<double><<<blocks_for(c, P, T), T, 0, c->stream>>>(r, P, &L->scal->ss);
  k_lws_scale<<<1, 1, 0, c->stream>>>(L->scal, P, L->gain > 0 ? L->gain : 1.0);
  float *rec = nullptr;
  if (L->harvest && L->capacity > 0) L->slot = L->next;
  if (L->slot >= 0) rec = L->din + (size_t)L->slot * P;
  k_lws_input<<<blocks_for(c, P, T), T, 0, c->stream>>>(r, L->scal, L->x, rec, P);
  ISKRA_CUDA(c, cudaGetLastError());
  L->solves++;
  if (L->use) {
    int rc = lws_forward(c, L);
    if (rc) return rc;
    // the correction's value to CG is in its smooth part (the slow modes);
    // BF16 rounding noise would only add rough residual
    float *a = L->y, *b = L->dy;
    for (int k = 0; k < L->smooth; k++) {
      k_smooth<<<blocks_for(c, P, T), T, 0, c->stream>>>(a, b, L->H, L->W);
      std::swap(a, b);
    }
    ISKRA_CUDA(c, cudaGetLastError());
    *y = a;
    *scale = &L->scal->scale;
  }
  return ISKRA_OK;
}

// ϕ before the solve, for the harvested target (after any warm start is not
// applied yet: the pair is (residual, full correction))
int lws_mark_start(Ctx *c, const double *phi) {
  Lws *L = c->lws;
  if (L->slot < 0) return ISKRA_OK;
  ISKRA_CUDA(c, cudaMemcpyAsync(L->prev, phi, (size_t)L->H * L->W * sizeof(double), cudaMemcpyDeviceToDevice,
                                c->stream));
  return ISKRA_OK;
}

// After the solve: the harvested target of a converged solve
int lws_end(Ctx *c, const double *phi, bool converged) {
  Lws *L = c->lws;
  if (L->slot < 0) return ISKRA_OK;
  const int P = L->H * L->W;
  if (converged) {
    k_lws_target<<<blocks_for(c, P, 256), 256, 0, c->stream>>>(phi, L->prev, L->scal,
                                                                L->dout + (size_t)L->slot * P, P);
    ISKRA_CUDA(c, cudaGetLastError());
    L->next = (L->next + 1) % L->capacity;
    L->count = std::min(L->count + 1, L->capacity);
  }
  L->slot = -1;
  return ISKRA_OK;
}

void lws_destroy_ctx(Ctx *c) {
  if (c->lws) lws_free(c->lws);
  c->lws = nullptr;
}

}  // namespace iskra

using namespace iskra;

namespace iskra {
namespace {
Lws *get_lws(iskra_ctx *h) { return h ? h->c.lws : nullptr; }
}  // namespace
}  // namespace iskra

extern "C" {

int iskra_lws_create(iskra_ctx *h, int capacity, uint64_t seed) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (capacity < 0) return set_err(c, ISKRA_EINVAL, "capacity must be >= 0");
  if (c->nx % 8 || c->ny % 8 || c->nx < 8 || c->ny < 8)
    return set_err(c, ISKRA_EINVAL, "learned warm start needs nx and ny multiples of 8 (three 2x2 poolings)");
  lws_destroy_ctx(c);
  Lws *L = new Lws();
  L->H = c->ny;
  L->W = c->nx;
  for (int l = 0; l < 4; l++) {
    L->h[l] = L->H >> l;
    L->w[l] = L->W >> l;
  }
  L->capacity = capacity;
  const size_t P0 = (size_t)L->H * L->W;
  int rc = 0;
#define LWS_ALLOC(ptr, bytes)                                      \
  do {                                                             \
    rc = lws_alloc(c, L, (void **)&(ptr), (bytes));                \
    if (rc) {                                                      \
      lws_free(L);                                                 \
      return rc;                                                   \
    }                                                              \
  } while (0)
  LWS_ALLOC(L->w32, kParams * sizeof(float));
  LWS_ALLOC(L->g32, kParams * sizeof(float));
  LWS_ALLOC(L->m, kParams * sizeof(float));
  LWS_ALLOC(L->v, kParams * sizeof(float));
  LWS_ALLOC(L->wb, kParams * sizeof(bf16));
  LWS_ALLOC(L->wt, kParams * sizeof(bf16));
  LWS_ALLOC(L->x, P0 * sizeof(float));
  LWS_ALLOC(L->y, P0 * sizeof(float));
  LWS_ALLOC(L->dy, P0 * sizeof(float));
  LWS_ALLOC(L->te, P0 * sizeof(float));
  LWS_ALLOC(L->loss, sizeof(double));
  LWS_ALLOC(L->scal, sizeof(LwsScal));
  LWS_ALLOC(L->prev, P0 * sizeof(double));
  // level of each activation: a0..a3 at 0..3, a4 at 2, a5 at 1, a6 at 0
  const int lev[7] = {0, 1, 2, 3, 2, 1, 0};
  for (int i = 0; i < 7; i++) {
    const size_t n = (size_t)L->h[lev[i]] * L->w[lev[i]] * kCh * sizeof(bf16);
    LWS_ALLOC(L->a[i], n);
    LWS_ALLOC(L->dz[i], n);
  }
  for (int l = 1; l <= 3; l++) {
    const size_t n = (size_t)L->h[l] * L->w[l] * kCh * sizeof(bf16);
    LWS_ALLOC(L->p[l], n);
    LWS_ALLOC(L->dp[l], n);
  }
  for (int l = 0; l <= 2; l++) {
    const size_t n = (size_t)L->h[l] * L->w[l] * kCh * sizeof(bf16);
    LWS_ALLOC(L->u[l], n);
    LWS_ALLOC(L->du[l], n);
  }
  if (capacity > 0) {
    LWS_ALLOC(L->din, (size_t)capacity * P0 * sizeof(float));
    LWS_ALLOC(L->dout, (size_t)capacity * P0 * sizeof(float));
  }
#undef LWS_ALLOC
  make_maps(L);
  // He initialisation (std sqrt(2 / fan_in)); the output layer starts small
  std::vector<float> w0(kParams);
  std::mt19937_64 gen(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int l = 0; l < kLayers; l++) {
    const int n = (l == 0 || l == 7) ? kW1 : kW32;
    const float fan_in = (l == 0) ? 9.f : 9.f * kCh;
    const float sd = (l == 7) ? 0.1f * std::sqrt(1.f / fan_in) : std::sqrt(2.f / fan_in);
    for (int i = 0; i < n; i++) w0[layer_off(l) + i] = sd * nd(gen);
  }
  c->lws = L;
  rc = cuda_check(c, cudaMemcpy(L->w32, w0.data(), kParams * sizeof(float), cudaMemcpyHostToDevice), "weights");
  if (rc) return rc;
  rc = lws_sync_weights(c, L);
  if (rc) return rc;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  return ISKRA_OK;
}

int iskra_lws_destroy(iskra_ctx *h) {
  if (!h) return ISKRA_EINVAL;
  ISKRA_CUDA(&h->c, cudaStreamSynchronize(h->c.stream));
  lws_destroy_ctx(&h->c);
  return ISKRA_OK;
}

int iskra_lws_set_mode(iskra_ctx *h, int harvest, int use, int smooth) {
  Lws *L = get_lws(h);
  if (!L) return h ? set_err(&h->c, ISKRA_EINVAL, "no learned warm start: call iskra_lws_create") : ISKRA_EINVAL;
  if (harvest && L->capacity == 0) return set_err(&h->c, ISKRA_EINVAL, "harvesting needs capacity > 0");
  if (smooth < 0 || smooth > 64) return set_err(&h->c, ISKRA_EINVAL, "smoothing passes must be in [0, 64]");
  L->harvest = harvest != 0;
  L->use = use != 0;
  L->smooth = smooth;
  return ISKRA_OK;
}

int iskra_lws_info(iskra_ctx *h, int *pairs, int *nparams, int64_t *solves, int64_t *warm_solves,
                   double *mean_alpha, double *mean_ratio) {
  Lws *L = get_lws(h);
  if (!L) return h ? set_err(&h->c, ISKRA_EINVAL, "no learned warm start") : ISKRA_EINVAL;
  Ctx *c = &h->c;
  LwsScal st;
  ISKRA_CUDA(c, cudaMemcpyAsync(&st, L->scal, sizeof(LwsScal), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (pairs) *pairs = L->count;
  if (nparams) *nparams = kParams;
  if (solves) *solves = L->solves;
  if (warm_solves) *warm_solves = st.warm_solves;
  if (mean_alpha) *mean_alpha = st.warm_solves ? st.alpha_sum / st.warm_solves : 0.0;
  if (mean_ratio) *mean_ratio = st.warm_solves ? st.ratio_sum / st.warm_solves : 0.0;
  return ISKRA_OK;
}

int iskra_lws_weights(iskra_ctx *h, float *w_out, const float *w_in) {
  Lws *L = get_lws(h);
  if (!L) return h ? set_err(&h->c, ISKRA_EINVAL, "no learned warm start") : ISKRA_EINVAL;
  Ctx *c = &h->c;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (w_in) {
    ISKRA_CUDA(c, cudaMemcpy(L->w32, w_in, kParams * sizeof(float), cudaMemcpyHostToDevice));
    int rc = lws_sync_weights(c, L);
    if (rc) return rc;
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  if (w_out) ISKRA_CUDA(c, cudaMemcpy(w_out, L->w32, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  return ISKRA_OK;
}

int iskra_lws_forward(iskra_ctx *h, const float *in, float *out) {
  Lws *L = get_lws(h);
  if (!L || !in || !out) return h ? set_err(&h->c, ISKRA_EINVAL, "no learned warm start / null array") : ISKRA_EINVAL;
  Ctx *c = &h->c;
  const size_t P = (size_t)L->H * L->W;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpy(L->x, in, P * sizeof(float), cudaMemcpyHostToDevice));
  int rc = lws_forward(c, L);
  if (rc) return rc;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpy(out, L->y, P * sizeof(float), cudaMemcpyDeviceToHost));
  return ISKRA_OK;
}

int iskra_lws_loss_grad(iskra_ctx *h, const float *in, const float *target, double *loss, float *grad) {
  Lws *L = get_lws(h);
  if (!L || !in || !target) return h ? set_err(&h->c, ISKRA_EINVAL, "no learned warm start / null array") : ISKRA_EINVAL;
  Ctx *c = &h->c;
  const size_t P = (size_t)L->H * L->W;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpy(L->x, in, P * sizeof(float), cudaMemcpyHostToDevice));
  // the target is staged in the (P doubles) harvest buffer
  ISKRA_CUDA(c, cudaMemcpy(L->prev, target, P * sizeof(float), cudaMemcpyHostToDevice));
  ISKRA_CUDA(c, cudaMemset(L->loss, 0, sizeof(double)));
  int rc = lws_forward(c, L);
  if (rc) return rc;
  rc = lws_backward(c, L, (const float *)L->prev, 1.f);
  if (rc) return rc;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (loss) ISKRA_CUDA(c, cudaMemcpy(loss, L->loss, sizeof(double), cudaMemcpyDeviceToHost));
  if (grad) ISKRA_CUDA(c, cudaMemcpy(grad, L->g32, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  return ISKRA_OK;
}

// mean loss of the network over the harvested pairs and of the zero predictor
int iskra_lws_eval(iskra_ctx *h, double *loss, double *zero_loss) {
  Lws *L = get_lws(h);
  if (!L) return h ? set_err(&h->c, ISKRA_EINVAL, "no learned warm start") : ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (L->count == 0) return set_err(c, ISKRA_EINVAL, "no harvested pairs");
  int rc = lws_set_gain(c, L);
  if (rc) return rc;
  const size_t P = (size_t)L->H * L->W;
  const float ts = (float)(1.0 / L->gain);
  double *acc = (double *)L->prev;  // [0] network, [1] zero predictor
  ISKRA_CUDA(c, cudaMemsetAsync(acc, 0, 2 * sizeof(double), c->stream));
  const int b = blocks_for(c, (long long)P, 256);
  for (int k = 0; k < L->count; k++) {
    ISKRA_CUDA(c, cudaMemcpyAsync(L->x, L->din + k * P, P * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    rc = lws_forward(c, L);
    if (rc) return rc;
    const float *t = L->dout + k * P;
    if (L->energy_loss) {
      k_err<<<b, 256, 0, c->stream>>>(L->y, t, ts, L->te, (int)P);
      k_energy<<<b, 256, 0, c->stream>>>(L->te, nullptr, L->H, L->W, acc);
      ISKRA_CUDA(c, cudaMemsetAsync(L->dy, 0, P * sizeof(float), c->stream));  // the zero predictor
      k_err<<<b, 256, 0, c->stream>>>(L->dy, t, ts, L->te, (int)P);
      k_energy<<<b, 256, 0, c->stream>>>(L->te, nullptr, L->H, L->W, acc + 1);
    } else {
      k_mse<<<b, 256, 0, c->stream>>>(L->y, t, ts, L->dy, (int)P, acc);
      k_sumsq<float><<<b, 256, 0, c->stream>>>(t, (int)P, acc + 1);
    }
  }
  double hacc[2];
  ISKRA_CUDA(c, cudaMemcpyAsync(hacc, acc, sizeof(hacc), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (loss) *loss = hacc[0] / L->count;
  if (zero_loss)
    *zero_loss = L->energy_loss ? hacc[1] / L->count : hacc[1] / ((double)P * L->count) / (L->gain * L->gain);
  return ISKRA_OK;
}

// iters Adam steps on the harvested pairs (one pair per step, drawn
// uniformly with a seeded generator); *loss_out = mean loss of the last
// min(iters, 64) steps
int iskra_lws_train(iskra_ctx *h, int iters, double lr, uint64_t seed, double *loss_out) {
  Lws *L = get_lws(h);
  if (!L) return h ? set_err(&h->c, ISKRA_EINVAL, "no learned warm start") : ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (iters < 0 || !(lr > 0)) return set_err(c, ISKRA_EINVAL, "bad iteration count / learning rate");
  if (L->count == 0) return set_err(c, ISKRA_EINVAL, "no harvested pairs to train on");
  int rc0 = lws_set_gain(c, L);
  if (rc0) return rc0;
  const float ts = (float)(1.0 / L->gain);
  const size_t P = (size_t)L->H * L->W;
  std::mt19937_64 gen(seed);
  std::uniform_int_distribution<int> pick(0, L->count - 1);
  const int tail = std::min(iters, 64);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int it = 0; it < iters; it++) {
    if (it == iters - tail) ISKRA_CUDA(c, cudaMemsetAsync(L->loss, 0, sizeof(double), c->stream));
    const int k = pick(gen);
    ISKRA_CUDA(c, cudaMemcpyAsync(L->x, L->din + (size_t)k * P, P * sizeof(float), cudaMemcpyDeviceToDevice,
                                  c->stream));
    int rc = lws_forward(c, L);
    if (rc) return rc;
    rc = lws_backward(c, L, L->dout + (size_t)k * P, ts, L->energy_loss);
    if (rc) return rc;
    L->adam_t++;
    const float c1 = 1.f / (1.f - std::pow(b1, (float)L->adam_t));
    const float c2 = 1.f / (1.f - std::pow(b2, (float)L->adam_t));
    k_adam<<<blocks_for(c, kParams, 256), 256, 0, c->stream>>>(L->w32, L->g32, L->m, L->v, (float)lr, b1, b2, c1, c2,
                                                               eps);
    rc = lws_sync_weights(c, L);
    if (rc) return rc;
  }
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (loss_out) {
    double l = 0;
    if (tail > 0) ISKRA_CUDA(c, cudaMemcpy(&l, L->loss, sizeof(double), cudaMemcpyDeviceToHost));
    *loss_out = tail > 0 ? l / tail : 0.0;
  }
  return ISKRA_OK;
}

}  // extern "C"
