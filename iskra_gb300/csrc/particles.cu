// particles.cu -- the per-particle hot path:
//   k_push    : CIC gather (cloud_in_cell.jl:20-36) + Boris push with B = 0
//               (pushers.jl:37-50) + after_push wrap!/discard! (wrap.jl) +
//               CIC deposit (cloud_in_cell.jl:1-18) of the pushed particle,
//               fused in one pass over the particle store.
//   k_finalize: density = deposit ./ cell_volume (kinetic.jl:53,
//               RegularGrids.jl:26-38) and ρ = Σ q n (ParticleInCell.jl:118-122).
//   k_efield  : E = -∇ϕ (generalized_poisson.jl:398-410), FP32 copy for the
//               gather and FP64 copy for download.
//   sort      : counting sort by cell + compaction of discarded particles.
//
// Deposit arithmetic: offsets are multiples of 2^-24, u = hx*2^24 is an exact
// integer, so the CIC weights (2^24-u)(2^24-v), u(2^24-v), (2^24-u)v, uv are
// exact 48-bit integers.  Over the particles of one cell they sum to
//   W11 = Σuv,  W10 = 2^24 Σu - Σuv,  W01 = 2^24 Σv - Σuv,
//   W00 = 2^48 n - 2^24 Σu - 2^24 Σv + Σuv,
// so a warp reduces the moments (n, Σu, Σv, Σuv) over each run of lanes in
// the same cell, the run's last lane adds them to the block's window (16-bit
// pieces in 32-bit words) and the block adds the window's node sums with
// 64-bit integer atomics.  Integer addition is associative: the density
// is bit-identical for any particle order or launch shape.  A node's sum
// stays below 2^64 while each of its four cells holds at most 16383
// particles; the per-cell counts are kept alongside and checked by k_finalize.
#include <algorithm>
#include <cmath>

#include "internal.cuh"

namespace iskra {

struct PushParams {
  float h;          // 0.5 * Δt * q/m
  float dtdx, dtdy; // Δt/Δx, Δt/Δy
  int nx, ny;
  int mode_x, mode_y;
  int tiles_x;      // tiles per row
  // surface tracker (all nullptr without one)
  const unsigned char *trk_edge;  // 4 per cell: surface index + 1
  const unsigned char *trk_cell;  // 1: track! records the cell's particles
  const unsigned char *trk_kind;  // ISKRA_SURF_* per surface
  unsigned long long *trk_hits;   // this species' absorbed count per surface
};

// Particle-record loads of the unsorted tail and the ensemble push: read
// once, so they bypass L1 (L1::no_allocate measured 1.5 % faster steps than
// evict-first loads).
__device__ __forceinline__ float4 ld_stream(const float4 *p) {
  float4 r;
  asm volatile("ld.global.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p));
  return r;
}
__device__ __forceinline__ float2 ld_stream(const float2 *p) {
  float2 r;
  asm volatile("ld.global.L1::no_allocate.v2.f32 {%0,%1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
  return r;
}

// Moments of one particle: u, v < 2^24 and uv = hi 2^24 + lo with hi, lo < 2^24,
// so every sum over at most 32 lanes fits in 32 bits.
struct Moments {
  unsigned su, sv, hi, lo;
};

// Inclusive segmented sum of the moments over runs of lanes holding the same
// key (any particle order is correct; cell-sorted particles give long runs):
// shuffle rounds with a run-start guard, as many as the longest run needs
// (at most five).  Returns true on the last lane
// of each run, which then holds the run's sums; *n receives the run length.
// (A per-run __reduce_add_sync over the run's lane mask measured 2x slower on
// GB300 once the runs shorten between sorts.)
__device__ __forceinline__ bool reduce_runs(int key, Moments &m, unsigned &n) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(FULL, key, 1);
  const int next = __shfl_down_sync(FULL, key, 1);
  const bool head = lane == 0 || prev != key;
  const bool tail = lane == 31 || next != key;
  const unsigned heads = __ballot_sync(FULL, head);
  const int start = 31 - __clz(heads & ((2u << lane) - 1u));  // first lane of my run
  if (heads != FULL) {  // warp-uniform: some run is longer than one lane
    // rounds up to the longest run only (d < its length)
    const unsigned pos = (unsigned)(lane - start);
    const unsigned last = __reduce_max_sync(FULL, pos);
#pragma unroll
    for (unsigned d = 1; d < 32; d <<= 1) {
      if (d > last) break;
      const unsigned su = __shfl_up_sync(FULL, m.su, d);
      const unsigned sv = __shfl_up_sync(FULL, m.sv, d);
      const unsigned hi = __shfl_up_sync(FULL, m.hi, d);
      const unsigned lo = __shfl_up_sync(FULL, m.lo, d);
      if (pos >= d) {
        m.su += su;
        m.sv += sv;
        m.hi += hi;
        m.lo += lo;
      }
    }
  }
  n = (unsigned)(lane - start + 1);
  return tail;
}

// Move by d cells along one axis in FP32: offset h in [0,1) on the 2^-24 grid,
// cell index i (int).  Returns the new offset; i is updated in place.
// Move by d cells along one axis in FP32: offset h in [0,1) on the 2^-24
// grid, cell index i (int).  t0 = h + d (one rounding), its integer part k
// moves the cell, the fraction t0 - k goes onto the 2^-24 grid (a fraction
// that rounds up to 1 carries into the next cell).  Branch-free: in a warp
// some lane nearly always crosses a cell, and a branch for it would run for
// all.  Rounded intrinsics: no context-dependent contraction, so every kernel
// inlining this computes the same bits.  Returns the new offset; i is
// updated in place and uq receives the offset as an integer (< 2^24).
__device__ __forceinline__ float move_axis(float h, float d, int &i, unsigned &uq) {
  d = fminf(fmaxf(d, -1.0e9f), 1.0e9f);
  const float t0 = __fadd_rn(h, d);
  const float k = floorf(t0);
  const float t = __fsub_rn(t0, k);  // [0, 1]
  const int u = __float2int_rn(t * kOffScale);
  i += (int)k + (u >> 24);
  uq = (unsigned)u & 0xffffffu;
  return (float)uq * kOffInv;
}

// check! (pic/surfaces/check.jl:18-68) of one tracked particle with hit!
// (hit.jl:33-56, circuit_coupling.jl:45-63): the straight path from the old
// position (cell i, j; offsets hx, hy) over the step, with the new velocity
// dX, dY in cells per step, is walked cell by cell.  At an edge without a
// surface the walk goes on in the next cell; at a surface: PERIODIC ends the
// walk; REFLECT mirrors the rest of the step on the crossed axis (the
// reference's px -= v dt'; v_n = -v_n; px += v dt', so dX loses 2 u tau)
// and goes on from the edge, back on the near side with the flipped
// velocity (scattered!, hit.jl:17-25); the other kinds absorb.  Returns the
// absorbing surface or -1.  Times are fractions of the step: the x edge is
// reached after (1 - hx)/u or hx/|u| (the reference's Δh (1 - hx)/|v_x| over
// Δt, with Δh = Δy on the y axis).  Ties go to the y edge, as in check.jl:55.
__device__ __forceinline__ int track_path(const unsigned char *__restrict__ edge, const unsigned char *__restrict__ kinds,
                                       int nx, int ny, int i, int j, float hx, float hy, float &vx, float &vy,
                                       float &dX, float &dY) {
  float ux = dX, uy = dY, tau = 1.0f;
  for (int it = 0; it < 16; it++) {  // each pass crosses an edge; 16 bounds corner bounces
    const float tx = ux > 0.f ? __fdiv_rn(1.f - hx, ux) : (ux < 0.f ? __fdiv_rn(hx, -ux) : INFINITY);
    const float ty = uy > 0.f ? __fdiv_rn(1.f - hy, uy) : (uy < 0.f ? __fdiv_rn(hy, -uy) : INFINITY);
    if (tau < tx && tau < ty) return -1;  // stays in the cell
    if (i < 0 || j < 0 || i >= nx - 1 || j >= ny - 1) return -1;  // no surface outside the grid
    int dir, ni = i, nj = j;
    float t;
    if (tx < ty) {
      t = tx;
      dir = ux > 0.f ? kSurfDirXp : kSurfDirXm;
      ni += ux > 0.f ? 1 : -1;
    } else {
      t = ty;
      dir = uy > 0.f ? kSurfDirYp : kSurfDirYm;
      nj += uy > 0.f ? 1 : -1;
    }
    tau -= t;
    const int s = edge[4 * (i + nx * j) + dir];
    const bool xedge = dir <= kSurfDirXp;
    if (xedge) hy = fmaf(uy, t, hy);
    else hx = fmaf(ux, t, hx);
    if (s == 0) {  // no surface: on into the next cell
      if (xedge) hx = ux > 0.f ? 0.f : 1.f;
      else hy = uy > 0.f ? 0.f : 1.f;
      i = ni;
      j = nj;
      continue;
    }
    const int kind = kinds[s - 1];
    if (kind == ISKRA_SURF_PERIODIC) return -1;
    if (kind != ISKRA_SURF_REFLECT) return s - 1;
    if (xedge) {
      dX = fmaf(-2.f * ux, tau, dX);
      ux = -ux;
      vx = -vx;
      hx = dir == kSurfDirXp ? 1.f : 0.f;
    } else {
      dY = fmaf(-2.f * uy, tau, dY);
      uy = -uy;
      vy = -vy;
      hy = dir == kSurfDirYp ? 1.f : 0.f;
    }
  }
  return -1;
}

// after_push along one axis with P = n-1 cells (wrap period (n-1)Δh,
// wrap.jl:20-33; discard! removes α ≠ 0, wrap.jl:1-18).  Returns 0 = keep,
// 1 = absorbed at the low wall, 2 = absorbed at the high wall,
// 3 = out of the grid without a boundary rule.
template <int MODE>
__device__ __forceinline__ int apply_boundary(int &i, int P) {
  if (i >= 0 && i < P) return 0;
  if (MODE == ISKRA_BND_WRAP) {
    i %= P;
    if (i < 0) i += P;
    return 0;
  }
  if (MODE == ISKRA_BND_DISCARD) return i < 0 ? 1 : 2;
  return 3;
}

// Tile-block size of the push and the minimum resident blocks per SM asked
// of the register allocator, tuned on GB300 (interleaved 1000-step runs of
// the 512x512 slab, ring-staged push): 192-thread blocks, 5 per SM, ran
// 0.9 % faster than 128 x 7 and 0.2-0.5 % faster than 160 x 6, 256 x 4 and
// 192 x 6.  The ensemble push keeps 256 x 5.
#ifndef ISKRA_PUSH_THREADS
#define ISKRA_PUSH_THREADS 192
#endif
#ifndef ISKRA_PUSH_MIN_BLOCKS
#define ISKRA_PUSH_MIN_BLOCKS 5
#endif
#ifndef ISKRA_PUSH_TRK_MIN_BLOCKS  // the instantiation with a surface tracker
#define ISKRA_PUSH_TRK_MIN_BLOCKS ISKRA_PUSH_MIN_BLOCKS
#endif
#ifndef ISKRA_PUSH_RUNS_MIN_BLOCKS
#define ISKRA_PUSH_RUNS_MIN_BLOCKS 5
#endif
#ifndef ISKRA_PUSH_STAGES
#define ISKRA_PUSH_STAGES 4
#endif
// Each warp of a tile block streams its slice of particle records through a
// ring of kStages shared-memory stages filled by asynchronous copies
// (cp.async): kStages - 1 warp iterations (768 B each) are in flight while
// one is pushed, without holding registers for them.  With one iteration in
// flight per warp (register prefetch) the push was bound by the bytes in
// flight per SM; 4 stages (128-thread blocks, 7 per SM: 64 KB in flight)
// ran the 512x512 slab step 3.4 % faster, 3 stages 3 %, 5 stages (6
// blocks per SM) 2.6 %.
constexpr int kStages = ISKRA_PUSH_STAGES;

// Shared-memory window of a tile block: the tile's cells and a kHalo-cell
// margin (particles drift off their tile between sorts).
constexpr int kWin = kTile + 2 * kHalo;  // window cells per axis
constexpr int kWinN = kWin + 1;          // window nodes per axis
constexpr int kWinCells = kWin * kWin;

// Per window cell, the deposit moments n, Σu, Σv and Σuv of the particles
// deposited there (u, v < 2^24, uv < 2^48), each sum kept as 32-bit words
// of 16-bit pieces: a run of n particles adds Σu >> 16 and Σu & 0xffff,
// likewise Σv, and Σuv >> 32, (Σuv >> 16) & 0xffff, Σuv & 0xffff.  Every
// word then stays below (particles of the cell) 2^16, exact for up to 65535
// particles per cell (k_finalize rejects cells above kMaxCell), and all
// eight additions of a run are fire-and-forget shared-memory atomics (no
// returned value to wait for).  A cell holds at most kMaxCell particles, so
// Σu, Σv < 2^38 and Σuv < 2^62.
enum { kMomN, kMomU1, kMomU0, kMomV1, kMomV0, kMomQ2, kMomQ1, kMomQ0, kMoms };

// Shared memory of an ensemble-run block: E records of the run's cells.
struct PushShared {
  float4 e[2 * kWinCells];        // E records of the window cells
  unsigned mom[kMoms][kWinCells];  // deposit moments of the window cells
};

// Shared memory of a tile block: the warps' record rings, E at the window's
// nodes (a cell's four corner fields are four 8-byte loads; 3.5 KB instead
// of 12.8 KB of per-cell records) and the window moments.
// ISKRA_PUSH_BULK=1 fills the rings with TMA bulk copies instead of per-lane
// cp.async: measured on GB300 (512x512 slab, 300 steps, interleaved runs) at
// 0.1580 ms per step against 0.1500 (k_push2 at 56.4-57.1 % of HBM against
// 62.6-62.7 %): the per-warp mbarrier round trip on every 32-record stage
// costs more than the L1 instructions it saves.  Kept as a build option.
#ifndef ISKRA_PUSH_BULK
#define ISKRA_PUSH_BULK 0
#endif
#if ISKRA_PUSH_BULK
constexpr int kRbStage = 34;  // {vz, cell} records of a stage from the 16-byte boundary at or below its first slot
#else
constexpr int kRbStage = 32;
#endif
struct TileShared {
  float4 ra[ISKRA_PUSH_THREADS / 32][kStages][32];        // staged records {hx, hy, vx, vy}
  float2 rb[ISKRA_PUSH_THREADS / 32][kStages][kRbStage];  // staged records {vz, cell}
  unsigned long long bar[ISKRA_PUSH_THREADS / 32][kStages];  // stage mbarriers (bulk-copy ring)
  float2 ne[kWinN * kWinN];
  unsigned mom[kMoms][kWinCells];
  unsigned char trk[kWinCells];  // track! flags of the window cells (with a surface tracker)
};

// asynchronous global -> shared copies of one lane's record (L2 only for
// the 16-byte part; the 8-byte form exists only with L1 allocation)
__device__ __forceinline__ void cp_async_record(float4 *sa, float2 *sb, const float4 *ga, const float2 *gb) {
  const unsigned da = (unsigned)__cvta_generic_to_shared(sa), db = (unsigned)__cvta_generic_to_shared(sb);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(da), "l"(ga) : "memory");
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(db), "l"(gb) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// ---- bulk-copy ring (TMA 1-D copies, mbarrier completion) ----
// A stage of a warp's ring is filled by two cp.async.bulk copies issued by
// lane 0 -- the stage's 32 {hx, hy, vx, vy} records (512 B) and its {vz,
// cell} records from the 16-byte boundary at or below the first slot (34
// records, 272 B) -- which complete on the stage's mbarrier with their byte
// count.  The copies run on the TMA unit: no per-lane LSU instruction and no
// L1 pass for the streamed particle records.  Source: this GPU's own memory;
// no multicast.
constexpr unsigned kMbarSpins = 1u << 20;  // polls of one stage before DERR_TIMEOUT

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void bulk_stage(unsigned long long *bar, float4 *dst_a, float2 *dst_b, const float4 *src_a,
                                           const float2 *src_b) {
  const unsigned b = smem_u32(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(512u + 16u * (kRbStage / 2))
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], 512, [%2];" ::"r"(
                   smem_u32(dst_a)),
               "l"(src_a), "r"(b)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst_b)),
               "l"(src_b), "r"(8u * kRbStage), "r"(b)
               : "memory");
}

// waits for the phase `parity` of a stage; false after `spins` polls
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, unsigned spins) {
  const unsigned b = smem_u32(bar);
  for (unsigned it = 0; it < spins; it++) {
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

// E records (corner fields) of window cell (la, lb)
__device__ __forceinline__ void win_record(const PushShared &sh, int la, int lb, int ww, float4 &r0, float4 &r1) {
  const int w = la + ww * lb;
  r0 = sh.e[2 * w];
  r1 = sh.e[2 * w + 1];
}
// track! flag of window cell w (ensemble blocks run without a tracker)
__device__ __forceinline__ bool win_tracked(const PushShared &, int) { return false; }
__device__ __forceinline__ bool win_tracked(const TileShared &sh, int w) { return sh.trk[w] != 0; }
__device__ __forceinline__ void win_record(const TileShared &sh, int la, int lb, int, float4 &r0, float4 &r1) {
  const int n = la + kWinN * lb;
  const float2 a = sh.ne[n], b = sh.ne[n + 1], c = sh.ne[n + kWinN], d = sh.ne[n + kWinN + 1];
  r0 = make_float4(a.x, a.y, b.x, b.y);
  r1 = make_float4(c.x, c.y, d.x, d.y);
}

// a run of n particles of window cell `key` with sums su = Σu, sv = Σv and
// q = Σuv
template <class SH>
__device__ __forceinline__ void window_add(SH &sh, int key, unsigned n, unsigned long long su,
                                           unsigned long long sv, unsigned long long q) {
  atomicAdd(&sh.mom[kMomN][key], n);
  atomicAdd(&sh.mom[kMomU1][key], (unsigned)(su >> 16));
  atomicAdd(&sh.mom[kMomU0][key], (unsigned)su & 0xffffu);
  atomicAdd(&sh.mom[kMomV1][key], (unsigned)(sv >> 16));
  atomicAdd(&sh.mom[kMomV0][key], (unsigned)sv & 0xffffu);
  atomicAdd(&sh.mom[kMomQ2][key], (unsigned)(q >> 32));
  atomicAdd(&sh.mom[kMomQ1][key], (unsigned)(q >> 16) & 0xffffu);
  atomicAdd(&sh.mom[kMomQ0][key], (unsigned)q & 0xffffu);
}
template <class SH>
__device__ __forceinline__ void window_add(SH &sh, int key, unsigned n, const Moments &m) {
  window_add(sh, key, n, m.su, m.sv, ((unsigned long long)m.hi << 24) + m.lo);
}

// zeroes the window's moments (threads of the block, before its barrier)
template <class SH>
__device__ __forceinline__ void window_clear(SH &sh, int t) {
#pragma unroll
  for (int q = 0; q < kMoms; q++) sh.mom[q][t] = 0u;
}

// CIC node weights of window cell w: W00 at its lower-left node, W10, W01,
// W11
template <class SH>
__device__ __forceinline__ void window_cell(const SH &sh, int w, unsigned long long W[4]) {
  typedef unsigned long long u64;
  const u64 n = sh.mom[kMomN][w];
  const u64 su = ((u64)sh.mom[kMomU1][w] << 16) + sh.mom[kMomU0][w];
  const u64 sv = ((u64)sh.mom[kMomV1][w] << 16) + sh.mom[kMomV0][w];
  const u64 UV = ((u64)sh.mom[kMomQ2][w] << 32) + ((u64)sh.mom[kMomQ1][w] << 16) + sh.mom[kMomQ0][w];
  const u64 U = su << 24, V = sv << 24;
  W[0] = (n << 48) - U - V + UV;
  W[1] = U - UV;
  W[2] = V - UV;
  W[3] = UV;
}

// One warp step over the slots base + lane: gather, Boris push, boundary
// rules and the deposit of the new positions.  Cells inside the block's
// window (origin ox, oy) read E from and deposit into shared memory; other
// cells (particles that drifted off the window, the unsorted tail) use the
// global records and 64-bit atomics.  The deposit key is the window cell, or
// kWinCells + the global cell index, so runs never mix the two.
template <bool PUSH, int MX, int MY, bool WIN, bool TRK = false, class SH>
__device__ __forceinline__ int push_one(float4 *__restrict__ xv, float2 *__restrict__ zc, long long p, bool valid,
                                        float4 a, float2 b, const float2 *__restrict__ E2, const SH &sh,
                                        int ox, int oy, int ww, int wh, const PushParams &P, unsigned ab[4],
                                        int &flags, Moments &m, float4 *out_a = nullptr, float2 *out_b = nullptr) {
  const int nx = P.nx;
  int key = -1;
  m = Moments{0u, 0u, 0u, 0u};
  if (out_b) *out_b = make_float2(0.f, __int_as_float(-1));  // (no live particle unless pushed below)
  if (valid) {
    int cell = __float_as_int(b.y);
    if (cell >= 0) {
      int i0 = cell & 0xffff, j0 = cell >> 16;
      float hx = a.x, hy = a.y;
      unsigned ux, uy;  // offsets on the 2^-24 grid as integers
      if (PUSH) {
        float4 r0, r1;  // the cell's corner fields
        const int la = i0 - ox, lb = j0 - oy;
        const bool inwin = WIN && (unsigned)la < (unsigned)ww && (unsigned)lb < (unsigned)wh;
        if (inwin) {
          win_record(sh, la, lb, ww, r0, r1);
        } else {
          const int n0 = i0 + nx * j0;
          cell_record(E2, n0, nx, r0, r1);
        }
        // CIC weights and interpolation with explicitly rounded products and
        // fused sums, so that every kernel inlining this code (single species,
        // species pairs, ensemble runs) computes the same bits
        const float gx = __fsub_rn(1.0f, hx), gy = __fsub_rn(1.0f, hy);
        const float w00 = __fmul_rn(gx, gy), w10 = __fmul_rn(hx, gy);
        const float w01 = __fmul_rn(gx, hy), w11 = __fmul_rn(hx, hy);
        const float2 e00 = make_float2(r0.x, r0.y), e10 = make_float2(r0.z, r0.w);
        const float2 e01 = make_float2(r1.x, r1.y), e11 = make_float2(r1.z, r1.w);
        const float ex = fmaf(w00, e00.x, fmaf(w10, e10.x, fmaf(w01, e01.x, __fmul_rn(w11, e11.x))));
        const float ey = fmaf(w00, e00.y, fmaf(w10, e10.y, fmaf(w01, e01.y, __fmul_rn(w11, e11.y))));
        // Boris with B = 0: v- = v + hE ; v = hE + v+ (v+ = v-)
        float vx = fmaf(P.h, ex, a.z);
        float vy = fmaf(P.h, ey, a.w);
        vx = fmaf(P.h, ex, vx);
        vy = fmaf(P.h, ey, vy);
        if (!isfinite(vx) || !isfinite(vy)) {
          flags |= DERR_NAN;
          cell = -1;
        } else {
          float dX = __fmul_rn(vx, P.dtdx), dY = __fmul_rn(vy, P.dtdy);
          int hit = -1;
          if (TRK && (inwin ? win_tracked(sh, la + ww * lb) : P.trk_cell[i0 + nx * j0] != 0))
            hit = track_path(P.trk_edge, P.trk_kind, nx, P.ny, i0, j0, hx, hy, vx, vy, dX, dY);
          if (hit >= 0) {  // absorbed by a surface: removed like a discarded particle
            atomicAdd(P.trk_hits + hit, 1ull);
            cell = -1;
          } else {
            hx = move_axis(hx, dX, i0, ux);
            hy = move_axis(hy, dY, j0, uy);
            int rx = apply_boundary<MX>(i0, nx - 1);
            int ry = rx ? 0 : apply_boundary<MY>(j0, P.ny - 1);
            if (rx == 3 || ry == 3) {
              flags |= DERR_DOMAIN;
              cell = -1;
            } else if (rx) {
              ab[rx - 1]++;
              cell = -1;
            } else if (ry) {
              ab[ry + 1]++;
              cell = -1;
            } else {
              cell = i0 | (j0 << 16);
            }
          }
        }
        __stcs(xv + p, make_float4(hx, hy, vx, vy));
        __stcs(zc + p, make_float2(b.x, __int_as_float(cell)));
        if (out_a) {  // the pushed record, for a caller that selects it for the next MCC step
          *out_a = make_float4(hx, hy, vx, vy);
          *out_b = make_float2(b.x, __int_as_float(cell));
        }
      }
      if (cell >= 0) {
        const int la = i0 - ox, lb = j0 - oy;
        key = (WIN && (unsigned)la < (unsigned)ww && (unsigned)lb < (unsigned)wh) ? la + ww * lb
                                                                                  : kWinCells + i0 + nx * j0;
        if (!PUSH) {
          ux = __float2uint_rn(hx * kOffScale);
          uy = __float2uint_rn(hy * kOffScale);
        }
        const unsigned long long uv = (unsigned long long)ux * uy;
        m.su = ux;
        m.sv = uy;
        m.hi = (unsigned)(uv >> 24);
        m.lo = (unsigned)uv & 0xffffffu;
      }
    }
  }
  return key;
}

// Warp-collective deposit of one particle per lane (key from push_one).
template <bool WIN, class SH>
__device__ __forceinline__ void deposit_warp(const SpeciesDev &s, SH &sh, int key, Moments m, int nx) {
  unsigned n;
  if (reduce_runs(key, m, n) && key >= 0) {
    if (WIN && key < kWinCells) {
      window_add(sh, key, n, m);
    } else {
      const unsigned long long U = (unsigned long long)m.su << 24, V = (unsigned long long)m.sv << 24;
      const unsigned long long UV = ((unsigned long long)m.hi << 24) + m.lo;
      const int g = key - kWinCells;
      atomicAdd(s.acc + g, ((unsigned long long)n << 48) - U - V + UV);
      atomicAdd(s.acc + g + 1, U - UV);
      atomicAdd(s.acc + g + nx, V - UV);
      atomicAdd(s.acc + g + nx + 1, UV);
      atomicAdd(s.cnt + g, n);
    }
  }
}

template <bool PUSH, int MX, int MY, bool WIN, bool TRK = false, class SH>
__device__ __forceinline__ void push_warp(const SpeciesDev &s, float4 *__restrict__ xv, float2 *__restrict__ zc,
                                          long long p, bool valid, float4 a, float2 b,
                                          const float2 *__restrict__ E2, SH &sh, int ox, int oy, int ww,
                                          int wh, const PushParams &P, unsigned ab[4], int &flags,
                                          float4 *out_a = nullptr, float2 *out_b = nullptr) {
  Moments m;
  const int key = push_one<PUSH, MX, MY, WIN, TRK>(xv, zc, p, valid, a, b, E2, sh, ox, oy, ww, wh, P, ab, flags, m,
                                                   out_a, out_b);
  deposit_warp<WIN>(s, sh, key, m, P.nx);
}

// One block of the push: a tile block (tile >= 0) takes the particles the
// last sort grouped in its tile: stage E at the window's nodes, push (each
// warp a contiguous slice, streamed through its record ring), deposit into
// the window, then add the window's nonzero node sums and cell counts to
// the global accumulators.  A tail block (tile < 0, tail_block of
// tail_blocks) walks the slots appended since that sort.  Integer sums: the
// density is the same bit for bit whichever block adds what.
template <bool PUSH, int MX, int MY, bool TRK = false>
__device__ __forceinline__ void push_block(const SpeciesDev &s, const PushParams &P, const float2 *__restrict__ E2,
                                           TileShared &sh, int tile, int tail_block, int tail_blocks, int *err) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  const int cur = s.st->cur;
  float4 *__restrict__ xv = pick(s.xv[0], s.xv[1], cur);
  float2 *__restrict__ zc = pick(s.zc[0], s.zc[1], cur);
  unsigned ab[4] = {0, 0, 0, 0};
  int flags = 0;
  const int nx = P.nx;
  if (tile >= 0) {
    const long long begin = s.tile_begin[tile], end = s.tile_begin[tile + 1];
    if (begin < end) {  // block-uniform
      const int ox = (tile % P.tiles_x) * kTile - kHalo, oy = (tile / P.tiles_x) * kTile - kHalo;
      if (PUSH) {
        for (int t = threadIdx.x; t < kWinN * kWinN; t += blockDim.x) {
          const int i = ox + t % kWinN, j = oy + t / kWinN;
          sh.ne[t] = (i >= 0 && i < nx && j >= 0 && j < P.ny) ? __ldg(E2 + i + nx * j) : make_float2(0.f, 0.f);
        }
      }
      for (int t = threadIdx.x; t < kWinCells; t += blockDim.x) {
        window_clear(sh, t);
        if (TRK) {
          const int i = ox + t % kWin, j = oy + t / kWin;
          sh.trk[t] = (i >= 0 && i < nx - 1 && j >= 0 && j < P.ny - 1) ? P.trk_cell[i + nx * j] : 0;
        }
      }
      __syncthreads();
      // each warp takes a contiguous slice of the tile's slots (cell-sorted
      // slices touch few cells in common)
      const long long len = end - begin;
      const long long slice = ((len + nwb * 32 - 1) / (nwb * 32)) * 32;
      const long long w0 = begin + wib * slice;
      // the warp's slice as pointers and a 32-bit count (a tile holds far
      // fewer than 2^31 slots): 32-bit loop arithmetic
      const int cnt = (int)max(0LL, min(end, w0 + slice) - w0);
      float4 *__restrict__ xw = xv + w0;
      float2 *__restrict__ zw = zc + w0;
#if ISKRA_PUSH_BULK
      // {vz, cell} stages start at the 16-byte boundary at or below their
      // first slot: w0 + o has the parity of `begin` (slices and stages are
      // multiples of 32 slots)
      const int sft = (int)(begin & 1);
      if (lane == 0) {
#pragma unroll
        for (int d = 0; d < kStages; d++) mbar_init(&sh.bar[wib][d], 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      }
      __syncwarp();
      if (lane == 0) {  // prologue: the first kStages - 1 iterations' records in flight
#pragma unroll
        for (int d = 0; d < kStages - 1; d++)
          if (32 * d < cnt) bulk_stage(&sh.bar[wib][d], sh.ra[wib][d], sh.rb[wib][d], xw + 32 * d, zw + 32 * d - sft);
      }
      unsigned phase = 0u;  // bit st: parity of stage st's next completion
      int st = 0;           // stage of the current iteration
      for (int o = 0; o < cnt; o += 32) {
        __syncwarp();  // every lane has read the stage refilled next (one iteration ago)
        {
          const int q = o + 32 * (kStages - 1);
          const int sn = st == 0 ? kStages - 1 : st - 1;
          if (lane == 0 && q < cnt) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the reads precede the copy's writes
            bulk_stage(&sh.bar[wib][sn], sh.ra[wib][sn], sh.rb[wib][sn], xw + q, zw + q - sft);
          }
        }
        // bounded: a stage that never completes is flagged and its records
        // skipped; the later stages are still waited for (each bounded), so
        // no copy is in flight when the block leaves the ring
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&sh.bar[wib][st], (phase >> st) & 1u, kMbarSpins));
        if (!ok) flags |= DERR_TIMEOUT;
        phase ^= 1u << st;
        const float4 a = sh.ra[wib][st][lane];
        const float2 b = sh.rb[wib][st][lane + sft];
        st = st + 1 == kStages ? 0 : st + 1;
        push_warp<PUSH, MX, MY, true, TRK>(s, xw, zw, o + lane, ok && o + lane < cnt, a, b, E2, sh, ox, oy, kWin,
                                           kWin, P, ab, flags);
      }
      __syncthreads();
#else
      // prologue: the first kStages - 1 iterations' records in flight
#pragma unroll
      for (int d = 0; d < kStages - 1; d++) {
        const int q = 32 * d + lane;
        if (q < cnt) cp_async_record(&sh.ra[wib][d][lane], &sh.rb[wib][d][lane], xw + q, zw + q);
        cp_async_commit();
      }
      int st = 0;  // stage of the current iteration
      for (int o = 0; o < cnt; o += 32) {
        {
          const int q = o + 32 * (kStages - 1) + lane;
          const int sn = st == 0 ? kStages - 1 : st - 1;  // the stage read one iteration ago
          if (q < cnt) cp_async_record(&sh.ra[wib][sn][lane], &sh.rb[wib][sn][lane], xw + q, zw + q);
          cp_async_commit();
        }
        cp_async_wait<kStages - 1>();  // this lane's copies of the current stage have landed
        const float4 a = sh.ra[wib][st][lane];
        const float2 b = sh.rb[wib][st][lane];
        st = st + 1 == kStages ? 0 : st + 1;
        push_warp<PUSH, MX, MY, true, TRK>(s, xw, zw, o + lane, o + lane < cnt, a, b, E2, sh, ox, oy, kWin, kWin, P,
                                           ab, flags);
      }
      cp_async_wait<0>();
      __syncthreads();
#endif
      // node sums from the moments of the up to four window cells around each node
      for (int t = threadIdx.x; t < kWinN * kWinN; t += blockDim.x) {
        const int a = t % kWinN, b = t / kWinN;
        unsigned long long v = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int ca = a - (c & 1), cb = b - (c >> 1);  // cell whose corner (c & 1, c >> 1) is this node
          if (ca < 0 || cb < 0 || ca >= kWin || cb >= kWin) continue;
          const int w = ca + kWin * cb;
          if (!sh.mom[kMomN][w]) continue;
          unsigned long long W[4];
          window_cell(sh, w, W);
          v += W[c];
        }
        if (v) atomicAdd(s.acc + (ox + a) + nx * (oy + b), v);
      }
      for (int t = threadIdx.x; t < kWinCells; t += blockDim.x) {
        const unsigned v = sh.mom[kMomN][t];
        if (v) atomicAdd(s.cnt + (ox + t % kWin) + nx * (oy + t / kWin), v);
      }
    }
  } else {
    const long long np = s.st->np, t0 = s.st->sorted_n;
    const long long warp = (long long)tail_block * nwb + wib;
    const long long nwarps = (long long)tail_blocks * nwb;
    for (long long base = t0 + warp * 32; base < np; base += nwarps * 32) {
      const long long p = base + lane;
      const bool v = p < np;
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
      float2 b = make_float2(0.f, 0.f);
      if (v) {
        a = ld_stream(xv + p);
        b = ld_stream(zc + p);
      }
      push_warp<PUSH, MX, MY, false, TRK>(s, xv, zc, p, v, a, b, E2, sh, 0, 0, 0, 0, P, ab, flags);
    }
  }
  if (PUSH) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      unsigned t = __reduce_add_sync(FULL, ab[k]);
      if (lane == 0 && t) atomicAdd(&s.st->absorbed[k], (unsigned long long)t);
    }
    int f = __reduce_or_sync(FULL, flags);
    if (lane == 0 && f) atomicOr(err, f);
  }
}

// TRK: with the surface tracker (a separate instantiation keeps the walk's
// registers out of the push without one)
template <bool PUSH, int MX, int MY, bool TRK = false>
__global__ void __launch_bounds__(ISKRA_PUSH_THREADS, TRK ? ISKRA_PUSH_TRK_MIN_BLOCKS : ISKRA_PUSH_MIN_BLOCKS)
    k_push(SpeciesDev s, const float2 *__restrict__ E2, PushParams P, int ntiles, int *err) {
  pdl_wait();
  __shared__ TileShared sh;
  const int b = blockIdx.x;
  if (b < ntiles) push_block<PUSH, MX, MY, TRK>(s, P, E2, sh, b, 0, 0, err);
  else push_block<PUSH, MX, MY, TRK>(s, P, E2, sh, -1, b - ntiles, gridDim.x - ntiles, err);
}

// Two species in one launch (the step's electrons and ions): their pushes
// are independent until ρ is formed, so the second species' tiles fill the
// SMs as the first species' tiles drain instead of waiting for a second
// launch.  Blocks [0, ntiles) first species' tiles, [ntiles, 2 ntiles) the
// second's, the rest both tails.
// step_ctr (optional): the step counter, advanced here when no MCC set reads
// it earlier in the step (saves the step's opening launch).
template <int MX, int MY, bool TRK = false>
__global__ void __launch_bounds__(ISKRA_PUSH_THREADS, TRK ? ISKRA_PUSH_TRK_MIN_BLOCKS : ISKRA_PUSH_MIN_BLOCKS)
    k_push2(SpeciesDev s0, SpeciesDev s1, const float2 *__restrict__ E2, PushParams P0, PushParams P1, int ntiles,
            int *err, unsigned long long *step_ctr) {
  pdl_wait();
  __shared__ TileShared sh;
  const int b = blockIdx.x;
  if (step_ctr && b == 0 && threadIdx.x == 0) *step_ctr += 1ull;
  if (b < ntiles) {
    push_block<true, MX, MY, TRK>(s0, P0, E2, sh, b, 0, 0, err);
  } else if (b < 2 * ntiles) {
    push_block<true, MX, MY, TRK>(s1, P1, E2, sh, b - ntiles, 0, 0, err);
  } else {
    const int tb = b - 2 * ntiles, nt = gridDim.x - 2 * ntiles;
    push_block<true, MX, MY, TRK>(s0, P0, E2, sh, -1, tb, nt, err);
    push_block<true, MX, MY, TRK>(s1, P1, E2, sh, -1, tb, nt, err);
  }
}

static cudaError_t launch_push_modes(Ctx *c, Species &s, PushParams P, int blocks) {
  const int T = ISKRA_PUSH_THREADS;
#define ISKRA_PUSH_CASE(MX, MY)                                                                       \
  if (P.mode_x == MX && P.mode_y == MY) {                                                             \
    auto kern = c->trk ? k_push<true, MX, MY, true> : k_push<true, MX, MY, false>;                   \
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                        \
                         (int)cudaSharedmemCarveoutMaxShared);                                        \
    return launch_pdl(kern, blocks, T, 0, c->stream, s.dev, (const float2 *)c->E32, P, c->ntiles,     \
                      c->d_err);                                                                      \
  }
  ISKRA_PUSH_CASE(0, 0) ISKRA_PUSH_CASE(0, 1) ISKRA_PUSH_CASE(0, 2)
  ISKRA_PUSH_CASE(1, 0) ISKRA_PUSH_CASE(1, 1) ISKRA_PUSH_CASE(1, 2)
  ISKRA_PUSH_CASE(2, 0) ISKRA_PUSH_CASE(2, 1) ISKRA_PUSH_CASE(2, 2)
#undef ISKRA_PUSH_CASE
  return cudaErrorInvalidValue;
}

// one block per tile plus a grid-stride set for the unsorted tail
static int push_blocks(Ctx *c) { return c->ntiles + c->num_sms; }

static int sort_blocks(Ctx *c, Species &s) {
  long long want = (s.cap + 255) / 256;
  long long maxb = (long long)c->num_sms * 8;
  if (want < 1) want = 1;
  return (int)(want < maxb ? want : maxb);
}

static PushParams push_params(Ctx *c, const Species &s, float dt) {
  PushParams P{};
  P.h = (float)(0.5 * (double)dt * (s.q / s.m));
  P.dtdx = (float)((double)dt / c->g.dx);
  P.dtdy = (float)((double)dt / c->g.dy);
  P.nx = c->nx;
  P.ny = c->ny;
  P.mode_x = s.bnd[0];
  P.mode_y = s.bnd[1];
  P.tiles_x = c->tiles_x;
  P.trk_edge = nullptr;
  P.trk_cell = nullptr;
  P.trk_kind = nullptr;
  P.trk_hits = nullptr;
  if (c->trk) {
    P.trk_edge = c->trk->d_edge;
    P.trk_cell = c->trk->d_cell;
    P.trk_kind = c->trk->d_kind;
    P.trk_hits = c->trk->d_hits + (size_t)(&s - c->species.data()) * kMaxSurfaces;
  }
  return P;
}

// a species' accumulator before its push: cleared unless known zero
static int clear_acc(Ctx *c, Species &s) {
  if (s.acc_zero) return ISKRA_OK;
  ISKRA_CUDA(c, cudaMemsetAsync(s.dev.acc, 0, (size_t)c->nn * sizeof(unsigned long long), c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(s.dev.cnt, 0, (size_t)c->nn * sizeof(unsigned), c->stream));
  return ISKRA_OK;
}

static void mark_pushed(Species &s) {
  s.acc_valid = true;  // accumulator = deposit of the pushed positions (unconsumed)
  s.acc_zero = false;
  s.n_valid = false;
}

int launch_advance(Ctx *c, int sid, float dt) {
  Species &s = c->species[sid];
  int rc = clear_acc(c, s);
  if (rc) return rc;
  ISKRA_CUDA(c, launch_push_modes(c, s, push_params(c, s, dt), push_blocks(c)));
  ISKRA_CUDA(c, cudaGetLastError());
  mark_pushed(s);
  return launch_surface_charge(c);  // hit! of floating electrodes, as part of advance!
}

// Every species of a step: two species with the same boundary rules in one
// launch (k_push2, which also advances step_ctr when given: *folded), otherwise
// one launch each.
int launch_advance_all(Ctx *c, float dt, unsigned long long *step_ctr, bool *folded) {
  if (folded) *folded = false;
  const int ns = (int)c->species.size();
  if (ns == 2 && c->species[0].bnd[0] == c->species[1].bnd[0] && c->species[0].bnd[1] == c->species[1].bnd[1]) {
    Species &a = c->species[0], &b = c->species[1];
    int rc = clear_acc(c, a);
    if (!rc) rc = clear_acc(c, b);
    if (rc) return rc;
    const PushParams Pa = push_params(c, a, dt), Pb = push_params(c, b, dt);
    const int blocks = 2 * c->ntiles + c->num_sms;
    cudaError_t e = cudaErrorInvalidValue;
#define ISKRA_PUSH2_CASE(MX, MY)                                                                           \
  if (Pa.mode_x == MX && Pa.mode_y == MY) {                                                                \
    auto kern = c->trk ? k_push2<MX, MY, true> : k_push2<MX, MY, false>;                                  \
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                             \
                         (int)cudaSharedmemCarveoutMaxShared);                                             \
    e = launch_pdl(kern, blocks, ISKRA_PUSH_THREADS, 0, c->stream, a.dev, b.dev, (const float2 *)c->E32,   \
                   Pa, Pb, c->ntiles, c->d_err, step_ctr);                                                 \
  }
    ISKRA_PUSH2_CASE(0, 0) ISKRA_PUSH2_CASE(0, 1) ISKRA_PUSH2_CASE(0, 2)
    ISKRA_PUSH2_CASE(1, 0) ISKRA_PUSH2_CASE(1, 1) ISKRA_PUSH2_CASE(1, 2)
    ISKRA_PUSH2_CASE(2, 0) ISKRA_PUSH2_CASE(2, 1) ISKRA_PUSH2_CASE(2, 2)
#undef ISKRA_PUSH2_CASE
    ISKRA_CUDA(c, e);
    ISKRA_CUDA(c, cudaGetLastError());
    mark_pushed(a);
    mark_pushed(b);
    if (folded) *folded = step_ctr != nullptr;
    return launch_surface_charge(c);
  }
  for (int s = 0; s < ns; s++) {
    int rc = launch_advance(c, s, dt);
    if (rc) return rc;
  }
  return ISKRA_OK;
}

int launch_deposit(Ctx *c, int sid) {
  Species &s = c->species[sid];
  if (!s.acc_zero) {
    ISKRA_CUDA(c, cudaMemsetAsync(s.dev.acc, 0, (size_t)c->nn * sizeof(unsigned long long), c->stream));
    ISKRA_CUDA(c, cudaMemsetAsync(s.dev.cnt, 0, (size_t)c->nn * sizeof(unsigned), c->stream));
  }
  PushParams P{};
  P.nx = c->nx;
  P.ny = c->ny;
  P.tiles_x = c->tiles_x;
  cudaFuncSetAttribute(k_push<false, 0, 0>, cudaFuncAttributePreferredSharedMemoryCarveout,
                       (int)cudaSharedmemCarveoutMaxShared);
  k_push<false, 0, 0><<<push_blocks(c), ISKRA_PUSH_THREADS, 0, c->stream>>>(s.dev, c->E32, P, c->ntiles, c->d_err);
  ISKRA_CUDA(c, cudaGetLastError());
  s.acc_valid = true;
  s.acc_zero = false;
  return ISKRA_OK;
}

// ---------------------------------------------------------------------------
// density + charge density
// ---------------------------------------------------------------------------
struct FinalizeArgs {
  int ns;
  unsigned long long *acc[kMaxSpecies];
  unsigned *cnt[kMaxSpecies];
  double *n[kMaxSpecies];
  double scale[kMaxSpecies];  // w0 * 2^-48
  double q[kMaxSpecies];
  int consume[kMaxSpecies];
};



__global__ void k_finalize(FinalizeArgs A, const double *__restrict__ vol_inv, const double *__restrict__ bg,
                           double *__restrict__ rho, int nn, int *err) {
  pdl_wait();
  int flags = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    // all loads of the node first (independent, in flight together), then the
    // arithmetic and the stores
    const double vi = vol_inv[k];
    const double b = bg ? bg[k] : 0.0;
    unsigned long long a[kMaxSpecies];
    unsigned cn[kMaxSpecies];
    double nold[kMaxSpecies];
#pragma unroll
    for (int s = 0; s < kMaxSpecies; s++) {
      if (s >= A.ns) break;
      if (A.consume[s]) {
        a[s] = A.acc[s][k];
        cn[s] = A.cnt[s][k];
      } else {
        nold[s] = A.n[s][k];
      }
    }
    double r = 0.0;
#pragma unroll
    for (int s = 0; s < kMaxSpecies; s++) {
      if (s >= A.ns) break;
      double n;
      if (A.consume[s]) {
        if (cn[s] > kMaxCell) flags |= DERR_OVERFLOW;
        n = (double)a[s] * A.scale[s] * vi;
        A.n[s][k] = n;
        A.acc[s][k] = 0ull;
        A.cnt[s][k] = 0u;
      } else {
        n = nold[s];
      }
      r += n * A.q[s];
    }
    if (rho) rho[k] = r + b;
  }
  if (flags) atomicOr(err, flags);
}

// The same in double-float arithmetic on the FP32 pipes (GB300 runs FP64 at
// ~1/64 of its FP32 rate): the int64 sums split exactly into three FP32
// pieces, products by two-product FMA; ρ and the densities to ~2^-48
// relative, written as double-float pairs (FP64 copies on download).
// WARM: the step solve's warm start on the same nodes (ϕ <- 2ϕ_n - ϕ_(n-1)
// on free rows once the history is valid; the last block marks it valid)
template <bool WARM>
__global__ void k_finalize_df(FinalizeDfArgs A, const float2 *__restrict__ vol_inv, const float2 *__restrict__ bg,
                              float2 *__restrict__ rho, int nn, int *err, WarmArgs W) {
  pdl_wait();
  __shared__ int last;
  const bool hist = WARM && *W.hist != 0;
  int flags = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    finalize_df_node(A, vol_inv, bg, rho, k, flags);
    if (WARM) warm_node(W, hist, k);
  }
  if (flags) atomicOr(err, flags);
  if (WARM) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      last = atomicAdd(W.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
      *W.ticket = 0u;
      *W.hist = 1;
    }
  }
}

__global__ void k_df_to_f64(const float2 *__restrict__ a, double *__restrict__ b, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    b[k] = (double)a[k].x + (double)a[k].y;
}
__global__ void k_f64_to_df(const double *__restrict__ a, float2 *__restrict__ b, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float h = (float)a[k];
    b[k] = make_float2(h, (float)(a[k] - (double)h));
  }
}

static int node_blocks(Ctx *c) { return std::max(1, std::min(c->num_sms * 4, (c->nn + 255) / 256)); }

// FP64 copies on demand
int sync_rho64(Ctx *c) {
  if (c->rho64_valid) return ISKRA_OK;
  k_df_to_f64<<<node_blocks(c), 256, 0, c->stream>>>(c->rho_df, c->rho, c->nn);
  ISKRA_CUDA(c, cudaGetLastError());
  c->rho64_valid = true;
  return ISKRA_OK;
}
static int sync_n64(Ctx *c, Species &sp) {
  if (sp.n64_valid) return ISKRA_OK;
  k_df_to_f64<<<node_blocks(c), 256, 0, c->stream>>>(sp.n_df, sp.n, c->nn);
  ISKRA_CUDA(c, cudaGetLastError());
  sp.n64_valid = true;
  return ISKRA_OK;
}

// Brings every species' density up to date (depositing species whose
// positions changed without a deposit, consuming unconsumed accumulators) and,
// when with_rho, forms ρ -- in double-float when the next solve takes it so
// (separable operator with a double-float state), else in FP64.
static int finalize(Ctx *c, bool with_rho, bool step = false) {
  const bool df = with_rho && poisson_df_rho(c);
  c->warm_fused = false;
  FinalizeArgs A{};
  FinalizeDfArgs D{};
  A.ns = D.ns = (int)c->species.size();
  bool any = false;
  for (int s = 0; s < A.ns; s++) {
    Species &sp = c->species[s];
    if (!sp.acc_valid && !sp.n_valid) {
      int rc = launch_deposit(c, s);
      if (rc) return rc;
    }
    if (!sp.acc_valid) {  // the stored density enters: in the form this pass reads
      if (df && !sp.n_df_valid) {
        k_f64_to_df<<<node_blocks(c), 256, 0, c->stream>>>(sp.n, sp.n_df, c->nn);
        sp.n_df_valid = true;
      } else if (!df) {
        int rc = sync_n64(c, sp);
        if (rc) return rc;
      }
    }
    A.acc[s] = D.acc[s] = sp.dev.acc;
    A.cnt[s] = D.cnt[s] = sp.dev.cnt;
    A.n[s] = sp.n;
    D.n[s] = sp.n_df;
    A.scale[s] = sp.w0 * ldexp(1.0, -48);
    D.scale[s] = df_host(A.scale[s]);
    A.q[s] = sp.q;
    D.q[s] = df_host(sp.q);
    A.consume[s] = D.consume[s] = sp.acc_valid ? 1 : 0;
    any |= sp.acc_valid;
  }
  if (!any && !with_rho) return ISKRA_OK;
  if (df) {
    WarmArgs W{};
    if (step && poisson_warm_args(c, &W)) {
      ISKRA_CUDA(c, launch_pdl(k_finalize_df<true>, node_blocks(c), 256, 0, c->stream, D,
                               (const float2 *)c->vol_inv_df, (const float2 *)c->bg_df, c->rho_df, c->nn, c->d_err, W));
      c->warm_fused = true;
    } else {
      ISKRA_CUDA(c, launch_pdl(k_finalize_df<false>, node_blocks(c), 256, 0, c->stream, D,
                               (const float2 *)c->vol_inv_df, (const float2 *)c->bg_df, c->rho_df, c->nn, c->d_err, W));
    }
    c->rho_df_valid = true;
    c->rho64_valid = false;
  } else {
    ISKRA_CUDA(c, launch_pdl(k_finalize, node_blocks(c), 256, 0, c->stream, A, (const double *)c->vol_inv,
                             (const double *)c->rho_bg, with_rho ? c->rho : nullptr, c->nn, c->d_err));
    if (with_rho) {
      c->rho64_valid = true;
      c->rho_df_valid = false;
    }
  }
  ISKRA_CUDA(c, cudaGetLastError());
  for (int s = 0; s < A.ns; s++) {
    Species &sp = c->species[s];
    if (sp.acc_valid) {
      sp.acc_valid = false;
      sp.acc_zero = true;
      sp.n64_valid = !df;
      sp.n_df_valid = df;
    }
    sp.n_valid = true;
  }
  return ISKRA_OK;
}

int launch_charge_density(Ctx *c) { return finalize(c, true); }
int launch_step_density(Ctx *c) { return finalize(c, true, true); }


// ---------------------------------------------------------------------------
// E = -∇ϕ  (generalized_poisson.jl:398-410)
// ---------------------------------------------------------------------------
__global__ void k_efield(const double *__restrict__ phi, int nx, int ny, double idx2, double idx1, double idy2,
                         double idy1, float2 *__restrict__ E32, double *__restrict__ E64) {
  const int nn = nx * ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int i = k % nx, j = k / nx;
    double ex, ey;
    if (i == 0) ex = (phi[k] - phi[k + 1]) * idx1;
    else if (i == nx - 1) ex = (phi[k - 1] - phi[k]) * idx1;
    else ex = (phi[k - 1] - phi[k + 1]) * idx2;
    if (j == 0) ey = (phi[k] - phi[k + nx]) * idy1;
    else if (j == ny - 1) ey = (phi[k - nx] - phi[k]) * idy1;
    else ey = (phi[k - nx] - phi[k + nx]) * idy2;
    if (E32) E32[k] = make_float2((float)ex, (float)ey);
    E64[k] = ex;
    E64[k + nn] = ey;
    E64[k + 2 * nn] = 0.0;
  }
}

int launch_efield_from(Ctx *c, const double *phi) {
  int blocks = c->num_sms * 4;
  int need = (c->nn + 255) / 256;
  if (need < blocks) blocks = need;
  k_efield<<<blocks, 256, 0, c->stream>>>(phi, c->nx, c->ny, 1.0 / (2 * c->g.dx), 1.0 / c->g.dx,
                                          1.0 / (2 * c->g.dy), 1.0 / c->g.dy, c->E32, c->E64);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// FP64 E of ϕ for download only: the FP32 gather fields stay as the solve left them
int launch_efield64(Ctx *c, const double *phi) {
  int blocks = c->num_sms * 4;
  int need = (c->nn + 255) / 256;
  if (need < blocks) blocks = need;
  k_efield<<<blocks, 256, 0, c->stream>>>(phi, c->nx, c->ny, 1.0 / (2 * c->g.dx), 1.0 / c->g.dx,
                                          1.0 / (2 * c->g.dy), 1.0 / c->g.dy, nullptr, c->E64);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// ---------------------------------------------------------------------------
// counting sort by cell (histogram -> exclusive scan -> scatter), dropping
// discarded particles
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_hist(SpeciesDev s, int tiles_x, int *__restrict__ count) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long np = s.st->np;
  const int cur = s.st->cur;
  const float2 *__restrict__ zc = pick(s.zc[0], s.zc[1], cur);
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = warp * 32; base < np; base += nwarps * 32) {
    const long long p = base + lane;
    int key = -1;
    if (p < np) {
      int cell = __float_as_int(zc[p].y);
      if (cell >= 0) key = cell_key(cell & 0xffff, cell >> 16, tiles_x);
    }
    unsigned peers = __match_any_sync(FULL, key);
    if (key >= 0 && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(count + key, __popc(peers));
  }
}

// exclusive scan in three phases; block = 1024 threads x 4 items
constexpr int kScanItems = 4096;

__device__ __forceinline__ int block_scan_excl(int v, int *sh, int &total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int y = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += t;
    }
    sh[lane] = y;  // inclusive warp prefix
  }
  __syncthreads();
  int off = wid ? sh[wid - 1] : 0;
  total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return off + x - v;
}

__global__ void __launch_bounds__(1024) k_scan_reduce(const int *__restrict__ in, int n, int *__restrict__ part) {
  __shared__ int sh[32];
  long long b0 = (long long)blockIdx.x * kScanItems;
  int v = 0;
  for (int k = 0; k < 4; k++) {
    long long idx = b0 + threadIdx.x * 4 + k;
    if (idx < n) v += in[idx];
  }
  int tot;
  block_scan_excl(v, sh, tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_top(int *__restrict__ part, int nb) {
  __shared__ int sh[32];
  int carry = 0;
  for (int b = 0; b < nb; b += 1024) {
    int idx = b + threadIdx.x;
    int v = idx < nb ? part[idx] : 0;
    int tot;
    int e = block_scan_excl(v, sh, tot);
    if (idx < nb) part[idx] = e + carry;
    carry += tot;
    __syncthreads();
  }
}

// out = exclusive scan of in (n + 1 entries, the last the total); tile_begin
// receives the entries at the multiples of kTile^2 (the first slot of each tile)
__global__ void __launch_bounds__(1024) k_scan_down(const int *__restrict__ in, int n, const int *__restrict__ part,
                                                    int *__restrict__ out, int *__restrict__ tile_begin) {
  __shared__ int sh[32];
  long long b0 = (long long)blockIdx.x * kScanItems;
  int v[4];
  int sum = 0;
  for (int k = 0; k < 4; k++) {
    long long idx = b0 + threadIdx.x * 4 + k;
    v[k] = idx < n ? in[idx] : 0;
    sum += v[k];
  }
  int tot;
  int e = block_scan_excl(sum, sh, tot) + part[blockIdx.x];
  constexpr int kKeysPerTile = kTile * kTile;
  for (int k = 0; k < 4; k++) {
    long long idx = b0 + threadIdx.x * 4 + k;
    if (idx < n) {
      out[idx] = e;
      if (idx % kKeysPerTile == 0) tile_begin[idx / kKeysPerTile] = e;
    }
    e += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) {  // grand total
    out[n] = e;
    tile_begin[n / kKeysPerTile] = e;
  }
}

__global__ void __launch_bounds__(256) k_scatter(SpeciesDev s, int tiles_x, int *__restrict__ cursor) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long np = s.st->np;
  const int cur = s.st->cur;
  const float4 *__restrict__ xv = pick(s.xv[0], s.xv[1], cur);
  const float2 *__restrict__ zc = pick(s.zc[0], s.zc[1], cur);
  const uint32_t *__restrict__ id = pick(s.id[0], s.id[1], cur);
  float4 *__restrict__ xo = pick(s.xv[0], s.xv[1], cur ^ 1);
  float2 *__restrict__ zo = pick(s.zc[0], s.zc[1], cur ^ 1);
  uint32_t *__restrict__ io = pick(s.id[0], s.id[1], cur ^ 1);
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = warp * 32; base < np; base += nwarps * 32) {
    const long long p = base + lane;
    int key = -1;
    float4 a;
    float2 b;
    uint32_t pid = 0;
    if (p < np) {
      a = xv[p];
      b = zc[p];
      pid = id[p];
      int cell = __float_as_int(b.y);
      if (cell >= 0) key = cell_key(cell & 0xffff, cell >> 16, tiles_x);
    }
    unsigned peers = __match_any_sync(FULL, key);
    int leader = __ffs(peers) - 1;
    int rank = __popc(peers & ((1u << lane) - 1u));
    int pos = 0;
    if (key >= 0 && lane == leader) pos = atomicAdd(cursor + key, __popc(peers));
    pos = __shfl_sync(FULL, pos, leader) + rank;
    if (key >= 0) {
      xo[pos] = a;
      zo[pos] = b;
      io[pos] = pid;
    }
  }
}

__global__ void k_sort_finish(SpeciesState *st, const int *__restrict__ total) {
  st->np = *total;
  st->sorted_n = *total;
  st->cur ^= 1;
}

int launch_sort(Ctx *c, int sid) {
  Species &s = c->species[sid];
  const int nk = c->nkeys;
  ISKRA_CUDA(c, cudaMemsetAsync(c->cell_count, 0, (size_t)(nk + 1) * sizeof(int), c->stream));
  int blocks = sort_blocks(c, s);
  k_hist<<<blocks, 256, 0, c->stream>>>(s.dev, c->tiles_x, c->cell_count);
  ISKRA_CUDA(c, cudaGetLastError());
  int nb = (nk + kScanItems - 1) / kScanItems;
  k_scan_reduce<<<nb, 1024, 0, c->stream>>>(c->cell_count, nk, c->scan_tmp);
  k_scan_top<<<1, 1024, 0, c->stream>>>(c->scan_tmp, nb);
  k_scan_down<<<nb, 1024, 0, c->stream>>>(c->cell_count, nk, c->scan_tmp, c->cell_cursor, s.dev.tile_begin);
  ISKRA_CUDA(c, cudaGetLastError());
  // cell_count is free again: keep the grand total there for k_sort_finish
  ISKRA_CUDA(c, cudaMemcpyAsync(c->cell_count + nk, c->cell_cursor + nk, sizeof(int), cudaMemcpyDeviceToDevice,
                                c->stream));
  k_scatter<<<blocks, 256, 0, c->stream>>>(s.dev, c->tiles_x, c->cell_cursor);
  k_sort_finish<<<1, 1, 0, c->stream>>>(s.dev.st, c->cell_count + nk);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// ---------------------------------------------------------------------------
// ensemble push: run r = blockIdx.y; every block of a run stages the run's
// whole E grid (cx*cy <= kWinCells cells), pushes a grid-stride share of the
// run's particles (any order), deposits into shared memory and adds the
// node sums to the run's accumulator.
// ---------------------------------------------------------------------------
//
// SEL: the species is the source of an MCC set, and the push also makes the
// set's work list for the next step -- each pushed particle that stays draws
// its selection count for step + 1 from its own stream (the draw
// k_mcc_select would make at the start of that step: nothing changes the
// particle in between) and, when selected, its new record goes to the run's
// list.  The next step's collision pass then starts without a selection pass
// over all particles.
template <int MX, int MY, bool SEL>
__global__ void __launch_bounds__(256, ISKRA_PUSH_RUNS_MIN_BLOCKS) k_push_runs(const SpeciesDev *__restrict__ runs,
                                                                          const float2 *__restrict__ E2, int nnode,
                                                                          PushParams P, int *err, PushSelect S) {
  pdl_wait();
  __shared__ PushShared sh;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  const int r = blockIdx.y;
  const SpeciesDev s = runs[r];
  const int nx = P.nx, cx = P.nx - 1, cy = P.ny - 1;
  E2 += (size_t)r * nnode;
  for (int t = threadIdx.x; t < cx * cy; t += blockDim.x) {
    const int i = t % cx, j = t / cx;
    const int n0 = i + nx * j;
    cell_record(E2, n0, nx, sh.e[2 * t], sh.e[2 * t + 1]);
    window_clear(sh, t);
  }
  __syncthreads();
  const long long np = s.st->np;
  const int cur = s.st->cur;
  float4 *__restrict__ xv = pick(s.xv[0], s.xv[1], cur);
  float2 *__restrict__ zc = pick(s.zc[0], s.zc[1], cur);
  unsigned ab[4] = {0, 0, 0, 0};
  int flags = 0;
  const uint32_t *__restrict__ ids = pick(s.id[0], s.id[1], cur);
  const unsigned long long step1 = SEL ? *S.d_step + 1ull : 0ull;
  const uint2 key = SEL ? S.keys[r] : make_uint2(0u, 0u);
  const float expl = __expf(-S.lam);  // as k_mcc_select and k_mcc_collide form it
  MccWork *__restrict__ seg = SEL ? S.work + (size_t)r * S.cap_run : nullptr;
  const long long warp = (long long)blockIdx.x * nwb + wib, nwarps = (long long)gridDim.x * nwb;
  for (long long base = warp * 32; base < np; base += nwarps * 32) {
    const long long p = base + lane;
    const bool v = p < np;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 b = make_float2(0.f, 0.f);
    if (v) {
      a = ld_stream(xv + p);
      b = ld_stream(zc + p);
    }
    float4 na;
    float2 nb;
    push_warp<true, MX, MY, true>(s, xv, zc, p, v, a, b, E2, sh, 0, 0, cx, cy, P, ab, flags, SEL ? &na : nullptr,
                                  SEL ? &nb : nullptr);
    if (SEL) {
      int nsel = 0;
      uint32_t pid = 0;
      if (v && __float_as_int(nb.y) >= 0) {
        pid = ids[p];
        Stream R = particle_stream(pid, step1, key);
        nsel = draw_selections(R, S.lam, expl);
      }
      const unsigned m = __ballot_sync(FULL, nsel > 0);
      if (m) {
        const int leader = __ffs(m) - 1;
        unsigned long long at = 0;
        if (lane == leader) at = atomicAdd(S.nwork + r, (unsigned long long)__popc(m));
        at = __shfl_sync(FULL, at, leader) + __popc(m & ((1u << lane) - 1u));
        if (nsel > 0) {
          if (at < S.cap_run) seg[at] = mcc_entry(na, nb, pid, (uint32_t)p);
          else flags |= DERR_CAPACITY;
        }
      }
    }
  }
  __syncthreads();
  const int wn = cx + 1;
  for (int t = threadIdx.x; t < (cx + 1) * (cy + 1); t += blockDim.x) {
    const int a = t % wn, b = t / wn;
    unsigned long long v = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int ca = a - (c & 1), cb = b - (c >> 1);
      if (ca < 0 || cb < 0 || ca >= cx || cb >= cy) continue;
      const int w = ca + cx * cb;
      if (!sh.mom[kMomN][w]) continue;
      unsigned long long W[4];
      window_cell(sh, w, W);
      v += W[c];
    }
    if (v) atomicAdd(s.acc + a + nx * b, v);
  }
  for (int t = threadIdx.x; t < cx * cy; t += blockDim.x) {
    const unsigned v = sh.mom[kMomN][t];
    if (v) atomicAdd(s.cnt + (t % cx) + nx * (t / cx), v);
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    unsigned t = __reduce_add_sync(FULL, ab[k]);
    if (lane == 0 && t) atomicAdd(&s.st->absorbed[k], (unsigned long long)t);
  }
  int f = __reduce_or_sync(FULL, flags);
  if (lane == 0 && f) atomicOr(err, f);
}

// Ensemble push of one species (runs: device array of R run views).
int launch_push_runs(Ctx *c, int sid, const SpeciesDev *runs, int R, const float2 *E2, float dt, int blocks_per_run,
                     int *err, cudaStream_t st, const PushSelect *sel) {
  Species &s = c->species[sid];
  if ((c->nx - 1) * (c->ny - 1) > kWinCells) return set_err(c, ISKRA_EINVAL, "ensemble grid larger than one window");
  PushParams P{};  // no surface tracker in ensembles
  P.h = (float)(0.5 * (double)dt * (s.q / s.m));
  P.dtdx = (float)((double)dt / c->g.dx);
  P.dtdy = (float)((double)dt / c->g.dy);
  P.nx = c->nx;
  P.ny = c->ny;
  P.mode_x = s.bnd[0];
  P.mode_y = s.bnd[1];
  P.tiles_x = 0;
  const int nnode = c->nn;
  const dim3 grid(blocks_per_run, R);
  const PushSelect S = sel ? *sel : PushSelect{};
#define ISKRA_PUSH_RUNS_CASE(MX, MY)                                                                           \
  if (P.mode_x == MX && P.mode_y == MY) {                                                                       \
    auto kern = sel ? k_push_runs<MX, MY, true> : k_push_runs<MX, MY, false>;                                   \
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                                  \
                         (int)cudaSharedmemCarveoutMaxShared);                                                  \
    ISKRA_CUDA(c, launch_pdl(kern, grid, 256, 0, st, runs, E2, nnode, P, err, S));                             \
    return ISKRA_OK;                                                                                            \
  }
  ISKRA_PUSH_RUNS_CASE(0, 0) ISKRA_PUSH_RUNS_CASE(0, 1) ISKRA_PUSH_RUNS_CASE(0, 2)
  ISKRA_PUSH_RUNS_CASE(1, 0) ISKRA_PUSH_RUNS_CASE(1, 1) ISKRA_PUSH_RUNS_CASE(1, 2)
  ISKRA_PUSH_RUNS_CASE(2, 0) ISKRA_PUSH_RUNS_CASE(2, 1) ISKRA_PUSH_RUNS_CASE(2, 2)
#undef ISKRA_PUSH_RUNS_CASE
  return set_err(c, ISKRA_EINVAL, "bad boundary mode");
}

// Σ (vx² + vy²) and the number of live particles (for the sort cadence)
__global__ void k_speed2(SpeciesDev s, double *__restrict__ out) {
  __shared__ float sh[2][8];
  const long long np = s.st->np;
  const int cur = s.st->cur;
  const float4 *__restrict__ xv = pick(s.xv[0], s.xv[1], cur);
  const float2 *__restrict__ zc = pick(s.zc[0], s.zc[1], cur);
  float v2 = 0.f, n = 0.f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    if (__float_as_int(zc[p].y) < 0) continue;
    const float4 a = xv[p];
    v2 = fmaf(a.z, a.z, fmaf(a.w, a.w, v2));
    n += 1.f;
  }
  for (int o = 16; o > 0; o >>= 1) {
    v2 += __shfl_down_sync(0xffffffffu, v2, o);
    n += __shfl_down_sync(0xffffffffu, n, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = v2;
    sh[1][threadIdx.x >> 5] = n;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      a += sh[0][w];
      b += sh[1][w];
    }
    atomicAdd(out, a);
    atomicAdd(out + 1, b);
  }
}

int species_speed2(Ctx *c, int sid, double *mean_v2) {
  Species &s = c->species[sid];
  ISKRA_CUDA(c, cudaMemsetAsync(c->d_scratch, 0, 2 * sizeof(double), c->stream));
  k_speed2<<<c->num_sms * 4, 256, 0, c->stream>>>(s.dev, c->d_scratch);
  ISKRA_CUDA(c, cudaGetLastError());
  double h[2];
  ISKRA_CUDA(c, cudaMemcpyAsync(h, c->d_scratch, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  *mean_v2 = h[1] > 0 ? h[0] / h[1] : 0.0;
  return ISKRA_OK;
}

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_advance(iskra_ctx *h, int sid, double dt) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (sid < 0 || sid >= (int)c->species.size()) return set_err(c, ISKRA_EINVAL, "bad species id");
  if (!(dt > 0)) return set_err(c, ISKRA_EINVAL, "dt must be positive");
  return launch_advance(c, sid, (float)dt);
}

int iskra_advance_all(iskra_ctx *h, double dt) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!(dt > 0)) return set_err(c, ISKRA_EINVAL, "dt must be positive");
  return launch_advance_all(c, (float)dt, nullptr, nullptr);
}

int iskra_density(iskra_ctx *h, int sid, double *n_out) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (sid < 0 || sid >= (int)c->species.size()) return set_err(c, ISKRA_EINVAL, "bad species id");
  Species &s = c->species[sid];
  if (!s.n_valid || s.acc_valid) {
    int rc = finalize(c, false);
    if (rc) return rc;
  }
  if (n_out) {
    int rc = sync_n64(c, s);
    if (rc) return rc;
    ISKRA_CUDA(c, cudaMemcpyAsync(n_out, s.n, (size_t)c->nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
    return collect_device_errors(c);
  }
  return ISKRA_OK;
}

int iskra_charge_density(iskra_ctx *h) {
  if (!h) return ISKRA_EINVAL;
  return launch_charge_density(&h->c);
}

}  // extern "C"
