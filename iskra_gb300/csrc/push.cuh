// push.cuh -- the fused particle push (gather, Boris push, wrap!/discard!,
// deposit) as templates, shared by particles.cu (16 x 16-cell tiles, the
// ensemble push) and the translation units of the other tile sizes.
#pragma once
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
#define ISKRA_PUSH_RUNS_MIN_BLOCKS 4
#endif
// ensemble push blocks per run = the ensemble's blocks per run × this / 8
#ifndef ISKRA_PUSH_RUNS_SCALE8
#define ISKRA_PUSH_RUNS_SCALE8 8
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

// Shared-memory window of an ensemble-run block: the run's whole grid (at
// most kEnsWinCells cells).
constexpr int kEnsWin = 20;
constexpr int kEnsWinCells = kEnsWin * kEnsWin;

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
// Dynamic shared memory of an ensemble push block (53 KB: 4 blocks per SM):
// per warp a ring of kEnsStages record stages filled by cp.async (two warp
// iterations in flight while the third is pushed), the selection buffer,
// E at the window's nodes, the deposit moments.
constexpr int kEnsStages = 3;
constexpr int kEnsWinNodes = 2 * kEnsWinCells + 2;  // most nodes of a window of at most kEnsWinCells cells
struct PushShared {
  static constexpr int kWinCells = kEnsWinCells;
  float4 ra[8][kEnsStages][32];     // staged records {hx, hy, vx, vy}
  float2 rb[8][kEnsStages][32];     // staged records {vz, cell}
  MccWork wbuf[8][64];              // selected work-list entries, per warp
  float2 ne[kEnsWinNodes];          // E at the window's nodes (row stride: cells per row + 1)
  unsigned mom[kMoms][kWinCells];   // deposit moments of the window cells
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
#if ISKRA_PUSH_BULK == 1
constexpr int kRbStage = 34;  // {vz, cell} records of a stage from the 16-byte boundary at or below its first slot
#else
constexpr int kRbStage = 32;
#endif
// ISKRA_PUSH_BULK=2: one ring per block instead of one per warp -- a
// producer warp (added to the ISKRA_PUSH_THREADS consumers) fills stages of
// ISKRA_PUSH_THREADS records (one per consumer thread) with two bulk copies
// each and a full/empty mbarrier pair per stage, so the records never pass
// through the LSU on their way into shared memory and the mbarrier round
// trip is paid once per 192 records.  Measured on GB300 (512x512 slab):
// 0.0975-0.098 ms per two-species push against 0.0888 ms for the per-lane
// cp.async rings (4 or 6 stages; 8 stages 0.106 ms) -- the hand-off between
// the producer and the slowest consumer warp costs more than it saves.
constexpr int kPushBlock = ISKRA_PUSH_THREADS + (ISKRA_PUSH_BULK == 2 ? 32 : 0);
// The window of a tile of 2^TS x 2^TS cells: the tile and a kHalo-cell
// margin (particles drift off their tile between sorts).  Dynamic shared
// memory (the 32 x 32-cell tile's window needs 72 KB).
template <int TS>
struct TileShared {
  static constexpr int kTileC = 1 << TS;
  static constexpr int kWin = kTileC + 2 * kHalo;  // window cells per axis
  static constexpr int kWinN = kWin + 1;           // window nodes per axis
  static constexpr int kWinCells = kWin * kWin;
#if ISKRA_PUSH_BULK == 2
  float4 ra[kStages][ISKRA_PUSH_THREADS];      // staged records {hx, hy, vx, vy}
  float2 rb[kStages][ISKRA_PUSH_THREADS + 2];  // {vz, cell} from the 16-byte boundary at or below the first
  unsigned long long full[kStages], empty[kStages];
#else
  float4 ra[ISKRA_PUSH_THREADS / 32][kStages][32];        // staged records {hx, hy, vx, vy}
  float2 rb[ISKRA_PUSH_THREADS / 32][kStages][kRbStage];  // staged records {vz, cell}
  unsigned long long bar[ISKRA_PUSH_THREADS / 32][kStages];  // stage mbarriers (bulk-copy ring)
#endif
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
#if ISKRA_PUSH_BULK
constexpr unsigned kMbarSpins = 1u << 20;  // polls of one stage before DERR_TIMEOUT
#endif

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
  const int n = la + (ww + 1) * lb;
  const float2 a = sh.ne[n], b = sh.ne[n + 1], c = sh.ne[n + ww + 1], d = sh.ne[n + ww + 2];
  r0 = make_float4(a.x, a.y, b.x, b.y);
  r1 = make_float4(c.x, c.y, d.x, d.y);
}
// track! flag of window cell w (ensemble blocks run without a tracker)
__device__ __forceinline__ bool win_tracked(const PushShared &, int) { return false; }
template <int TS>
__device__ __forceinline__ bool win_tracked(const TileShared<TS> &sh, int w) { return sh.trk[w] != 0; }
template <int TS>
__device__ __forceinline__ void win_record(const TileShared<TS> &sh, int la, int lb, int, float4 &r0, float4 &r1) {
  constexpr int kWinN = TileShared<TS>::kWinN;
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
// SH::kWinCells + the global cell index, so runs never mix the two.
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
                                                                                  : SH::kWinCells + i0 + nx * j0;
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
    if (WIN && key < SH::kWinCells) {
      window_add(sh, key, n, m);
    } else {
      const unsigned long long U = (unsigned long long)m.su << 24, V = (unsigned long long)m.sv << 24;
      const unsigned long long UV = ((unsigned long long)m.hi << 24) + m.lo;
      const int g = key - SH::kWinCells;
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
template <bool PUSH, int MX, int MY, bool TRK, int TS>
__device__ __forceinline__ void push_block(const SpeciesDev &s, const PushParams &P, const float2 *__restrict__ E2,
                                           TileShared<TS> &sh, int tile, int tail_block, int tail_blocks, int *err) {
  constexpr int kWin = TileShared<TS>::kWin, kWinN = TileShared<TS>::kWinN, kWinCells = TileShared<TS>::kWinCells;
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
      const int ox = ((tile % P.tiles_x) << TS) - kHalo, oy = ((tile / P.tiles_x) << TS) - kHalo;
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
#if ISKRA_PUSH_BULK == 2
      constexpr int C = ISKRA_PUSH_THREADS;  // records per stage, one per consumer thread
      if (threadIdx.x == 0) {
#pragma unroll
        for (int d = 0; d < kStages; d++) {
          mbar_init(&sh.full[d], 1u);
          mbar_init(&sh.empty[d], (unsigned)(C / 32));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      }
      __syncthreads();
      {
        const long long len = end - begin;
        const int nchunks = (int)((len + C - 1) / C);
        const int sft = (int)(begin & 1);  // chunks start at begin + q C: the same parity (C is even)
        if (threadIdx.x >= C) {
          // producer: chunk q into stage q % kStages once the consumers have
          // released that stage's previous chunk
          if (lane == 0) {
            for (int q = 0; q < nchunks; q++) {
              const int st = q % kStages;
              if (q >= kStages) {
                if (!mbar_wait(&sh.empty[st], (unsigned)((q / kStages) - 1) & 1u, kMbarSpins)) {
                  flags |= DERR_TIMEOUT;  // the consumers time out on the chunks not issued
                  break;
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // their reads precede the copy's writes
              }
              const long long r0 = begin + (long long)q * C;
              const int n = (int)min((long long)C, end - r0);
              const unsigned ba = 16u * n, bb = 8u * ((n + sft + 1) & ~1);  // both multiples of 16 bytes
              const unsigned bar = smem_u32(&sh.full[st]);
              asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(ba + bb)
                           : "memory");
              asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                               "r"(smem_u32(&sh.ra[st][0])), "l"(xv + r0), "r"(ba), "r"(bar)
                           : "memory");
              asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                               "r"(smem_u32(&sh.rb[st][0])), "l"(zc + r0 - sft), "r"(bb), "r"(bar)
                           : "memory");
            }
          }
        } else {
          float4 *__restrict__ xw = xv + begin;
          float2 *__restrict__ zw = zc + begin;
          for (int q = 0; q < nchunks; q++) {
            const int st = q % kStages;
            // bounded: a stage that never completes is flagged and its records skipped
            const bool ok = __all_sync(FULL, mbar_wait(&sh.full[st], (unsigned)(q / kStages) & 1u, kMbarSpins));
            if (!ok) flags |= DERR_TIMEOUT;
            const int o = q * C + threadIdx.x;
            const bool v = ok && o < len;
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
            float2 b = make_float2(0.f, 0.f);
            if (v) {
              a = sh.ra[st][threadIdx.x];
              b = sh.rb[st][threadIdx.x + sft];
            }
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&sh.empty[st])) : "memory");
            push_warp<PUSH, MX, MY, true, TRK>(s, xw, zw, o, v, a, b, E2, sh, ox, oy, kWin, kWin, P, ab, flags);
          }
        }
      }
      __syncthreads();
#else
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
#if ISKRA_PUSH_BULK == 1
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
#endif  // ISKRA_PUSH_BULK == 2
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
template <bool PUSH, int MX, int MY, bool TRK, int TS>
__global__ void __launch_bounds__(kPushBlock, TRK ? ISKRA_PUSH_TRK_MIN_BLOCKS : ISKRA_PUSH_MIN_BLOCKS)
    k_push(SpeciesDev s, const float2 *__restrict__ E2, PushParams P, int ntiles, int *err) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char push_smem[];
  TileShared<TS> &sh = *reinterpret_cast<TileShared<TS> *>(push_smem);
  const int b = blockIdx.x;
  if (b < ntiles) push_block<PUSH, MX, MY, TRK, TS>(s, P, E2, sh, b, 0, 0, err);
  else push_block<PUSH, MX, MY, TRK, TS>(s, P, E2, sh, -1, b - ntiles, gridDim.x - ntiles, err);
}

// Two species in one launch (the step's electrons and ions): their pushes
// are independent until ρ is formed, so the second species' tiles fill the
// SMs as the first species' tiles drain instead of waiting for a second
// launch.  Blocks [0, ntiles) first species' tiles, [ntiles, 2 ntiles) the
// second's, the rest both tails.
// step_ctr (optional): the step counter, advanced here when no MCC set reads
// it earlier in the step (saves the step's opening launch).
template <int MX, int MY, bool TRK, int TS>
__global__ void __launch_bounds__(kPushBlock, TRK ? ISKRA_PUSH_TRK_MIN_BLOCKS : ISKRA_PUSH_MIN_BLOCKS)
    k_push2(SpeciesDev s0, SpeciesDev s1, const float2 *__restrict__ E2, PushParams P0, PushParams P1, int ntiles,
            int *err, unsigned long long *step_ctr) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char push_smem[];
  TileShared<TS> &sh = *reinterpret_cast<TileShared<TS> *>(push_smem);
  const int b = blockIdx.x;
  if (step_ctr && b == 0 && threadIdx.x == 0) *step_ctr += 1ull;
  if (b < ntiles) {
    push_block<true, MX, MY, TRK, TS>(s0, P0, E2, sh, b, 0, 0, err);
  } else if (b < 2 * ntiles) {
    push_block<true, MX, MY, TRK, TS>(s1, P1, E2, sh, b - ntiles, 0, 0, err);
  } else {
    const int tb = b - 2 * ntiles, nt = gridDim.x - 2 * ntiles;
    push_block<true, MX, MY, TRK, TS>(s0, P0, E2, sh, -1, tb, nt, err);
    push_block<true, MX, MY, TRK, TS>(s1, P1, E2, sh, -1, tb, nt, err);
  }
}

// The push kernels of one tile size (k_push with PUSH = true for every pair of
// boundary rules, with and without a surface tracker; the deposit-only
// k_push; the species-pair k_push2).  Each tile size is instantiated in its
// own translation unit (push_t8.cu, particles.cu, push_t32.cu) so the three
// compile in parallel.
template <int TS>
struct PushTile {
  static constexpr size_t kSmem = sizeof(TileShared<TS>);
  template <class K>
  static void prepare(K kern) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  }
  // one species: push (push = true) or deposit only
  static cudaError_t one(cudaStream_t st, bool push, bool trk, const SpeciesDev &s, const float2 *E2,
                         const PushParams &P, int ntiles, int blocks, int *err) {
    if (!push) {
      auto kern = k_push<false, 0, 0, false, TS>;
      prepare(kern);
      return launch_pdl(kern, blocks, kPushBlock, kSmem, st, s, E2, P, ntiles, err);
    }
#define ISKRA_PUSH_CASE(MX, MY)                                                                \
  if (P.mode_x == MX && P.mode_y == MY) {                                                      \
    auto kern = trk ? k_push<true, MX, MY, true, TS> : k_push<true, MX, MY, false, TS>;        \
    prepare(kern);                                                                             \
    return launch_pdl(kern, blocks, kPushBlock, kSmem, st, s, E2, P, ntiles, err);             \
  }
    ISKRA_PUSH_CASE(0, 0) ISKRA_PUSH_CASE(0, 1) ISKRA_PUSH_CASE(0, 2)
    ISKRA_PUSH_CASE(1, 0) ISKRA_PUSH_CASE(1, 1) ISKRA_PUSH_CASE(1, 2)
    ISKRA_PUSH_CASE(2, 0) ISKRA_PUSH_CASE(2, 1) ISKRA_PUSH_CASE(2, 2)
#undef ISKRA_PUSH_CASE
    return cudaErrorInvalidValue;
  }
  // two species with the same boundary rules in one launch
  static cudaError_t two(cudaStream_t st, bool trk, const SpeciesDev &a, const SpeciesDev &b, const float2 *E2,
                         const PushParams &Pa, const PushParams &Pb, int ntiles, int blocks, int *err,
                         unsigned long long *step_ctr) {
#define ISKRA_PUSH2_CASE(MX, MY)                                                                          \
  if (Pa.mode_x == MX && Pa.mode_y == MY) {                                                               \
    auto kern = trk ? k_push2<MX, MY, true, TS> : k_push2<MX, MY, false, TS>;                             \
    prepare(kern);                                                                                        \
    return launch_pdl(kern, blocks, kPushBlock, kSmem, st, a, b, E2, Pa, Pb, ntiles, err, step_ctr);         \
  }
    ISKRA_PUSH2_CASE(0, 0) ISKRA_PUSH2_CASE(0, 1) ISKRA_PUSH2_CASE(0, 2)
    ISKRA_PUSH2_CASE(1, 0) ISKRA_PUSH2_CASE(1, 1) ISKRA_PUSH2_CASE(1, 2)
    ISKRA_PUSH2_CASE(2, 0) ISKRA_PUSH2_CASE(2, 1) ISKRA_PUSH2_CASE(2, 2)
#undef ISKRA_PUSH2_CASE
    return cudaErrorInvalidValue;
  }
};

// entry points of the per-tile-size translation units
cudaError_t push_tile_one(int ts, cudaStream_t st, bool push, bool trk, const SpeciesDev &s, const float2 *E2,
                          const PushParams &P, int ntiles, int blocks, int *err);
cudaError_t push_tile_two(int ts, cudaStream_t st, bool trk, const SpeciesDev &a, const SpeciesDev &b,
                          const float2 *E2, const PushParams &Pa, const PushParams &Pb, int ntiles, int blocks,
                          int *err, unsigned long long *step_ctr);
#define ISKRA_PUSH_TILE_TU(TS, NAME)                                                                          \
  cudaError_t push_tile_one_##NAME(cudaStream_t st, bool push, bool trk, const SpeciesDev &s, const float2 *E2, \
                                   const PushParams &P, int ntiles, int blocks, int *err) {                    \
    return PushTile<TS>::one(st, push, trk, s, E2, P, ntiles, blocks, err);                                    \
  }                                                                                                            \
  cudaError_t push_tile_two_##NAME(cudaStream_t st, bool trk, const SpeciesDev &a, const SpeciesDev &b,         \
                                   const float2 *E2, const PushParams &Pa, const PushParams &Pb, int ntiles,   \
                                   int blocks, int *err, unsigned long long *step_ctr) {                       \
    return PushTile<TS>::two(st, trk, a, b, E2, Pa, Pb, ntiles, blocks, err, step_ctr);                        \
  }

}  // namespace iskra
