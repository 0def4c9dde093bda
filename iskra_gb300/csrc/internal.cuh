// internal.cuh -- device data structures shared by the libiskra_gpu.so sources.
//
// Particle store (per species, structure of arrays, double-buffered for the
// counting sort):
//   xv[b][p] : float4 {hx, hy, vx, vy}   in-cell offsets and velocity x/y
//   zc[b][p] : float2 {vz, cell}         cell = (i0 | j0 << 16) as int bits,
//                                        -1 marks a discarded particle
//   id[b][p] : uint32 particle identifier (KineticSpecies.id)
// i0, j0 are the 0-based lower-left node of the particle's cell; the
// reference's particle_cell gives i = i0 + 1, hx = x/Δx - i0
// (ParticleInCell.jl:28-35).  Offsets are kept on the 2^-24 grid so that the
// CIC weights are exact 48-bit integer products (deposit is then exact,
// deterministic and order-independent without FP64 arithmetic).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/iskra_gpu.h"

namespace iskra {

constexpr float kOffScale = 16777216.0f;  // 2^24
constexpr float kOffInv = 5.9604644775390625e-08f;  // 2^-24
constexpr int kMaxSpecies = 8;
// A node sums the deposit weights of the particles in its four cells; with at
// most kMaxCell particles per cell the sum stays below 4 * 16383 * 2^48 < 2^64.
constexpr unsigned kMaxCell = 16383;
constexpr int kMaxMcc = 8;
// slots allocated past a species' capacity in its record arrays (whole-stage
// bulk copies of the push may read up to 33 records past a slice's end)
constexpr int kStorePad = 64;

// device error flags (bitmask in Ctx::d_err)
enum : int {
  DERR_CAPACITY = 1,
  DERR_DOMAIN = 2,
  DERR_PROB = 4,
  DERR_NAN = 8,
  DERR_TIMEOUT = 16,
  DERR_NOTCONV = 32,
  DERR_OVERFLOW = 64,
};

// device-resident, written by kernels; one 128-byte line each, so that the
// states of an ensemble's runs (an array) do not share lines between the
// runs' atomics
struct alignas(128) SpeciesState {
  long long np;                // slots in use (live + discarded holes)
  int cur;                     // active buffer of the double-buffered store
  int pad;
  unsigned long long absorbed[4];  // discard! counts per wall
  unsigned int next_id;        // identifier for appended particles
  unsigned int pad2;
  long long np_new;            // append cursor used while a kernel appends
  long long sorted_n;          // slots [0, sorted_n) are grouped by tile (last sort); the rest is unsorted
};

struct SpeciesDev {            // kernel view of one species (by value)
  float4 *xv[2];
  float2 *zc[2];
  uint32_t *id[2];
  SpeciesState *st;
  unsigned long long *acc;     // (nx*ny) fixed-point deposit accumulator
  long long cap;
  unsigned *cnt;               // (nx*ny) particles deposited per cell (overflow guard)
  int *tile_begin;             // (ntiles + 1) first slot of each tile after the last sort
};

// Tiles: the push runs one block per tile of 2^ts x 2^ts cells (ts =
// Ctx::tile_shift: 8, 16 or 32 cells per axis, chosen by the autotuner;
// 16 by default) over the particles the last sort grouped there, with E at
// the nodes and the deposit moments of the tile and a kHalo-cell margin in
// shared memory.  The sort key of a cell is tile-major: tile * 4^ts + the
// cell's position in the tile.
constexpr int kTileShiftMin = 3, kTileShiftMax = 5, kTileShiftDefault = 4;
constexpr int kHalo = 2;

__device__ __host__ __forceinline__ int cell_key(int i0, int j0, int tiles_x, int ts) {
  const int t = (i0 >> ts) + tiles_x * (j0 >> ts);
  const int m = (1 << ts) - 1;
  return (t << (2 * ts)) + (i0 & m) + ((j0 & m) << ts);
}

// tile counts of a grid of nx x ny nodes for tile shift ts
inline void tile_geometry(int nx, int ny, int ts, int &tiles_x, int &tiles_y) {
  const int t = 1 << ts;
  tiles_x = ((nx > 1 ? nx - 1 : 1) + t - 1) / t;
  tiles_y = ((ny > 1 ? ny - 1 : 1) + t - 1) / t;
}

// Buffer of a double-buffered array without dynamic indexing of a kernel
// parameter (which would place the parameter struct in local memory).
template <class T>
__device__ __forceinline__ T *pick(T *a, T *b, int cur) {
  return cur ? b : a;
}

// The gather's record of cell (ci, cj) (index k = ci + nx cj) from the node
// field E2 (FP32 {Ex, Ey} per node): float4 {E(ci,cj), E(ci+1,cj)} and float4
// {E(ci,cj+1), E(ci+1,cj+1)}.  The push stages the records of its window in
// shared memory from the node values, so the field passes write E once per
// node (coalesced) instead of into the four cell records around each node.
__device__ __forceinline__ void cell_record(const float2 *__restrict__ E2, int k, int nx, float4 &r0, float4 &r1) {
  const float2 a = __ldg(E2 + k), b = __ldg(E2 + k + 1), c = __ldg(E2 + k + nx), d = __ldg(E2 + k + nx + 1);
  r0 = make_float4(a.x, a.y, b.x, b.y);
  r1 = make_float4(c.x, c.y, d.x, d.y);
}

// ---- Philox4x32-10 (Salmon et al., SC'11), counter-based: the MCC and the
// particle sources key it by (seed, stream, step, particle) ------------------
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// MCC work-list entry (mcc.cu): a selected particle's record as the
// collision pass needs it -- a = {hx, hy, vx, vy}, b = {vz bits, cell, id,
// slot} -- one 32-byte sector.
struct __align__(16) MccWork {
  float4 a;
  uint4 b;
};
__device__ __forceinline__ MccWork mcc_entry(float4 a, float2 b, uint32_t pid, uint32_t slot) {
  MccWork e;
  e.a = a;
  e.b = make_uint4(__float_as_uint(b.x), __float_as_uint(b.y), pid, slot);
  return e;
}

// uniform in [0,1) with 24 random bits
__device__ __forceinline__ float u01(uint32_t v) { return (float)(v >> 8) * 5.9604644775390625e-08f; }

struct Stream {
  U4 ctr;
  uint32_t k0, k1;
  U4 buf;
  int left;
  __device__ float next() {
    if (left == 0) {
      buf = philox4x32_10(ctr, k0, k1);
      ctr.w += 1;
      left = 4;
    }
    uint32_t v = left == 4 ? buf.x : left == 3 ? buf.y : left == 2 ? buf.z : buf.w;
    left--;
    return u01(v);
  }
  __device__ float normal() {  // Box-Muller (one of the pair)
    float a = next();
    float b = next();
    a = fmaxf(a, 1.0e-12f);
    float rad = sqrtf(-2.0f * logf(a));
    return rad * cospif(2.0f * b);
  }
  __device__ void normal2(float &n0, float &n1) {  // Box-Muller, both of the pair
    float a = next();
    const float b = next();
    a = fmaxf(a, 1.0e-12f);
    const float rad = sqrtf(-2.0f * logf(a));
    float s, c;
    sincospif(2.0f * b, &s, &c);
    n0 = rad * c;
    n1 = rad * s;
  }
  // three independent normal draws (a Box-Muller pair and one of a second)
  __device__ void normal3(float v[3], float scale) {
    normal2(v[0], v[1]);
    v[2] = normal();
    v[0] *= scale;
    v[1] *= scale;
    v[2] *= scale;
  }
};

// The MCC random stream of one particle in one step (mcc.cu): Philox keyed by
// the set's key, counter (particle id, step, draw).
__device__ __forceinline__ Stream particle_stream(uint32_t pid, unsigned long long step, uint2 key) {
  Stream R;
  R.ctr = U4{pid, (uint32_t)step, (uint32_t)(step >> 32), 0u};
  R.k0 = key.x;
  R.k1 = key.y;
  R.left = 0;
  return R;
}

// The uniform that decides a particle's number of selections in a step: a
// 64-bit mix of (key, step, particle id) -- the finalizer of SplitMix64
// (Steele, Lea and Flood, OOPSLA 2014) over the key and the id and step
// spread by odd multipliers -- 24 bits.  Every particle draws it every step
// (most draw no selection), so it is a tenth of a Philox evaluation; the
// collision draws of the selected particles come from their Philox stream.
__device__ __forceinline__ float selection_uniform(uint32_t pid, unsigned long long step, uint2 key) {
  unsigned long long z = (((unsigned long long)key.y << 32) | key.x) ^ (step * 0x9E3779B97F4A7C15ull) ^
                         ((unsigned long long)pid * 0xD1B54A32D192ED03ull);
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * 5.9604644775390625e-08f;
}

// selections ~ Poisson(lam) by inversion (bounded) of the selection uniform u
__device__ __forceinline__ int draw_selections(float u, float lam, float expl) {
  float pk = expl, cdf = expl;
  int nsel = 0;
  while (u > cdf && nsel < 16) {
    nsel++;
    pk *= lam / nsel;
    cdf += pk;
  }
  return nsel;
}

// The runs' work-list counters lie a 128-byte line apart: every warp of a
// run reserves list positions on its run's counter, and counters that share
// a line serialise in one L2 slice.
constexpr int kNworkStride = 16;

// Selection for the next MCC step folded into an ensemble push (k_push_runs):
// per run, the set's key, its work list segment and counter.
struct PushSelect {
  float lam;                    // N maxPt of the MCC set
  const uint2 *keys;            // R
  MccWork *work;                // R x cap_run
  unsigned long long *nwork;    // R counters, kNworkStride apart
  unsigned long long cap_run;
  const unsigned long long *d_step;  // the current step (entries are for step + 1)
};


// CrossSection: linear interpolation, flat extrapolation (cross_section.jl:8-14)
// The bracket e[lo] <= x < e[lo+1] is found by bisection, or for tables on a
// log-uniform grid from log(x) and then corrected against the table itself
// (the same bracket either way).
__device__ __forceinline__ float sigma_at(const float *e, const float *s, int n, float x, int logu, float le0,
                                          float idl) {
  if (x <= e[0]) return s[0];
  if (x >= e[n - 1]) return s[n - 1];
  int lo;
  if (logu) {
    lo = (int)((__logf(x) - le0) * idl);
    lo = max(0, min(n - 2, lo));
    while (lo > 0 && e[lo] > x) lo--;
    while (lo < n - 2 && e[lo + 1] <= x) lo++;
  } else {
    lo = 0;
    int hi = n - 1;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (e[mid] <= x) lo = mid;
      else hi = mid;
    }
  }
  const int hi = lo + 1;
  const float t = (x - e[lo]) / (e[hi] - e[lo]);
  return (1.0f - t) * s[lo] + t * s[hi];
}

// particle_cell (ParticleInCell.jl:28-35) on the device side of an upload or a
// source: i0 = floor(x/Δh) (the reference's i - 1, formed without the 1 + ...
// that can round x just below the far wall onto node nx), the offset rounded
// to the nearest point of the 2^-24 grid; a carry into the next cell is taken
// unless that cell does not exist (then the offset stays at 1 - 2^-24), so a
// download/upload round trip reproduces the state.  Returns the packed cell
// (i0 | j0 << 16) or -1 outside the grid.
__device__ __forceinline__ int cell_of_units(double fx, double fy, int nx, int ny, long long &ux, long long &uy) {
  const double ix = floor(fx), jy = floor(fy);
  long long i0 = (long long)ix, j0 = (long long)jy;
  ux = llrint((fx - ix) * 16777216.0);
  uy = llrint((fy - jy) * 16777216.0);
  if (ux >= 16777216LL) {
    if (i0 + 1 <= nx - 2) {
      i0 += 1;
      ux = 0;
    } else {
      ux = 16777215LL;
    }
  }
  if (uy >= 16777216LL) {
    if (j0 + 1 <= ny - 2) {
      j0 += 1;
      uy = 0;
    } else {
      uy = 16777215LL;
    }
  }
  if (i0 < 0 || j0 < 0 || i0 > nx - 2 || j0 > ny - 2) return -1;
  return (int)(i0 | (j0 << 16));
}
// the same from a position in metres (f = x / Δh)
__device__ __forceinline__ int cell_of_position(double X, double Y, double dx, double dy, int nx, int ny,
                                                 long long &ux, long long &uy) {
  return cell_of_units(X / dx, Y / dy, nx, ny, ux, uy);
}

struct Species {
  double q = 0, m = 0, w0 = 0;
  long long cap = 0;
  int bnd[2] = {ISKRA_BND_NONE, ISKRA_BND_NONE};
  SpeciesDev dev{};
  SpeciesDev *dview = nullptr; // device copy of dev (kernels over run views take arrays)
  double *n = nullptr;         // FP64 density (nx*ny)
  float2 *n_df = nullptr;      // double-float density (written when ρ is formed in double-float)
  bool n64_valid = true;       // n holds the density
  bool n_df_valid = false;     // n_df holds the density
  // accumulator / density bookkeeping (host side):
  bool acc_valid = false;      // acc holds the unconsumed deposit of the current positions
  bool acc_zero = true;        // acc is all zero
  bool n_valid = true;         // n matches the current positions
};

struct Poisson;                // poisson.cu
struct Mcc;                    // mcc.cu
struct Lws;                    // lws.cu (learned warm start of CG solves)
struct Mg;                     // multigrid.cu (V-cycle preconditioner of CG solves)
int mg_build(struct Ctx *c, int nx, int ny, const std::vector<double> &s0, const std::vector<double> &sW,
             const std::vector<double> &sE, const std::vector<double> &sS, const std::vector<double> &sN,
             const std::vector<char> &free_row, int per_x, int per_y, Mg **out);
int mg_queue_cycle(struct Ctx *c, Mg *m, const double *r, double *z, const int *skip);
int mg_levels(const Mg *m);
void mg_destroy(Mg *m);
struct CircuitDev {            // device-resident circuit state (FP64)
  double R, L, C, amp, freq, dc, area, scale;
  double t, i, q, vext;
  int sigma_dof;               // 0-based index into Poisson sigma
  int pad;
};

// Surface tracker (pic/surfaces/*.jl): per cell (numbered like nodes,
// i0 + nx j0) the surface behind each of its four edges, in the order of
// kSurfDir, and whether track! records particles of the cell.
constexpr int kMaxSurfaces = 64;
enum { kSurfDirXm, kSurfDirXp, kSurfDirYm, kSurfDirYp };
struct Tracker {
  std::vector<unsigned char> edge;       // 4 per cell: surface index + 1, 0 = no surface
  std::vector<unsigned char> cell;       // 1: the cell is one side of some surface edge
  std::vector<int> kind;                 // ISKRA_SURF_* per surface
  std::vector<int> sigma_dof;            // 0-based σ dof (FLOATING), else -1
  std::vector<double> area;
  unsigned char *d_edge = nullptr, *d_cell = nullptr, *d_kind = nullptr;
  unsigned long long *d_hits = nullptr;  // [kMaxSpecies][kMaxSurfaces] absorbed particles
  unsigned long long *d_seen = nullptr;  // same, already credited to σ
  bool any_floating = false;
};

struct Ctx {
  iskra_grid_t g{};
  int nx = 0, ny = 0, nn = 0;
  int tile_shift = kTileShiftDefault;                   // push tiles of 2^tile_shift cells per axis
  int tiles_x = 0, tiles_y = 0, ntiles = 0, nkeys = 0;  // push tiles; sort keys = ntiles * 4^tile_shift
  int ntiles_cap = 0, nkeys_cap = 0;                    // allocated for the largest of the tile sizes
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int device = 0, num_sms = 0;
  std::string err;
  std::vector<Species> species;
  // fields
  float2 *E32 = nullptr;       // (nx*ny) {Ex, Ey} at the nodes (MCC target term)
  double *E64 = nullptr;       // (nx*ny*3) download scratch
  bool e_from_phi = false;     // E comes from the last solve (E64 is rebuilt from ϕ on download)
  double *rho = nullptr;       // (nx*ny)
  double *rho_bg = nullptr;    // optional background charge density
  double *vol_inv = nullptr;   // 1 / cell_volume
  // ρ in double-float, formed on the FP32 pipes when the separable solver's
  // state is double-float (the FP64 copy is produced on demand)
  float2 *rho_df = nullptr, *vol_inv_df = nullptr, *bg_df = nullptr;
  bool rho64_valid = true;     // rho holds ρ
  bool warm_fused = false;     // the ρ pass of the step being queued ran the warm start
  // which copies of ρ / the densities a replay of the step graph leaves
  // current (recorded at capture, re-applied after replays)
  bool g_rho64 = true, g_rho_df = false;
  bool g_n64[kMaxSpecies] = {}, g_n_df[kMaxSpecies] = {};
  bool rho_df_valid = false;   // rho_df holds ρ
  int *d_err = nullptr;        // device error flags
  int *h_err = nullptr;        // pinned mirror
  // scratch for scans / sort
  int *cell_count = nullptr;   // (nkeys + 1)
  int *cell_cursor = nullptr;  // (nkeys + 1)
  int *scan_tmp = nullptr;
  double *stage = nullptr;     // upload/download staging (device)
  size_t stage_bytes = 0;
  // non-blocking field downloads: snapshot on the context stream into one of
  // two staging buffers (alternating), copy to the host on dl_stream
  double *dl_stage = nullptr;            // 2 x (nx*ny*3)
  cudaStream_t dl_stream = nullptr;
  cudaEvent_t dl_ready = nullptr, dl_done[2] = {nullptr, nullptr};
  bool dl_used[2] = {false, false};      // dl_done[b] recorded for staging buffer b
  int dl_next = 0;                       // staging buffer of the next download
  bool dl_pending = false;
  Poisson *ps = nullptr;
  Lws *lws = nullptr;
  std::vector<Mcc *> mccs;
  CircuitDev *cir_d = nullptr;
  CircuitDev cir_h{};
  bool has_circuit = false;
  int cir_pos_ref = -1, cir_neg_ref = -1;  // reference nodes of the electrodes
  int cir_wall = -1;                       // discard wall feeding the floating electrode
  unsigned long long *cir_seen = nullptr;  // absorbed counts already credited
  Tracker *trk = nullptr;                  // surface tracker (optional)
  void *sources = nullptr;                 // particle sources (source.cu)
  void *dsmcs = nullptr;                   // DSMC collision sets (dsmc.cu)

  // step state
  unsigned long long step = 0;  // steps completed by iskra_step
  int sort_every = -1;                   // > 0 fixed period, 0 never, < 0 per species from its speed
  double sort_scale = 1.0;               // factor on the speed-based periods (iskra_autotune_sort)
  int sort_period[kMaxSpecies] = {};     // steps between sorts of each species (0 = never)
  bool periods_valid = false;
  double periods_dt = 0;
  cudaGraphExec_t graph = nullptr;       // one PIC step
  cudaGraphExec_t sort_graph[kMaxSpecies] = {};  // tile sort of one species
  unsigned long long graph_kernels = 0, sort_graph_kernels[kMaxSpecies] = {};
  double *d_scratch = nullptr;           // 16 doubles of reduction scratch
  std::vector<void *> ensembles;         // ensembles built on this context (as template)
  void *mcc_work = nullptr;              // MCC work list (entries of the largest species)
  unsigned long long mcc_work_cap = 0;
  unsigned long long *mcc_nwork = nullptr;
  unsigned long long launches = 0;       // kernels launched by iskra_step
  double graph_dt = 0;
  double graph_rtol = 0;
  uint64_t graph_seed = 0;
  unsigned long long *d_step = nullptr;  // device step counter (graph reads it)
  unsigned long long d_step_known = ~0ull;  // value d_step holds, when known on the host
  unsigned long long d_step_host = 0;       // source of the d_step upload
};

// ---- double-float arithmetic (a value is hi + lo, two FP32 words, |lo| <=
// ulp(hi)/2: ~48 significant bits) with the error-free transformations
// two-sum (Knuth) and two-product by FMA.  GB300 runs FP32 at ~64x its FP64
// rate; the separable solver keeps ϕ, b and ρ in this form.
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 df_fast(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return make_float2(s, b - (s - a));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  float2 s = df_two_sum(a.x, b.x);
  s.y += a.y + b.y;
  return df_fast(s.x, s.y);
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  return df_fast(p, e);
}
__device__ __forceinline__ float2 df_add_f(float2 a, float b) {
  float2 s = df_two_sum(a.x, b);
  s.y += a.y;
  return df_fast(s.x, s.y);
}
__device__ __forceinline__ float2 df_from(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double df_value(float2 a) { return (double)a.x + (double)a.y; }
// an unsigned 64-bit integer as a double-float: three exact FP32 pieces
// of at most 24 bits, summed (error below 2^-48 relative)
__device__ __forceinline__ float2 df_from_u64(unsigned long long a) {
  const float p2 = (float)(unsigned)(a >> 48) * 281474976710656.0f;          // x 2^48, exact
  const float p1 = (float)(unsigned)((a >> 24) & 0xffffffu) * 16777216.0f;  // x 2^24, exact
  const float p0 = (float)(unsigned)(a & 0xffffffu);
  return df_add_f(df_add_f(make_float2(p2, 0.f), p1), p0);
}
// host split of a double into a double-float constant
inline float2 df_host(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

// ---- programmatic dependent launch ----
// Step kernels are launched with programmatic stream serialisation: the next
// kernel is scheduled while the previous one drains, and waits here (before
// its first access to anything an earlier kernel wrote) until that kernel
// has completed and its memory is visible.  Outside such a launch the wait
// returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... K, typename... A>
inline cudaError_t launch_pdl(void (*kern)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              A &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<A &&>(args)...);
}

// ---- helpers (ctx.cu) ----
int set_err(Ctx *c, int code, const std::string &msg);
int cuda_check(Ctx *c, cudaError_t e, const char *what);
int grid_blocks(Ctx *c, int threads, int per_sm);
int collect_device_errors(Ctx *c);   // synchronises
void invalidate_graphs(Ctx *c);      // the captured step no longer matches the setup
void set_tile_shift_geometry(Ctx *c, int ts);  // tiles_x, tiles_y, ntiles, nkeys of tile shift ts
int set_tile_shift(Ctx *c, int ts);   // new tile size: geometry, re-sort of every species, new step graph

#define ISKRA_CUDA(c, call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_check((c), e_, #call); \
  } while (0)

// ---- ensemble (batched runs) launchers ----
struct FieldRunsHost {
  int ns;
  unsigned long long *acc[kMaxSpecies];  // run 0 of each species' accumulator; run stride nn
  unsigned *cnt[kMaxSpecies];
  double scale[kMaxSpecies];             // w0 2^-48
  double q[kMaxSpecies];
  double *rho, *x;                       // R x nn
  float2 *E32;                           // R x nn
  const double *amp;                     // R x ngroups
  const unsigned long long *d_step;
  double dt;
  int *err;
};
int launch_field_runs(Ctx *c, int R, FieldRunsHost &H, cudaStream_t st);
int upload_particles(Ctx *c, const double *x, const double *v, const uint32_t *id, int64_t np, int64_t ld,
                     float4 *xv, float2 *zc, uint32_t *idd, unsigned *next_id = nullptr);
int download_particles(Ctx *c, const float4 *xv, const float2 *zc, const uint32_t *idd, long long np, double *x,
                       double *v, uint32_t *id, int64_t ld);
int launch_push_runs(Ctx *c, int sid, const SpeciesDev *runs, int R, const float2 *E2, float dt, int blocks_per_run,
                     int *err, cudaStream_t st, const PushSelect *sel = nullptr);
// phases of an MCC launch over runs: selection then collisions; collisions
// only (the work list was made by the previous step's push); selection only,
// for the step after the device step counter's (a list made before a step)
enum { kMccBoth = 0, kMccCollideOnly = 1, kMccSelectAhead = 2 };
int launch_mcc_runs(Ctx *c, int mid, double dt, int R, const SpeciesDev *src, const SpeciesDev *prod,
                    const uint2 *keys, unsigned long long *counts, const float2 *E32, int nn, int blocks_per_run,
                    void *work, unsigned long long *nwork, unsigned long long cap_work,
                    const unsigned long long *d_step, int *err, cudaStream_t st, int phases = kMccBoth);
int mcc_push_select(Ctx *c, int mid, double dt, PushSelect *S);
// bytes of a work list of R runs x cap entries: the entries, then one hit bit
// per entry (k_mcc_test -> k_mcc_collide)
size_t mcc_work_bytes(size_t R, size_t cap);
int ensure_mcc_work(Ctx *c);
void ensembles_detach(Ctx *c);
void mcc_key(uint64_t seed, int set_index, uint32_t &k0, uint32_t &k1);
int mcc_nproc(Ctx *c, int mid);
int mcc_download_nu(Ctx *c, int mid, unsigned *out);  // accepted collisions per node and process, then zeroed
int mcc_src(Ctx *c, int mid);
int mcc_prod(Ctx *c, int mid);
int mcc_set_index(Ctx *c, int mid);
int poisson_ndrive(Ctx *c);
int poisson_upload_fp64(Ctx *c);
int poisson_sync_x(Ctx *c);
int poisson_set_precision(Ctx *c, double rtol);
double poisson_drive_amp(Ctx *c, int g);

// ---- kernels / launchers shared across files ----
int launch_advance(Ctx *c, int sid, float dt);
// every species of a step (two in one launch when they can; that launch also
// advances step_ctr when given, reported through *folded)
int launch_advance_all(Ctx *c, float dt, unsigned long long *step_ctr, bool *folded);
int launch_deposit(Ctx *c, int sid);
int launch_charge_density(Ctx *c);
int launch_efield_from(Ctx *c, const double *phi);
int launch_efield64(Ctx *c, const double *phi);
int launch_sort(Ctx *c, int sid);
int species_speed2(Ctx *c, int sid, double *mean_v2);  // <vx² + vy²> of the live particles (synchronises)
int launch_mcc(Ctx *c, int mid, double dt, uint64_t seed, const unsigned long long *d_step, uint64_t step_host);
int launch_circuit(Ctx *c, double dt);
int launch_surface_charge(Ctx *c);  // σ credit of floating-electrode hits (after a push)
void tracker_destroy(Ctx *c);
int launch_step_sources(Ctx *c, double dt, uint64_t seed);  // sources sampled every step
void sources_destroy(Ctx *c);
int launch_step_dsmc(Ctx *c, double dt, uint64_t seed);     // DSMC sets of a step
void dsmc_destroy(Ctx *c);
int poisson_prepare(Ctx *c);
bool poisson_df_rho(Ctx *c);   // ρ of the next solve may be formed in double-float
int sync_rho64(Ctx *c);        // FP64 ρ up to date (particles.cu)
// the step solve's warm start (ϕ <- 2ϕ_n - ϕ_(n-1) on free rows), run inside
// the double-float ρ pass of a step
struct WarmArgs {
  const uint16_t *cls;         // row classes, fixed_bit on fixed rows
  float2 *xd, *xh;             // ϕ and the previous step's ϕ (double-float)
  int *hist;                   // xh is valid
  unsigned *ticket;            // blocks finished (last-block marking of hist)
  unsigned fixed_bit;
};
bool poisson_warm_args(Ctx *c, WarmArgs *w);
__device__ __forceinline__ void warm_node(const WarmArgs &W, bool hist, int k) {
  const float2 xa = W.xd[k];
  if (hist && !(W.cls[k] & W.fixed_bit)) W.xd[k] = df_add(make_float2(2.f * xa.x, 2.f * xa.y), df_neg(W.xh[k]));
  W.xh[k] = xa;
}

// Density of every species and ρ = Σ q n at one node in double-float
// (kinetic.jl:53, RegularGrids.jl:26-38, ParticleInCell.jl:118-122): the
// int64 node sums of the species whose deposit is unconsumed are turned into
// densities (and cleared), the others' stored densities enter as they are.
struct FinalizeDfArgs {
  int ns;
  unsigned long long *acc[kMaxSpecies];
  unsigned *cnt[kMaxSpecies];
  float2 *n[kMaxSpecies];
  float2 scale[kMaxSpecies];  // w0 * 2^-48
  float2 q[kMaxSpecies];
  int consume[kMaxSpecies];
};
__device__ __forceinline__ void finalize_df_node(const FinalizeDfArgs &A, const float2 *__restrict__ vol_inv,
                                                 const float2 *__restrict__ bg, float2 *__restrict__ rho, int k,
                                                 int &flags) {
  const float2 vi = vol_inv[k];
  float2 r = bg ? bg[k] : make_float2(0.f, 0.f);
  unsigned long long a[kMaxSpecies];
  unsigned cn[kMaxSpecies];
  float2 nold[kMaxSpecies];
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
#pragma unroll
  for (int s = 0; s < kMaxSpecies; s++) {
    if (s >= A.ns) break;
    float2 n;
    if (A.consume[s]) {
      if (cn[s] > kMaxCell) flags |= DERR_OVERFLOW;
      n = df_mul(df_mul(df_from_u64(a[s]), A.scale[s]), vi);
      A.n[s][k] = n;
      A.acc[s][k] = 0ull;
      A.cnt[s][k] = 0u;
    } else {
      n = nold[s];
    }
    r = df_add(r, df_mul(n, A.q[s]));
  }
  rho[k] = r;
}
int launch_step_density(Ctx *c);  // ρ of a graph step (with the fused warm start)
void poisson_destroy(Poisson *p);
void mcc_destroy(Mcc *m);

// learned warm start (lws.cu), called by CG solves after their first residual
struct LwsScal {               // device-resident scalars of the learned warm start
  double ss;                   // Σ r² of the solve's first (scaled) residual
  double inv_s, scale;         // 1/s and s·gain, s = RMS of r (both 0 when r = 0)
  double alpha;                // line-search step of the correction (0: not applied)
  double res2_before;          // squared residual norm before the correction
  double alpha_sum, ratio_sum; // over the applied corrections
  long long warm_solves;
};
bool lws_active(Ctx *c);
bool lws_harvesting(Ctx *c);
// queues the network on r; *y (device; nullptr unless in use mode) times
// *scale (device) is the predicted correction
int lws_begin(Ctx *c, const double *r, const float **y, const double **scale);
LwsScal *lws_scal(Ctx *c);
int lws_mark_start(Ctx *c, const double *phi);
int lws_end(Ctx *c, const double *phi, bool converged);
void lws_destroy_ctx(Ctx *c);

}  // namespace iskra

struct iskra_ctx {
  iskra::Ctx c;
};
