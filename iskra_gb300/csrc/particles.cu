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
#include "push.cuh"

namespace iskra {

// the 16 x 16-cell tile push of this translation unit; 8 x 8 and 32 x 32
// in push_t8.cu and push_t32.cu
ISKRA_PUSH_TILE_TU(4, t16)
cudaError_t push_tile_one_t8(cudaStream_t, bool, bool, const SpeciesDev &, const float2 *, const PushParams &, int,
                             int, int *);
cudaError_t push_tile_two_t8(cudaStream_t, bool, const SpeciesDev &, const SpeciesDev &, const float2 *,
                             const PushParams &, const PushParams &, int, int, int *, unsigned long long *);
cudaError_t push_tile_one_t32(cudaStream_t, bool, bool, const SpeciesDev &, const float2 *, const PushParams &, int,
                              int, int *);
cudaError_t push_tile_two_t32(cudaStream_t, bool, const SpeciesDev &, const SpeciesDev &, const float2 *,
                              const PushParams &, const PushParams &, int, int, int *, unsigned long long *);

cudaError_t push_tile_one(int ts, cudaStream_t st, bool push, bool trk, const SpeciesDev &s, const float2 *E2,
                          const PushParams &P, int ntiles, int blocks, int *err) {
  switch (ts) {
    case 3: return push_tile_one_t8(st, push, trk, s, E2, P, ntiles, blocks, err);
    case 4: return push_tile_one_t16(st, push, trk, s, E2, P, ntiles, blocks, err);
    case 5: return push_tile_one_t32(st, push, trk, s, E2, P, ntiles, blocks, err);
  }
  return cudaErrorInvalidValue;
}

cudaError_t push_tile_two(int ts, cudaStream_t st, bool trk, const SpeciesDev &a, const SpeciesDev &b,
                          const float2 *E2, const PushParams &Pa, const PushParams &Pb, int ntiles, int blocks,
                          int *err, unsigned long long *step_ctr) {
  switch (ts) {
    case 3: return push_tile_two_t8(st, trk, a, b, E2, Pa, Pb, ntiles, blocks, err, step_ctr);
    case 4: return push_tile_two_t16(st, trk, a, b, E2, Pa, Pb, ntiles, blocks, err, step_ctr);
    case 5: return push_tile_two_t32(st, trk, a, b, E2, Pa, Pb, ntiles, blocks, err, step_ctr);
  }
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
  ISKRA_CUDA(c, push_tile_one(c->tile_shift, c->stream, true, c->trk != nullptr, s.dev, c->E32, push_params(c, s, dt),
                              c->ntiles, push_blocks(c), c->d_err));
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
    ISKRA_CUDA(c, push_tile_two(c->tile_shift, c->stream, c->trk != nullptr, a.dev, b.dev, c->E32, Pa, Pb, c->ntiles,
                                blocks, c->d_err, step_ctr));
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
  ISKRA_CUDA(c, push_tile_one(c->tile_shift, c->stream, false, false, s.dev, c->E32, P, c->ntiles, push_blocks(c),
                              c->d_err));
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
__global__ void __launch_bounds__(256) k_hist(SpeciesDev s, int tiles_x, int ts, int *__restrict__ count) {
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
      if (cell >= 0) key = cell_key(cell & 0xffff, cell >> 16, tiles_x, ts);
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
// receives the entries at the multiples of 4^ts (the first slot of each tile)
__global__ void __launch_bounds__(1024) k_scan_down(const int *__restrict__ in, int n, const int *__restrict__ part,
                                                    int *__restrict__ out, int *__restrict__ tile_begin, int ts) {
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
  const int tsh = 2 * ts, kmask = (1 << tsh) - 1;
  for (int k = 0; k < 4; k++) {
    long long idx = b0 + threadIdx.x * 4 + k;
    if (idx < n) {
      out[idx] = e;
      if ((idx & kmask) == 0) tile_begin[idx >> tsh] = e;
    }
    e += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) {  // grand total
    out[n] = e;
    tile_begin[n >> tsh] = e;
  }
}

__global__ void __launch_bounds__(256) k_scatter(SpeciesDev s, int tiles_x, int ts, int *__restrict__ cursor) {
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
      if (cell >= 0) key = cell_key(cell & 0xffff, cell >> 16, tiles_x, ts);
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

// A new push tile size: the tile geometry, a sort of every species by the new
// tile-major keys (so tile_begin describes the new tiles) and new graphs.
int set_tile_shift(Ctx *c, int ts) {
  if (ts < kTileShiftMin || ts > kTileShiftMax) return set_err(c, ISKRA_EINVAL, "tile size must be 8, 16 or 32 cells");
  if (ts == c->tile_shift) return ISKRA_OK;
  set_tile_shift_geometry(c, ts);
  invalidate_graphs(c);
  for (int s = 0; s < (int)c->species.size(); s++) {
    const int rc = launch_sort(c, s);
    if (rc) return rc;
  }
  return ISKRA_OK;
}

int launch_sort(Ctx *c, int sid) {
  Species &s = c->species[sid];
  const int nk = c->nkeys;
  ISKRA_CUDA(c, cudaMemsetAsync(c->cell_count, 0, (size_t)(nk + 1) * sizeof(int), c->stream));
  int blocks = sort_blocks(c, s);
  k_hist<<<blocks, 256, 0, c->stream>>>(s.dev, c->tiles_x, c->tile_shift, c->cell_count);
  ISKRA_CUDA(c, cudaGetLastError());
  int nb = (nk + kScanItems - 1) / kScanItems;
  k_scan_reduce<<<nb, 1024, 0, c->stream>>>(c->cell_count, nk, c->scan_tmp);
  k_scan_top<<<1, 1024, 0, c->stream>>>(c->scan_tmp, nb);
  k_scan_down<<<nb, 1024, 0, c->stream>>>(c->cell_count, nk, c->scan_tmp, c->cell_cursor, s.dev.tile_begin,
                                          c->tile_shift);
  ISKRA_CUDA(c, cudaGetLastError());
  // cell_count is free again: keep the grand total there for k_sort_finish
  ISKRA_CUDA(c, cudaMemcpyAsync(c->cell_count + nk, c->cell_cursor + nk, sizeof(int), cudaMemcpyDeviceToDevice,
                                c->stream));
  k_scatter<<<blocks, 256, 0, c->stream>>>(s.dev, c->tiles_x, c->tile_shift, c->cell_cursor);
  k_sort_finish<<<1, 1, 0, c->stream>>>(s.dev.st, c->cell_count + nk);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// Appends a warp's n <= 32 buffered work-list entries to its run's list
// (counter cnt, segment seg of cap entries).
__device__ __forceinline__ void flush_entries(const MccWork *buf, int n, unsigned long long *cnt,
                                              MccWork *__restrict__ seg, unsigned long long cap, int &flags) {
  const int lane = threadIdx.x & 31;
  __syncwarp();  // the entries are in buf
  unsigned long long at = 0;
  if (lane == 0) at = atomicAdd(cnt, (unsigned long long)n);
  at = __shfl_sync(0xffffffffu, at, 0) + (unsigned)lane;
  if (lane < n) {
    if (at < cap) seg[at] = buf[lane];
    else flags |= DERR_CAPACITY;
  }
  __syncwarp();  // buf may be written again
}

// ---------------------------------------------------------------------------
// ensemble push: run r = blockIdx.y; every block of a run stages the run's
// whole E grid (cx*cy <= kEnsWinCells cells), pushes a grid-stride share of the
// run's particles (any order), deposits into shared memory and adds the
// node sums to the run's accumulator.
// ---------------------------------------------------------------------------
//
// SEL: the species is the source of an MCC set, and the push also makes the
// set's work list for the next step -- each pushed particle that stays draws
// its selection count for step + 1 from the hash of (set key, step + 1, id)
// (the draw k_mcc_select would make at the start of that step: nothing
// changes the particle in between) and, when selected, its new record goes
// to the run's list.  The next step's collision pass then starts without a selection pass
// over all particles.
template <int MX, int MY, bool SEL>
__global__ void __launch_bounds__(256, ISKRA_PUSH_RUNS_MIN_BLOCKS) k_push_runs(const SpeciesDev *__restrict__ runs,
                                                                          const float2 *__restrict__ E2, int nnode,
                                                                          PushParams P, int *err, PushSelect S) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char push_runs_smem[];
  PushShared &sh = *reinterpret_cast<PushShared *>(push_runs_smem);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  const int r = blockIdx.y;
  const SpeciesDev s = runs[r];
  const int nx = P.nx, cx = P.nx - 1, cy = P.ny - 1;
  E2 += (size_t)r * nnode;
  // the window is the run's whole grid: its nodes are the grid's
  for (int t = threadIdx.x; t < nnode; t += blockDim.x) sh.ne[t] = __ldg(E2 + t);
  for (int t = threadIdx.x; t < cx * cy; t += blockDim.x) window_clear(sh, t);
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
  // The records stream through the warp's ring of kEnsStages shared-memory
  // stages filled by cp.async: two later iterations' records are in flight
  // while one is pushed (the loop was bound by the load latency); each lane
  // reads back only its own copies.  The identifier (for the selection draw)
  // is loaded one iteration ahead.  Slots of later iterations are no slots
  // this iteration's push writes.
  const long long stride = nwarps * 32;
#pragma unroll
  for (int d = 0; d < kEnsStages - 1; d++) {
    const long long q = warp * 32 + d * stride + lane;
    if (q < np) cp_async_record(&sh.ra[wib][d][lane], &sh.rb[wib][d][lane], xv + q, zc + q);
    cp_async_commit();
  }
  uint32_t idn = 0;
  if (SEL && warp * 32 + lane < np) idn = ids[warp * 32 + lane];
  // A warp's selected entries gather in its shared-memory buffer and go to
  // the run's list 32 at a time: one reservation (an atomic on the run's
  // counter, which every warp of the run shares) per 32 entries instead of
  // one per iteration, and 1 KB contiguous stores.  nbuf: entries buffered
  // (warp-uniform, < 32 between iterations).
  MccWork(&wbuf)[8][64] = sh.wbuf;
  int nbuf = 0;
  int st = 0;  // ring stage of the current iteration
  for (long long base = warp * 32; base < np; base += stride) {
    const long long p = base + lane;
    const bool v = p < np;
    {
      const long long q = p + (kEnsStages - 1) * stride;
      const int sn = st == 0 ? kEnsStages - 1 : st - 1;  // the stage read one iteration ago
      if (q < np) cp_async_record(&sh.ra[wib][sn][lane], &sh.rb[wib][sn][lane], xv + q, zc + q);
      cp_async_commit();
    }
    cp_async_wait<kEnsStages - 1>();  // this lane's copies of the current stage have landed
    const float4 a = sh.ra[wib][st][lane];
    const float2 b = sh.rb[wib][st][lane];
    st = st + 1 == kEnsStages ? 0 : st + 1;
    const uint32_t idc = idn;
    if (SEL && p + stride < np) idn = ids[p + stride];
    float4 na;
    float2 nb;
    push_warp<true, MX, MY, true>(s, xv, zc, p, v, a, b, E2, sh, 0, 0, cx, cy, P, ab, flags, SEL ? &na : nullptr,
                                  SEL ? &nb : nullptr);
    if (SEL) {
      int nsel = 0;
      uint32_t pid = 0;
      if (v && __float_as_int(nb.y) >= 0) {
        pid = idc;
        nsel = draw_selections(selection_uniform(pid, step1, key), S.lam, expl);
      }
      const unsigned m = __ballot_sync(FULL, nsel > 0);
      if (nsel > 0) wbuf[wib][nbuf + __popc(m & ((1u << lane) - 1u))] = mcc_entry(na, nb, pid, (uint32_t)p);
      nbuf += __popc(m);
      if (nbuf >= 32) {
        flush_entries(wbuf[wib], 32, S.nwork + (size_t)r * kNworkStride, seg, S.cap_run, flags);
        nbuf -= 32;
        if (lane < nbuf) wbuf[wib][lane] = wbuf[wib][32 + lane];
        __syncwarp();
      }
    }
  }
  if (SEL && nbuf) flush_entries(wbuf[wib], nbuf, S.nwork + (size_t)r * kNworkStride, seg, S.cap_run, flags);
  cp_async_wait<0>();  // no copy is in flight when the block leaves the ring
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
  if ((c->nx - 1) * (c->ny - 1) > kEnsWinCells)
    return set_err(c, ISKRA_EINVAL, "ensemble grid larger than one window");
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
  const dim3 grid(std::max(1, blocks_per_run * ISKRA_PUSH_RUNS_SCALE8 / 8), R);
  const PushSelect S = sel ? *sel : PushSelect{};
#define ISKRA_PUSH_RUNS_CASE(MX, MY)                                                                           \
  if (P.mode_x == MX && P.mode_y == MY) {                                                                       \
    auto kern = sel ? k_push_runs<MX, MY, true> : k_push_runs<MX, MY, false>;                                   \
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,                                  \
                         (int)cudaSharedmemCarveoutMaxShared);                                                  \
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PushShared));          \
    ISKRA_CUDA(c, launch_pdl(kern, grid, 256, sizeof(PushShared), st, runs, E2, nnode, P, err, S));            \
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
