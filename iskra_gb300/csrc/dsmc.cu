// dsmc.cu -- Direct Simulation Monte Carlo between two kinetic species
// (Chemistry/src/dsmc.jl): PIC.perform!(::DirectSimulationMonteCarlo, E, Δt,
// config) (:86-138) with perform!(::DSMC.ElasticCollision, s, t) (:31-84),
// the only collision kind the reference implements.
//
// Each perform! buckets the live particles of both species by cell (the
// reference's cache!, :24-29: counts, an exclusive scan, a scatter of slot
// indices), then a warp per cell orders its two index lists by particle
// identifier (so the random picks do not depend on memory order), stages the
// velocities in shared memory and runs the reference's loop for the cell in
// order with the warp: Nc from the cell counts
// and the remainder carried from the last step, floor(Nc) random pairs, each
// accepted with probability σ(g) g / σgmax and scattered isotropically in
// the centre-of-mass frame.  Cells hold disjoint particles, so the cells run
// in parallel without conflicts.  Randomness: Philox keyed by (seed, set,
// step, cell, pair).
#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "internal.cuh"

namespace iskra {

struct Dsmc {
  int a = 0, b = 0;             // source, target species
  int ntab = 0;
  float *d_tab = nullptr;       // g[ntab] then σ[ntab] (FP32, for sigma_at)
  double sgmax = 0;             // maximum(σ) * argmax(σ) (dsmc.jl:101)
  double *remaining = nullptr;  // collisions_remaining per cell (nn)
  int *cnt = nullptr;           // [2][nn + 1] per-cell counts, then exclusive offsets
  int *fill = nullptr;          // [2][nn] scatter cursors
  unsigned *idx[2] = {nullptr, nullptr};  // slot indices by cell, per species
  unsigned *ord[2] = {nullptr, nullptr};  // the lists of crowded cells in identifier order
  unsigned *nu = nullptr;       // accepted collisions per cell, last perform! (the "nuDSMC" field)
};

struct DsmcArgs {
  SpeciesDev s[2];
  double m[2], w[2];
  const float *tab;
  int ntab;
  double sgmax, dt, inv_area;   // 1 / (Δx Δy)
  int nn;
  bool same;                    // source and target are one species
  double *remaining;
  int *cnt[2], *fill[2];
  unsigned *idx[2], *ord[2];
  unsigned *nu;
  uint32_t k0, k1, set;
  const unsigned long long *step;
  unsigned long long step_value;
};

// cache! (dsmc.jl:24-29): per-cell counts of the live particles
// (cells numbered like nodes: i0 + nx j0 from the packed cell i0 | j0 << 16)
__global__ void k_dsmc_count(SpeciesDev s, int nx, int *__restrict__ cnt) {
  pdl_wait();
  const long long np = s.st->np;
  const float2 *zc = pick(s.zc[0], s.zc[1], s.st->cur);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    const int cell = __float_as_int(zc[p].y);
    if (cell >= 0) atomicAdd(&cnt[(cell & 0xffff) + nx * (cell >> 16)], 1);
  }
}

// exclusive scan of the counts in place (one block; DSMC grids are small and
// this is not the hot path): cnt[k] <- sum of cnt[0..k), cnt[n] <- total
__global__ void k_dsmc_scan(int *__restrict__ cnt, int n) {
  __shared__ int part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int per = (n + T - 1) / T;
  const int lo = min(n, t * per), hi = min(n, lo + per);
  int s = 0;
  for (int k = lo; k < hi; k++) s += cnt[k];
  part[t] = s;
  __syncthreads();
  for (int d = 1; d < T; d <<= 1) {  // inclusive scan of the partials
    const int v = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = t ? part[t - 1] : 0;
  for (int k = lo; k < hi; k++) {
    const int c = cnt[k];
    cnt[k] = run;
    run += c;
  }
  if (t == T - 1) cnt[n] = part[T - 1];
}

__global__ void k_dsmc_scatter(SpeciesDev s, int nx, const int *__restrict__ start, int *__restrict__ fill,
                               unsigned *__restrict__ idx) {
  const long long np = s.st->np;
  const float2 *zc = pick(s.zc[0], s.zc[1], s.st->cur);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    const int cell = __float_as_int(zc[p].y);
    if (cell < 0) continue;
    const int k = (cell & 0xffff) + nx * (cell >> 16);
    idx[start[k] + atomicAdd(&fill[k], 1)] = (unsigned)p;
  }
}

// a cell's slots ordered by particle identifier (insertion sort: cells hold
// few particles), so the picks depend neither on the order the scatter wrote
// them in nor on where the sort left the particles in memory
__device__ __forceinline__ float3 vel_of(const SpeciesDev &s, unsigned p) {
  const int cur = s.st->cur;
  const float4 a = pick(s.xv[0], s.xv[1], cur)[p];
  const float2 b = pick(s.zc[0], s.zc[1], cur)[p];
  return make_float3(a.z, a.w, b.x);
}
__device__ __forceinline__ void set_vel(const SpeciesDev &s, unsigned p, float3 v) {
  const int cur = s.st->cur;
  float4 *xv = pick(s.xv[0], s.xv[1], cur);
  float2 *zc = pick(s.zc[0], s.zc[1], cur);
  const float4 a = xv[p];
  xv[p] = make_float4(a.x, a.y, v.x, v.y);
  zc[p] = make_float2(v.z, zc[p].y);
}

// The pairs of one cell in order (dsmc.jl:108-133), by the whole warp:
// ncol pairs from the id-ordered lists (positions ra < Na, rb < Nb), pair c
// drawing its own random numbers (Philox keyed by (seed, set, step, cell,
// c)), accepted with probability σ(g) g / σgmax and scattered by
// perform!(::ElasticCollision) (dsmc.jl:31-84, vss_inv = 1: an isotropic
// direction for the relative velocity in the CM frame).  The 32 lanes test
// 32 consecutive pairs against the current velocities; the first accepted
// one collides (its lane writes the velocities) and the test resumes after
// it, so the outcome is that of testing the pairs one by one (acceptance is
// rare: the 05_dsmc problem accepts ~1 pair in 1500).  A pair of one species
// draws its second particle among the other Nb - 1 (the reference redraws
// until they differ, :112-114: the same distribution).  get/set reach the
// velocities of the r-th particle of each list (shared or global memory).
// Returns the accepted collisions (on every lane).
template <class GA, class SA, class GB, class SB>
__device__ unsigned dsmc_pairs(const DsmcArgs &A, int cell, unsigned long long step, long long ncol, int Na, int Nb,
                               int lane, GA get_a, SA set_a, GB get_b, SB set_b) {
  const unsigned FULL = 0xffffffffu;
  const double Wa = A.w[0], Wb = A.w[1];
  const float ma = (float)A.m[0], mb = (float)A.m[1];
  const float mr1 = ma / (ma + mb), mr2 = mb / (ma + mb);
  const float sgmax = (float)A.sgmax;
  const float *gt = A.tab, *st = A.tab + A.ntab;
  const uint32_t k1 = A.k1 ^ (uint32_t)(step >> 32);
  unsigned accepted = 0;
  long long c = 0;
  while (c < ncol) {
    const long long my = c + lane;
    bool acc = false;
    int ra = 0, rb = 0;
    U4 r0{0, 0, 0, 0}, r1{0, 0, 0, 0};
    float3 va{0, 0, 0}, vb{0, 0, 0};
    float g = 0.f;
    if (my < ncol) {
      r0 = philox4x32_10(U4{(uint32_t)my, (uint32_t)cell, (uint32_t)step, A.set}, A.k0, k1);
      r1 = philox4x32_10(U4{(uint32_t)my, (uint32_t)cell, (uint32_t)step, A.set | 0x80000000u}, A.k0, k1);
      ra = min(Na - 1, (int)(u01(r0.x) * Na));
      if (A.same) rb = (ra + 1 + min(Nb - 2, (int)(u01(r0.y) * (Nb - 1)))) % Nb;
      else rb = min(Nb - 1, (int)(u01(r0.y) * Nb));
      va = get_a(ra);
      vb = get_b(rb);
      const float gx = va.x - vb.x, gy = va.y - vb.y, gz = va.z - vb.z;
      g = sqrtf(gx * gx + gy * gy + gz * gz);
      const float P = sigma_at(gt, st, A.ntab, g, 0, 0.f, 0.f) * g / sgmax;
      acc = !(P < u01(r0.z));
    }
    const unsigned m = __ballot_sync(FULL, acc);
    if (m == 0u) {
      c += 32;
      continue;
    }
    const int f = __ffs(m) - 1;
    if (lane == f) {
      const float vcx = mr1 * va.x + mr2 * vb.x, vcy = mr1 * va.y + mr2 * vb.y, vcz = mr1 * va.z + mr2 * vb.z;
      const float B = 2.0f * u01(r0.w) - 1.0f;
      const float Aa = sqrtf(fmaxf(1.0f - B * B, 0.0f));
      float sC, cC;
      sincospif(2.0f * u01(r1.x), &sC, &cC);
      const float rx = g * B, ry = g * Aa * cC, rz = g * Aa * sC;
      if (A.w[0] == A.w[1]) {
        set_a(ra, make_float3(vcx + mr2 * rx, vcy + mr2 * ry, vcz + mr2 * rz));
        set_b(rb, make_float3(vcx - mr1 * rx, vcy - mr1 * ry, vcz - mr1 * rz));
      } else {  // unequal weights (dsmc.jl:72-83)
        const float u = u01(r1.y);
        if ((float)(Wb / Wa) > u) set_a(ra, make_float3(vcx + mr2 * rx, vcy + mr2 * ry, vcz + mr2 * rz));
        if ((float)(Wa / Wb) > u) set_b(rb, make_float3(vcx - mr2 * rx, vcy - mr2 * ry, vcz - mr2 * rz));
      }
    }
    __syncwarp();
    accepted++;
    c += f + 1;
  }
  return accepted;
}

// cells whose lists fit are staged in shared memory: the pair loop then
// waits on shared-memory loads instead of dependent global ones
constexpr int kDsmcStage = 512;
struct __align__(16) DsmcShared {  // 16-byte aligned: tid is read as uint4
  float3 va[kDsmcStage], vb[kDsmcStage];      // velocities, id order
  unsigned sa[kDsmcStage], sb[kDsmcStage];    // slots, id order
  unsigned tslot[kDsmcStage];                 // a list as scattered
  uint32_t tid[kDsmcStage];                   // its identifiers
};

// the list l[0..n) ordered by identifier into out (ids are unique: each
// element's rank is the number of smaller ids); the warp's lanes share it
__device__ __forceinline__ void warp_rank_sort(const unsigned *__restrict__ l, int n, const uint32_t *__restrict__ id,
                                               DsmcShared &sh, unsigned *out, int lane) {
  for (int e = lane; e < n; e += 32) {
    sh.tslot[e] = l[e];
    sh.tid[e] = id[l[e]];
  }
  __syncwarp();
  for (int e = lane; e < n; e += 32) {
    const uint32_t key = sh.tid[e];
    int r = 0;
    for (int q = 0; q < n; q++) r += sh.tid[q] < key;
    out[r] = sh.tslot[e];
  }
  __syncwarp();
}

// The same order for a list of any length, into global memory: each lane
// ranks one element of every 32 against all ids, staged through shared
// memory kDsmcStage at a time (n²/32 shared-memory compares per lane, no
// dependent global loads).
__device__ void warp_rank_sort_long(const unsigned *__restrict__ l, int n, const uint32_t *__restrict__ id,
                                    DsmcShared &sh, unsigned *__restrict__ out, int lane) {
  for (int g = 0; g < n; g += 32) {
    const int e = g + lane;
    const unsigned slot = e < n ? l[e] : 0u;
    const uint32_t key = e < n ? id[slot] : 0u;
    int r = 0;
    for (int c0 = 0; c0 < n; c0 += kDsmcStage) {
      const int m = min(kDsmcStage, n - c0);
      __syncwarp();
      for (int q = lane; q < m; q += 32) sh.tid[q] = id[l[c0 + q]];
      __syncwarp();
      int q = 0;
      for (; q + 4 <= m; q += 4) {
        const uint4 t = *reinterpret_cast<const uint4 *>(sh.tid + q);
        r += (t.x < key) + (t.y < key) + (t.z < key) + (t.w < key);
      }
      for (; q < m; q++) r += sh.tid[q] < key;
    }
    if (e < n) out[r] = slot;
  }
  __syncwarp();
}

// PIC.perform!(dsmc, ...) for one cell (dsmc.jl:103-134), a warp per cell.
// Cells are numbered like nodes (i0 + nx j0; the reference's (i0+1, j0+1)).
__global__ void __launch_bounds__(32) k_dsmc_cells(DsmcArgs A) {
  pdl_wait();
  __shared__ DsmcShared sh;
  const int k = blockIdx.x, lane = threadIdx.x;
  const int sa0 = A.cnt[0][k], Na = A.cnt[0][k + 1] - sa0;
  const int sb0 = A.cnt[1][k], Nb = A.cnt[1][k + 1] - sb0;
  if (Na < 2 || Nb < 2) {
    if (lane == 0) A.nu[k] = 0u;
    return;
  }
  // Nc = na Nb Δt σgmax / (Pab + (Wb/Wa) Pba), doubled for two species,
  // plus the remainder of the last step (dsmc.jl:94-117)
  const double Wa = A.w[0], Wb = A.w[1];
  double Pab = 1.0, Pba = 1.0;
  if (Wa > Wb) Pab = Wb / Wa;
  else Pba = Wa / Wb;
  const double na = Na * Wa * A.inv_area;
  double Nc = na * Nb * A.dt * A.sgmax;
  Nc /= Pab + (Wb / Wa) * Pba;
  if (!A.same) Nc *= 2.0;
  Nc += A.remaining[k];
  const double fl = floor(Nc);
  const long long ncol = (long long)fl;
  const unsigned long long step = A.step ? *A.step : A.step_value;
  const SpeciesDev &S0 = A.s[0], &S1 = A.s[1];
  const uint32_t *id0 = pick(S0.id[0], S0.id[1], S0.st->cur);
  const uint32_t *id1 = pick(S1.id[0], S1.id[1], S1.st->cur);
  unsigned *la = A.idx[0] + sa0, *lb = A.idx[1] + sb0;
  if (Na <= kDsmcStage && Nb <= kDsmcStage) {
    warp_rank_sort(la, Na, id0, sh, sh.sa, lane);
    if (!A.same) warp_rank_sort(lb, Nb, id1, sh, sh.sb, lane);
    for (int r = lane; r < Na; r += 32) sh.va[r] = vel_of(S0, sh.sa[r]);
    if (!A.same)
      for (int r = lane; r < Nb; r += 32) sh.vb[r] = vel_of(S1, sh.sb[r]);
    __syncwarp();
    float3 *vb = A.same ? sh.va : sh.vb;
    auto ga = [&](int r) { return sh.va[r]; };
    auto sa = [&](int r, float3 v) { sh.va[r] = v; };
    auto gb = [&](int r) { return vb[r]; };
    auto sb = [&](int r, float3 v) { vb[r] = v; };
    const unsigned nacc = dsmc_pairs(A, k, step, ncol, Na, Nb, lane, ga, sa, gb, sb);
    if (lane == 0) {
      A.nu[k] = nacc;
      A.remaining[k] = Nc - fl;
    }
    __syncwarp();
    for (int r = lane; r < Na; r += 32) set_vel(S0, sh.sa[r], sh.va[r]);
    if (!A.same)
      for (int r = lane; r < Nb; r += 32) set_vel(S1, sh.sb[r], sh.vb[r]);
    return;
  }
  // a crowded cell: lists ranked into identifier order in global memory,
  // velocities in global memory
  {
    unsigned *oa = A.ord[0] + sa0;
    warp_rank_sort_long(la, Na, id0, sh, oa, lane);
    la = oa;
    if (!A.same) {
      unsigned *ob = A.ord[1] + sb0;
      warp_rank_sort_long(lb, Nb, id1, sh, ob, lane);
      lb = ob;
    } else {
      lb = oa;
    }
  }
  auto ga = [&](int r) { return vel_of(S0, la[r]); };
  auto sa = [&](int r, float3 v) { set_vel(S0, la[r], v); };
  auto gb = [&](int r) { return vel_of(S1, lb[r]); };
  auto sb = [&](int r, float3 v) { set_vel(S1, lb[r], v); };
  const unsigned nacc = dsmc_pairs(A, k, step, ncol, Na, Nb, lane, ga, sa, gb, sb);
  if (lane == 0) {
    A.nu[k] = nacc;
    A.remaining[k] = Nc - fl;
  }
}

static std::vector<Dsmc *> &dsmc_of(Ctx *c) { return *reinterpret_cast<std::vector<Dsmc *> *>(c->dsmcs); }

static void dsmc_free(Dsmc *d) {
  cudaFree(d->d_tab);
  cudaFree(d->remaining);
  cudaFree(d->cnt);
  cudaFree(d->fill);
  cudaFree(d->idx[0]);
  if (d->idx[1] != d->idx[0]) cudaFree(d->idx[1]);
  cudaFree(d->ord[0]);
  if (d->ord[1] != d->ord[0]) cudaFree(d->ord[1]);
  cudaFree(d->nu);
  delete d;
}

void dsmc_destroy(Ctx *c) {
  if (!c->dsmcs) return;
  for (Dsmc *d : dsmc_of(c)) dsmc_free(d);
  delete reinterpret_cast<std::vector<Dsmc *> *>(c->dsmcs);
  c->dsmcs = nullptr;
}

int launch_dsmc(Ctx *c, int k, double dt, uint64_t seed, const unsigned long long *step,
                unsigned long long step_value) {
  Dsmc *d = dsmc_of(c)[k];
  const int nn = c->nn;
  ISKRA_CUDA(c, cudaMemsetAsync(d->cnt, 0, 2 * (size_t)(nn + 1) * sizeof(int), c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(d->fill, 0, 2 * (size_t)nn * sizeof(int), c->stream));
  const int blocks = c->num_sms * 4;
  const int nsp = d->a == d->b ? 1 : 2;
  for (int q = 0; q < nsp; q++) {
    const Species &sp = c->species[q == 0 ? d->a : d->b];
    k_dsmc_count<<<blocks, 256, 0, c->stream>>>(sp.dev, c->nx, d->cnt + (size_t)q * (nn + 1));
    k_dsmc_scan<<<1, 1024, 0, c->stream>>>(d->cnt + (size_t)q * (nn + 1), nn);
    k_dsmc_scatter<<<blocks, 256, 0, c->stream>>>(sp.dev, c->nx, d->cnt + (size_t)q * (nn + 1),
                                                   d->fill + (size_t)q * nn, d->idx[q]);
  }
  ISKRA_CUDA(c, cudaGetLastError());
  DsmcArgs A{};
  A.s[0] = c->species[d->a].dev;
  A.s[1] = c->species[d->b].dev;
  A.m[0] = c->species[d->a].m;
  A.m[1] = c->species[d->b].m;
  A.w[0] = c->species[d->a].w0;
  A.w[1] = c->species[d->b].w0;
  A.tab = d->d_tab;
  A.ntab = d->ntab;
  A.sgmax = d->sgmax;
  A.dt = dt;
  A.inv_area = 1.0 / (c->g.dx * c->g.dy);
  A.nn = nn;
  A.same = d->a == d->b;
  A.remaining = d->remaining;
  A.cnt[0] = d->cnt;
  A.cnt[1] = d->cnt + (A.same ? 0 : (size_t)(nn + 1));
  A.fill[0] = d->fill;
  A.fill[1] = d->fill + (A.same ? 0 : (size_t)nn);
  A.idx[0] = d->idx[0];
  A.idx[1] = A.same ? d->idx[0] : d->idx[1];
  A.ord[0] = d->ord[0];
  A.ord[1] = A.same ? d->ord[0] : d->ord[1];
  A.nu = d->nu;
  A.k0 = (uint32_t)seed;
  A.k1 = (uint32_t)(seed >> 32) ^ 0xD5AC0000u;
  A.set = (uint32_t)k;
  A.step = step;
  A.step_value = step_value;
  ISKRA_CUDA(c, launch_pdl(k_dsmc_cells, nn, 32, 0, c->stream, A));
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

int launch_step_dsmc(Ctx *c, double dt, uint64_t seed) {
  if (!c->dsmcs) return ISKRA_OK;
  for (int k = 0; k < (int)dsmc_of(c).size(); k++) {
    int rc = launch_dsmc(c, k, dt, seed, c->d_step, 0);
    if (rc) return rc;
  }
  return ISKRA_OK;
}

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_dsmc_create(iskra_ctx *h, int source, int target, const double *g, const double *sigma, int n, int *set) {
  if (!h || !g || !sigma || n < 1) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  const int ns = (int)c->species.size();
  if (source < 0 || source >= ns || target < 0 || target >= ns) return set_err(c, ISKRA_EINVAL, "bad species");
  for (int k = 0; k < n; k++)
    if (!std::isfinite(g[k]) || !std::isfinite(sigma[k]) || (k && !(g[k] > g[k - 1])))
      return set_err(c, ISKRA_EINVAL, "cross section: finite values, increasing g");
  Dsmc *d = new (std::nothrow) Dsmc();
  if (!d) return ISKRA_ENOMEM;
  d->a = source;
  d->b = target;
  d->ntab = n;
  // σgmax = maximum(rate) * argmax(rate) (dsmc.jl:101, cross_section.jl:15-16:
  // the largest σ times the g of its first occurrence)
  int im = 0;
  for (int k = 1; k < n; k++)
    if (sigma[k] > sigma[im]) im = k;
  d->sgmax = sigma[im] * g[im];
  if (!(d->sgmax > 0.0)) {
    delete d;
    return set_err(c, ISKRA_EINVAL, "cross section: max(σ) * argmax(σ) must be positive");
  }
  std::vector<float> tab(2 * n);
  for (int k = 0; k < n; k++) {
    tab[k] = (float)g[k];
    tab[n + k] = (float)sigma[k];
  }
  const size_t nn = c->nn;
  const Species &A = c->species[source], &B = c->species[target];
  bool ok = cudaMalloc(&d->d_tab, tab.size() * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&d->remaining, nn * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&d->cnt, 2 * (nn + 1) * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&d->fill, 2 * nn * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&d->idx[0], (size_t)std::max(1LL, A.cap) * sizeof(unsigned)) == cudaSuccess &&
            cudaMalloc(&d->ord[0], (size_t)std::max(1LL, A.cap) * sizeof(unsigned)) == cudaSuccess &&
            cudaMalloc(&d->nu, nn * sizeof(unsigned)) == cudaSuccess;
  if (ok && source != target)
    ok = cudaMalloc(&d->idx[1], (size_t)std::max(1LL, B.cap) * sizeof(unsigned)) == cudaSuccess &&
         cudaMalloc(&d->ord[1], (size_t)std::max(1LL, B.cap) * sizeof(unsigned)) == cudaSuccess;
  if (source == target) {
    d->idx[1] = d->idx[0];
    d->ord[1] = d->ord[0];
  }
  if (!ok) {
    dsmc_free(d);
    return set_err(c, ISKRA_ENOMEM, "out of device memory for DSMC");
  }
  ISKRA_CUDA(c, cudaMemcpy(d->d_tab, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice));
  ISKRA_CUDA(c, cudaMemset(d->remaining, 0, nn * sizeof(double)));
  ISKRA_CUDA(c, cudaMemset(d->nu, 0, nn * sizeof(unsigned)));
  if (!c->dsmcs) {
    c->dsmcs = new (std::nothrow) std::vector<Dsmc *>();
    if (!c->dsmcs) {
      dsmc_free(d);
      return ISKRA_ENOMEM;
    }
  }
  dsmc_of(c).push_back(d);
  invalidate_graphs(c);
  if (set) *set = (int)dsmc_of(c).size() - 1;
  return ISKRA_OK;
}

int iskra_dsmc_perform(iskra_ctx *h, int set, double dt, uint64_t seed, uint64_t step) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->dsmcs || set < 0 || set >= (int)dsmc_of(c).size()) return set_err(c, ISKRA_EINVAL, "bad DSMC set");
  if (!(dt > 0.0)) return set_err(c, ISKRA_EINVAL, "dt must be positive");
  return launch_dsmc(c, set, dt, seed, nullptr, step);  // velocities only: densities stay valid
}

int iskra_dsmc_state(iskra_ctx *h, int set, double *remaining, uint32_t *nu) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->dsmcs || set < 0 || set >= (int)dsmc_of(c).size()) return set_err(c, ISKRA_EINVAL, "bad DSMC set");
  Dsmc *d = dsmc_of(c)[set];
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (remaining)
    ISKRA_CUDA(c, cudaMemcpy(remaining, d->remaining, (size_t)c->nn * sizeof(double), cudaMemcpyDeviceToHost));
  if (nu) ISKRA_CUDA(c, cudaMemcpy(nu, d->nu, (size_t)c->nn * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  return collect_device_errors(c);
}

}  // extern "C"
