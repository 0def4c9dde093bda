// mcc.cu -- null-collision Monte Carlo collisions (Chemistry/src/mcc.jl).
//
// Reference algorithm (PIC.perform!, mcc.jl:231-289): per step draw
// Nc = floor(N*maxPt*np + remainder) particles uniformly WITH replacement; for
// each draw pick process k = floor(N*U)+1 with one uniform U, evaluate
// P_k = (1-exp(-n σ_k(ε) g Δt)) / (N*maxPt) and accept when U > k/N - P_k.
//
// Device algorithm: every live particle is selected c ~ Poisson(N*maxPt)
// times (the per-particle law of drawing Nc times with replacement, whose
// mean is N*maxPt per step including the carried remainder), and each
// selection runs the reference's k-choice, acceptance test and kinematics on
// that particle in order.  Randomness: the selection count from the
// SplitMix64 finalizer (Steele, Lea, Flood, OOPSLA 2014) of (set key, step,
// particle id); the draws of each selection from Philox4x32-10 (Salmon,
// Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11)
// keyed by (seed, set) with counter (particle id, step, draw), so the result
// does not depend on the particle order in memory.  Differences
// from the reference, both statistical only: particles created by ionisation
// in this step are not selected again in the same step (the reference re-reads
// np after each draw), and the number of draws per step is Poisson instead of
// the deterministic Nc.  Kinematics (mcc.jl:53-229) run in FP32 on the FP32
// particle velocities.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace iskra {

constexpr int kMaxProc = 8;
constexpr int kMaxTable = 8192;  // total table nodes of one set

struct MccDev {
  int N;
  int types[kMaxProc];
  float energy[kMaxProc];
  int off[kMaxProc + 1];
  const float *eps;      // table energies (eV)
  const float *sig;      // cross sections (m^2)
  const float *gas_n;    // (nx*ny) target density
  float m_ev;            // source mass in eV units (mcc.jl:26)
  float mr1, mr2;        // m_s/(m_s+m_t), m_t/(m_s+m_t)
  float vth_t;           // sqrt(2 kB T_t / m_t) (mcc.jl:74-77)
  float qmt_dt;          // (q_t/m_t) Δt for the target velocity term
  float lam;             // N*maxPt: mean selections per particle and step
  float inv_nmaxpt;      // 1/(N*maxPt)
  float dt;
  int mp;                // ions appended per ionisation (round(w0_s/w0_p))
  unsigned long long *counts;  // N
  unsigned int *nu;      // (nx*ny*N) accepted collisions per node and process
  uint32_t key0, key1;
  int logu[kMaxProc];    // table energies log-uniform: O(1) bracket guess
  float log_e0[kMaxProc], inv_dlog[kMaxProc];
  int staged;            // some table is not log-uniform: the collision pass stages the tables in shared memory
  float kthr[kMaxProc];  // (k + 1) / N in FP32: the first term of process k's acceptance threshold
};

struct Mcc {
  int src = -1, prod = -1;
  int N = 0;
  std::vector<int> types;
  std::vector<double> energies;
  std::vector<double> eps_h, sig_h;
  std::vector<int> off;
  double max_sigma_g = 0;
  double max_n = 0;
  double gas_mass = 0, gas_T = 0, gas_q = 0;
  float *eps = nullptr, *sig = nullptr, *gas_n = nullptr;
  unsigned long long *counts = nullptr;
  unsigned int *nu = nullptr;
  int set_index = 0;
  std::vector<int> logu;            // per process: energies on a log-uniform grid
  std::vector<float> log_e0, inv_dlog;
};

void mcc_destroy(Mcc *m) {
  if (!m) return;
  cudaFree(m->eps);
  cudaFree(m->sig);
  cudaFree(m->gas_n);
  cudaFree(m->counts);
  cudaFree(m->nu);
  delete m;
}

// ---- kinematics (mcc.jl:53-229) -------------------------------------------
// euler_angles (mcc.jl:89-106): cosθ = v_z/|v|, sinθ = sqrt(1 - cos²θ),
// cosϕ = v_x/|v|/sinθ, sinϕ = v_y/|v|/sinθ.  The same angles are formed here
// from the transverse speed ρ = sqrt(v_x² + v_y²) (sinθ = ρ/|v|, cosϕ = v_x/ρ),
// which keeps sin²+cos² = 1 to FP32 rounding when θ is small; sinθ = 0 takes
// the reference's sinθ ≈ 0 branch.
__device__ __forceinline__ void euler_angles(const float v[3], float &sth, float &cth, float &sph, float &cph) {
  const float rho = sqrtf(v[0] * v[0] + v[1] * v[1]);
  const float nv = sqrtf(rho * rho + v[2] * v[2]);
  if (!(nv > 0.0f)) {  // zero speed: unrotated frame (the reference yields NaN)
    sth = 0.0f;
    cth = 1.0f;
    sph = 0.0f;
    cph = 1.0f;
    return;
  }
  cth = v[2] / nv;
  sth = rho / nv;
  if (rho == 0.0f) {
    cph = 1.0f;
    sph = 0.0f;
  } else {
    cph = v[0] / rho;
    sph = v[1] / rho;
  }
}

// [sinχcosη sinχsinη cosχ] * unrotated(θ, ϕ)  (mcc.jl:83-87)
__device__ __forceinline__ void rotate(float sth, float cth, float sph, float cph, float sch, float cch, float seta,
                                       float ceta, float out[3]) {
  const float a0 = sch * ceta, a1 = sch * seta, a2 = cch;
  out[0] = a0 * (cph * cth) - a1 * sph + a2 * (cph * sth);
  out[1] = -a0 * (sph * cth) + a1 * cph + a2 * (sph * sth);
  out[2] = -a0 * sth + a2 * cth;
}

__device__ __forceinline__ void isotropic_scattering(const float v[3], float u1, float u2, float out[3]) {
  float sth, cth, sph, cph, sch, cch, seta, ceta;
  euler_angles(v, sth, cth, sph, cph);
  sincospif(2.0f * u1, &sch, &cch);  // χ = 2π u1 (mcc.jl:54)
  sincospif(2.0f * u2, &seta, &ceta);
  rotate(sth, cth, sph, cph, sch, cch, seta, ceta, out);
}

__device__ __forceinline__ void diffuse_reflection(const float v[3], float u1, float u2, float out[3]) {
  float sth, cth, sph, cph, seta, ceta;
  euler_angles(v, sth, cth, sph, cph);
  const float sch = sqrtf(u1);
  const float cch = -sqrtf(fmaxf(1.0f - sch * sch, 0.0f));
  sincospif(2.0f * u2, &seta, &ceta);
  rotate(sth, cth, sph, cph, sch, cch, seta, ceta, out);
}

// warp-aggregated slot reservation: every lane with want=true gets a slot
__device__ __forceinline__ long long warp_reserve(bool want, long long *np, unsigned int *next_id, uint32_t &nid) {
  const unsigned FULL = 0xffffffffu;
  const unsigned lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(FULL, want);
  long long base = 0;
  uint32_t idb = 0;
  const int leader = m ? __ffs(m) - 1 : 0;
  if (m && lane == (unsigned)leader) {
    base = atomicAdd((unsigned long long *)np, (unsigned long long)__popc(m));
    idb = atomicAdd(next_id, (unsigned)__popc(m));
  }
  base = __shfl_sync(FULL, base, leader);
  idb = __shfl_sync(FULL, idb, leader);
  const int rank = __popc(m & ((1u << lane) - 1u));
  nid = idb + rank;
  return base + rank;
}

// ---- two-phase null-collision step --------------------------------------
// Phase 1 (k_mcc_select, every live particle; in ensembles the push of the
// step before, k_push_runs): the particle's hash uniform gives its number of
// selections c ~ Poisson(N maxPt); particles with c > 0 go to a work list
// as their whole record (MccWork: position, velocity, cell, id, slot).
// Phase 2 (k_mcc_collide, the work list only): each entry replays its
// particle's count (the hash gives c again) and runs the c selections
// -- the k choice, acceptance test and kinematics -- in order, then writes
// the changed velocity back to the particle's slot.  With N maxPt ~ 0.1 a
// warp of phase 2 holds 32 colliding particles instead of the ~3 a single
// pass over all particles would, and it reads them as one contiguous
// 32-byte entry each instead of three scattered records.
constexpr int kSelChunk = 1024;  // particles per block pass of k_mcc_select
// words of hit bits per run (one bit per work-list entry), after the entries
__host__ __device__ __forceinline__ size_t hit_words(size_t cap) { return (cap + 31) / 32; }

// Phase 1 over the particles of run blockIdx.y (R = 1 for a single context):
// a block collects the selected particles of a chunk in shared memory and
// appends them to its run's segment [r cap_run, ...) of the work list with
// one atomic on the run's counter nwork[r kNworkStride].  step_ahead = 1 draws for the
// step after the device counter's (a list built before the step begins).
__global__ void __launch_bounds__(256) k_mcc_select(const SpeciesDev *__restrict__ src, float lam, uint2 key1,
                                                    const uint2 *__restrict__ keys,
                                                    const unsigned long long *__restrict__ d_step, int step_ahead,
                                                    MccWork *__restrict__ work, unsigned long long *__restrict__ nwork,
                                                    unsigned long long cap_run, int *err) {
  pdl_wait();
  __shared__ MccWork buf[kSelChunk];
  __shared__ unsigned cnt;
  __shared__ unsigned long long base;
  const unsigned FULL = 0xffffffffu;
  const int r = blockIdx.y;
  const SpeciesDev s = src[r];
  const uint2 key = keys ? keys[r] : key1;
  const int lane = threadIdx.x & 31;
  const long long np = s.st->np;
  const int cur = s.st->cur;
  const float4 *__restrict__ xv = pick(s.xv[0], s.xv[1], cur);
  const float2 *__restrict__ zc = pick(s.zc[0], s.zc[1], cur);
  const uint32_t *__restrict__ ids = pick(s.id[0], s.id[1], cur);
  const unsigned long long step = *d_step + (unsigned long long)step_ahead;
  const float expl = __expf(-lam);
  MccWork *__restrict__ seg = work + (size_t)r * cap_run;
  int flags = 0;
  for (long long c0 = (long long)blockIdx.x * kSelChunk; c0 < np; c0 += (long long)gridDim.x * kSelChunk) {
    if (threadIdx.x == 0) cnt = 0u;
    __syncthreads();
    for (int i = threadIdx.x; i < kSelChunk; i += blockDim.x) {
      const long long p = c0 + i;
      int nsel = 0;
      float2 b = make_float2(0.f, 0.f);
      uint32_t pid = 0;
      if (p < np) {
        b = zc[p];
        if (__float_as_int(b.y) >= 0) {
          pid = ids[p];
          nsel = draw_selections(selection_uniform(pid, step, key), lam, expl);
        }
      }
      const unsigned m = __ballot_sync(FULL, nsel > 0);
      if (!m) continue;
      const int leader = __ffs(m) - 1;
      unsigned at = 0;
      if (lane == leader) at = atomicAdd(&cnt, (unsigned)__popc(m));
      at = __shfl_sync(FULL, at, leader) + __popc(m & ((1u << lane) - 1u));
      if (nsel > 0) buf[at] = mcc_entry(xv[p], b, pid, (uint32_t)p);
    }
    __syncthreads();
    if (threadIdx.x == 0) base = atomicAdd(nwork + (size_t)r * kNworkStride, (unsigned long long)cnt);
    __syncthreads();
    for (unsigned i = threadIdx.x; i < cnt; i += blockDim.x) {
      const unsigned long long at = base + i;
      if (at < cap_run) seg[at] = buf[i];
      else flags |= DERR_CAPACITY;
    }
    __syncthreads();
  }
  const int f = __reduce_or_sync(FULL, flags);
  if (lane == 0 && f) atomicOr(err, f);
}

// Whether a work entry collides in this step: its selections replayed in
// order up to the first accepted one (a rejected selection changes nothing,
// so these are exactly the tests the collision code makes before its first
// collision); a probability above the bound counts as a hit (the collision
// code raises the flag).
__device__ __forceinline__ bool mcc_entry_hits(const MccWork &e, const MccDev &M, const float *te, const float *ts,
                                               const float2 *__restrict__ Er, int nx, unsigned long long step,
                                               uint2 key, float expl) {
  const int nsel = draw_selections(selection_uniform(e.b.z, step, key), M.lam, expl);
  if (nsel == 0) return false;
  Stream R = particle_stream(e.b.z, step, key);
  const int cell = (int)e.b.y;
  const int node = (cell & 0xffff) + nx * (cell >> 16);
  const float n = __ldg(M.gas_n + node);
  const float2 ef = __ldg(Er + node);
  const float gx = M.qmt_dt * ef.x - e.a.z, gy = M.qmt_dt * ef.y - e.a.w, gz = -__uint_as_float(e.b.x);
  const float g = sqrtf(gx * gx + gy * gy + gz * gz);
  const float eps = 0.5f * M.m_ev * g * g;
  for (int sidx = 0; sidx < nsel && n >= 0.0f; sidx++) {
    const float U = R.next();
    int k = (int)floorf(M.N * U);
    if (k >= M.N) k = M.N - 1;
    const float sg = sigma_at(te + M.off[k], ts + M.off[k], M.off[k + 1] - M.off[k], eps, M.logu[k],
                              M.log_e0[k], M.inv_dlog[k]) *
                     g;
    float Pk = -expm1f(-n * sg * M.dt);
    Pk *= M.inv_nmaxpt;
    if (Pk > 1.0f) return true;
    if (U > M.kthr[k] - Pk) return true;
  }
  return false;
}

// Phase 2 over the work list segment of run r = blockIdx.y: the run's stores
// src[r] / prod[r], node field E + r nn, key keys[r] (or M's key for a single
// context), counters counts_runs + r N (or M.counts).
// Blocks of 256 threads per SM asked of the register allocator for the
// collision kernel: 3 (80 registers) against 2 (102 registers) -- measured
// when the kernel also tested every entry: 245 against 283 us per electron
// pass of a 128-run ensemble.
#ifndef ISKRA_MCC_COLLIDE_MIN_BLOCKS
#define ISKRA_MCC_COLLIDE_MIN_BLOCKS 3
#endif
// Ensembles: collision-kernel blocks per run = the push's blocks per run /
// this.  A block's setup (run views, step, key) is a chain of dependent
// loads: with the testing still in this kernel, 2 gave 218 against 241 us
// per electron pass of a 128-run ensemble (4: 252, 8: 389, the largest runs'
// blocks then set the pass's length); after the split, 4 and 8 gave no gain.
#ifndef ISKRA_MCC_COLLIDE_SPLIT
#define ISKRA_MCC_COLLIDE_SPLIT 2
#endif
// Launch shape of k_mcc_test (electron pass of a 128-run ensemble, ncu):
// test blocks per run = the push's x SCALE8 / 8 -- 2x: 99 us, 1x: 106, 4x:
// 98, 0.5x: 132; UNROLL 2 (two words per warp and round): no change.
#ifndef ISKRA_MCC_TEST_UNROLL
#define ISKRA_MCC_TEST_UNROLL 1
#endif
#ifndef ISKRA_MCC_TEST_SCALE8
#define ISKRA_MCC_TEST_SCALE8 16
#endif
// Phase 2a over the work-list segment of run r = blockIdx.y: each warp
// tests 32 entries (mcc_entry_hits) and stores their hit bits, one word per
// 32 entries.  Apart from the collision code, the test needs few registers,
// so twice as many warps per SM hide its dependent loads (the entry, its
// node's gas density and field, the table bracket).
__global__ void __launch_bounds__(256) k_mcc_test(MccDev M, const uint2 *__restrict__ keys,
                                                  const float2 *__restrict__ E, int nn, int nx,
                                                  const unsigned long long *__restrict__ d_step,
                                                  const MccWork *__restrict__ work,
                                                  const unsigned long long *__restrict__ nwork,
                                                  unsigned long long cap_run, unsigned *__restrict__ hits) {
  pdl_wait();
  extern __shared__ float tab[];
  const float *te = M.eps, *ts = M.sig;
  if (M.staged) {
    const int ntab = M.off[M.N];
    for (int t = threadIdx.x; t < ntab; t += blockDim.x) {
      tab[t] = M.eps[t];
      tab[ntab + t] = M.sig[t];
    }
    __syncthreads();
    te = tab;
    ts = tab + ntab;
  }
  const unsigned long long step = *d_step;
  const int r = blockIdx.y;
  const long long nw = (long long)min(nwork[(size_t)r * kNworkStride], cap_run);
  const MccWork *__restrict__ seg = work + (size_t)r * cap_run;
  unsigned *__restrict__ hw = hits + (size_t)r * hit_words(cap_run);
  const float2 *Er = E + (size_t)r * nn;
  const uint2 key = keys ? keys[r] : make_uint2(M.key0, M.key1);
  const float expl = __expf(-M.lam);
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  constexpr int U = ISKRA_MCC_TEST_UNROLL;  // words of 32 entries per warp and round
  for (long long base = warp * 32 * U; base < nw; base += nwarps * 32 * U) {
    bool hit[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const long long wt = base + 32 * u + lane;
      hit[u] = wt < nw && mcc_entry_hits(seg[wt], M, te, ts, Er, nx, step, key, expl);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const unsigned hm = __ballot_sync(0xffffffffu, hit[u]);
      if (lane == 0 && base + 32 * u < nw) hw[(base >> 5) + u] = hm;
    }
  }
}

__global__ void __launch_bounds__(256, ISKRA_MCC_COLLIDE_MIN_BLOCKS) k_mcc_collide(const SpeciesDev *__restrict__ src,
                                                     const SpeciesDev *__restrict__ prod, int has_prod, MccDev M,
                                                     const uint2 *__restrict__ keys, unsigned long long *counts_runs,
                                                     const float2 *__restrict__ E, int nn, int nx,
                                                     const unsigned long long *__restrict__ d_step,
                                                     const MccWork *__restrict__ work,
                                                     const unsigned long long *__restrict__ nwork,
                                                     unsigned long long cap_run,
                                                     const unsigned *__restrict__ hits, int *err) {
  pdl_wait();
  extern __shared__ float tab[];
  const unsigned FULL = 0xffffffffu;
  // log-uniform tables take O(1) lookups, read through the caches; others
  // (binary search) are staged in shared memory
  const float *te = M.eps, *ts = M.sig;
  if (M.staged) {
    const int ntab = M.off[M.N];
    for (int t = threadIdx.x; t < ntab; t += blockDim.x) {
      tab[t] = M.eps[t];
      tab[ntab + t] = M.sig[t];
    }
    __syncthreads();
    te = tab;
    ts = tab + ntab;
  }
  const unsigned long long step = *d_step;
  const int r = blockIdx.y;
  const long long nw = (long long)min(nwork[(size_t)r * kNworkStride], cap_run);
  const MccWork *__restrict__ seg = work + (size_t)r * cap_run;
  const float expl = __expf(-M.lam);
  int flags = 0;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  const SpeciesDev s = src[r];
  const int cur = s.st->cur;
  float4 *__restrict__ xv = pick(s.xv[0], s.xv[1], cur);
  float2 *__restrict__ zc = pick(s.zc[0], s.zc[1], cur);
  unsigned long long *cnts = keys ? counts_runs + (size_t)r * M.N : M.counts;
  const float2 *Er = E + (size_t)r * nn;
  unsigned acc_k[kMaxProc];
#pragma unroll
  for (int k = 0; k < kMaxProc; k++) acc_k[k] = 0u;
  // Each warp reads the hit bits of 32 entries at a time (k_mcc_test) and
  // queues the ~5 % that collide in its own shared-memory queue; whenever 32 are queued
  // (and for the rest at the end) it runs the collision code on them densely,
  // instead of diverging into the kinematics for its one or two colliding
  // lanes of every 32.  Warps never wait for one another.
  __shared__ unsigned wq[8][64];
  const uint2 key = keys ? keys[r] : make_uint2(M.key0, M.key1);
  unsigned *q = wq[threadIdx.x >> 5];
  int qn = 0;  // queued entries (warp-uniform)
  const unsigned *__restrict__ hw = hits + (size_t)r * hit_words(cap_run);
  for (long long base = warp * 32;; base += nwarps * 32) {
    const bool more = base < nw;  // warp-uniform
    if (more) {
      const long long wt = base + lane;
      const unsigned hm = hw[base >> 5];  // bits past nw are zero
      const bool hit = (hm >> lane) & 1u;
      if (hit) q[qn + __popc(hm & ((1u << lane) - 1u))] = (unsigned)wt;
      qn += __popc(hm);
      __syncwarp();
    }
    if (qn < 32 && (more || qn == 0)) {
      if (more) continue;
      break;
    }
    const int take = qn < 32 ? qn : 32;
    const bool act = lane < take;
    const long long w = act ? (long long)q[lane] : 0;
    __syncwarp();
    if (lane < qn - take) q[lane] = q[take + lane];  // the rest moves to the front (at most 31)
    __syncwarp();
    qn -= take;
    {
    int nsel = 0;
    long long p = 0;
    MccWork e{};
    if (act) {
      e = seg[w];
      p = e.b.w;
    }
    bool ion_child = false;
    float cv[3] = {0, 0, 0};
    float tv_ion[3] = {0, 0, 0};
    float v[3] = {0, 0, 0};
    float4 a = make_float4(0, 0, 0, 0);
    float2 b = make_float2(0, 0);
    int cell = -1;
    if (act) {
      a = e.a;
      b = make_float2(__uint_as_float(e.b.x), __uint_as_float(e.b.y));
      cell = (int)e.b.y;
      const uint32_t pid = e.b.z;
      Stream R = particle_stream(pid, step, key);
      nsel = draw_selections(selection_uniform(pid, step, key), M.lam, expl);  // the phase-1 draw again: its count
      v[0] = a.z;
      v[1] = a.w;
      v[2] = b.x;
      const int i0 = cell & 0xffff, j0 = cell >> 16;
      const int node = i0 + nx * j0;
      const float n = __ldg(M.gas_n + node);
      const float2 e = __ldg(Er + node);
      const float tvx = M.qmt_dt * e.x, tvy = M.qmt_dt * e.y;
      bool changed = false;
      for (int sidx = 0; sidx < nsel && n >= 0.0f; sidx++) {
        const float U = R.next();
        int k = (int)floorf(M.N * U);
        if (k >= M.N) k = M.N - 1;
        const float gx = tvx - v[0], gy = tvy - v[1], gz = -v[2];
        const float g = sqrtf(gx * gx + gy * gy + gz * gz);
        const float eps = 0.5f * M.m_ev * g * g;
        const float sg = sigma_at(te + M.off[k], ts + M.off[k], M.off[k + 1] - M.off[k], eps, M.logu[k],
                                  M.log_e0[k], M.inv_dlog[k]) *
                         g;
        float Pk = -expm1f(-n * sg * M.dt);
        Pk *= M.inv_nmaxpt;
        if (Pk > 1.0f) {
          flags |= DERR_PROB;
          break;
        }
        if (!(U > M.kthr[k] - Pk)) continue;
        acc_k[k]++;
        if (M.nu && !keys) atomicAdd(M.nu + (size_t)node * M.N + k, 1u);
        const int type = M.types[k];
        if (type <= ISKRA_MCC_INELASTIC_BACKWARD) {
          float tv[3];
          R.normal3(tv, M.vth_t);
          float vr[3], wv[3], dir[3];
          for (int c = 0; c < 3; c++) {
            vr[c] = v[c] - tv[c];
            wv[c] = M.mr1 * v[c] + M.mr2 * tv[c];
          }
          const float nvr = sqrtf(vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]);
          float scale = nvr;
          if (type == ISKRA_MCC_INELASTIC_BACKWARD) scale = R.next() * nvr;
          const float u1 = R.next(), u2 = R.next();
          if (type == ISKRA_MCC_ELASTIC_ISOTROPIC) isotropic_scattering(vr, u1, u2, dir);
          else diffuse_reflection(vr, u1, u2, dir);
          for (int c = 0; c < 3; c++) v[c] = wv[c] + M.mr2 * (scale * dir[c]);
          changed = true;
          continue;
        }
        const float sE = 0.5f * M.m_ev * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) - M.energy[k];
        if (sE < 0.0f) continue;  // not enough energy (mcc.jl:179-182,220-223)
        const float al = sqrtf(2.0f / M.m_ev);
        if (type == ISKRA_MCC_EXCITATION) {
          const float ev = al * sqrtf(sE);
          float dir[3];
          const float u1 = R.next(), u2 = R.next();
          isotropic_scattering(v, u1, u2, dir);
          for (int c = 0; c < 3; c++) v[c] = ev * dir[c];
          changed = true;
          continue;
        }
        // ionisation (mcc.jl:174-213); one child electron per particle and step
        const float e1 = sE * R.next(), e2 = sE - e1;
        const float v1 = al * sqrtf(e1), v2 = al * sqrtf(e2);
        float dir[3];
        float u1 = R.next(), u2 = R.next();
        diffuse_reflection(v, u1, u2, dir);
        for (int c = 0; c < 3; c++) v[c] = v1 * dir[c];
        changed = true;
        if (!ion_child) {
          u1 = R.next();
          u2 = R.next();
          diffuse_reflection(v, u1, u2, dir);
          for (int c = 0; c < 3; c++) cv[c] = v2 * dir[c];
          R.normal3(tv_ion, M.vth_t);
          ion_child = true;
        }
      }
      if (changed) {
        if (!isfinite(v[0]) || !isfinite(v[1]) || !isfinite(v[2])) flags |= DERR_NAN;
        xv[p] = make_float4(a.x, a.y, v[0], v[1]);
        zc[p] = make_float2(v[2], b.y);
      }
    }
    // appends: child electron into the source species, ions into the product
    if (__any_sync(FULL, ion_child)) {
      uint32_t nid;
      const long long slot = warp_reserve(ion_child, &s.st->np_new, &s.st->next_id, nid);
      if (ion_child) {
        if (slot < s.cap) {
          xv[slot] = make_float4(a.x, a.y, cv[0], cv[1]);
          zc[slot] = make_float2(cv[2], __int_as_float(cell));
          pick(s.id[0], s.id[1], cur)[slot] = nid;
        } else {
          flags |= DERR_CAPACITY;
        }
      }
      if (has_prod) {
        const SpeciesDev pd = prod[r];
        const int pb = pd.st->cur;
        for (int m = 0; m < M.mp; m++) {
          uint32_t pid2;
          const long long ps = warp_reserve(ion_child, &pd.st->np_new, &pd.st->next_id, pid2);
          if (ion_child) {
            if (ps < pd.cap) {
              pick(pd.xv[0], pd.xv[1], pb)[ps] = make_float4(a.x, a.y, tv_ion[0], tv_ion[1]);
              pick(pd.zc[0], pd.zc[1], pb)[ps] = make_float2(tv_ion[2], __int_as_float(cell));
              pick(pd.id[0], pd.id[1], pb)[ps] = pid2;
            } else {
              flags |= DERR_CAPACITY;
            }
          }
        }
      }
    }
    }
    if (!more && qn == 0) break;
    if (!more) base -= nwarps * 32;  // more queued entries: another group without new tests
  }
#pragma unroll
  for (int k = 0; k < kMaxProc; k++) {
    if (k >= M.N) break;
    const unsigned t = __reduce_add_sync(FULL, acc_k[k]);
    if (lane == 0 && t) atomicAdd(cnts + k, (unsigned long long)t);
  }
  const int f = __reduce_or_sync(FULL, flags);
  if (lane == 0 && f) atomicOr(err, f);
}

__global__ void k_zero_u64(unsigned long long *p, int n, int stride) {
  pdl_wait();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[(size_t)i * stride] = 0ull;
}

// Appends reserve slots from np_new so that np (the loop bound of the running
// kernel) stays fixed during the launch; np takes the new extent afterwards,
// clamped to the capacity (failed appends already raised DERR_CAPACITY).
__global__ void k_append_begin(SpeciesState *a, SpeciesState *b) {
  pdl_wait();
  a->np_new = a->np;
  if (b) b->np_new = b->np;
}
__global__ void k_append_end(SpeciesState *st, long long cap) {
  pdl_wait();
  st->np = st->np_new > cap ? cap : st->np_new;
}

// Philox key of (seed, set)
void mcc_key(uint64_t seed, int set_index, uint32_t &k0, uint32_t &k1) {
  k0 = (uint32_t)seed;
  k1 = (uint32_t)(seed >> 32) ^ (0x632BE5ABu * (uint32_t)(set_index + 1));
}

// Kernel parameters of MCC set mid for time step dt (keys from seed).
static int mcc_params(Ctx *c, int mid, double dt, uint64_t seed, MccDev &M) {
  Mcc *m = c->mccs[mid];
  Species &s = c->species[m->src];
  const double maxPt = 1.0 - std::exp(-m->max_n * m->max_sigma_g * dt);
  if (maxPt > 1.0 / m->N)
    return set_err(c, ISKRA_EPROB, "maximum collision probability above 1/N (mcc.jl:244-246)");
  M = MccDev{};
  M.N = m->N;
  for (int k = 0; k < m->N; k++) {
    M.types[k] = m->types[k];
    M.energy[k] = (float)m->energies[k];
  }
  for (int k = 0; k <= m->N; k++) M.off[k] = m->off[k];
  M.eps = m->eps;
  M.sig = m->sig;
  M.gas_n = m->gas_n;
  const double m_ev = s.m / 1.60217646e-19;
  M.m_ev = (float)m_ev;
  M.mr1 = (float)(s.m / (s.m + m->gas_mass));
  M.mr2 = (float)(m->gas_mass / (s.m + m->gas_mass));
  M.vth_t = (float)std::sqrt(2 * 1.3806503e-23 * m->gas_T / m->gas_mass);
  M.qmt_dt = (float)(m->gas_q / m->gas_mass * dt);
  M.lam = (float)(m->N * maxPt);
  M.inv_nmaxpt = maxPt > 0 ? (float)(1.0 / (m->N * maxPt)) : 0.0f;
  M.dt = (float)dt;
  M.mp = 0;
  if (m->prod >= 0) M.mp = (int)std::llround(s.w0 / c->species[m->prod].w0);
  M.counts = m->counts;
  M.nu = m->nu;
  mcc_key(seed, m->set_index, M.key0, M.key1);
  M.staged = 0;
  for (int k = 0; k < m->N; k++) {
    M.kthr[k] = (float)(k + 1) / (float)m->N;  // IEEE division: the bits the device's division gave
    M.logu[k] = m->logu[k];
    M.log_e0[k] = m->log_e0[k];
    M.inv_dlog[k] = m->inv_dlog[k];
    if (!m->logu[k]) M.staged = 1;
  }
  return ISKRA_OK;
}

// Both phases for R runs: src/prod device views (R each), keys (R, or
// nullptr with key1 for a single context), per-run counters, node fields E
// (R x nn), work list of cap_work entries with its counter.
static int queue_mcc_phases(Ctx *c, int mid, const MccDev &M, int R, const SpeciesDev *src, const SpeciesDev *prod,
                            const uint2 *keys, unsigned long long *counts, const float2 *E, int nn, int select_blocks,
                            MccWork *work, unsigned long long *nwork, unsigned long long cap_work,
                            const unsigned long long *d_step, int *err, cudaStream_t st, int phases = kMccBoth) {
  Mcc *m = c->mccs[mid];
  const int ntab = m->off[m->N];
  const size_t smem = M.staged ? (size_t)2 * ntab * sizeof(float) : 0;
  if (smem > 48 * 1024) {  // tables of up to kMaxTable nodes
    ISKRA_CUDA(c, cudaFuncSetAttribute(k_mcc_test, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ISKRA_CUDA(c, cudaFuncSetAttribute(k_mcc_collide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const uint2 key1 = make_uint2(M.key0, M.key1);
  if (phases != kMccCollideOnly) {
    ISKRA_CUDA(c, launch_pdl(k_zero_u64, (R + 255) / 256, 256, 0, st, nwork, R, kNworkStride));
    ISKRA_CUDA(c, launch_pdl(k_mcc_select, dim3(select_blocks, R), 256, 0, st, src, M.lam, key1, keys, d_step,
                             phases == kMccSelectAhead ? 1 : 0, work, nwork, cap_work, err));
  }
  if (phases == kMccSelectAhead) return ISKRA_OK;
  unsigned *hits = reinterpret_cast<unsigned *>(work + (size_t)R * cap_work);
  ISKRA_CUDA(c, launch_pdl(k_mcc_test, dim3(R == 1 ? c->num_sms * 8 : std::max(1, select_blocks * ISKRA_MCC_TEST_SCALE8 / 8), R), 256, smem, st, M, keys,
                           E, nn, c->nx, d_step, (const MccWork *)work, (const unsigned long long *)nwork, cap_work,
                           hits));
  const int collide_blocks = R == 1 ? c->num_sms * 8 : std::max(1, select_blocks / ISKRA_MCC_COLLIDE_SPLIT);
  ISKRA_CUDA(c, launch_pdl(k_mcc_collide, dim3(collide_blocks, R), 256, smem, st, src, prod, (int)(m->prod >= 0), M,
                           keys, counts, E, nn, c->nx, d_step, (const MccWork *)work, (const unsigned long long *)nwork,
                           cap_work, (const unsigned *)hits, err));
  return ISKRA_OK;
}

int launch_mcc(Ctx *c, int mid, double dt, uint64_t seed, const unsigned long long *d_step, uint64_t step_host) {
  (void)step_host;
  Mcc *m = c->mccs[mid];
  Species &s = c->species[m->src];
  MccDev M;
  int rc = mcc_params(c, mid, dt, seed, M);
  if (rc) return rc;
  if (!c->mcc_work) return set_err(c, ISKRA_EINVAL, "MCC work list missing");
  long long want = (s.cap + kSelChunk - 1) / kSelChunk;
  long long maxb = (long long)c->num_sms * 4;
  int blocks = (int)(want < maxb ? (want < 1 ? 1 : want) : maxb);
  const SpeciesDev *pd = m->prod >= 0 ? c->species[m->prod].dview : s.dview;
  SpeciesState *pst = m->prod >= 0 ? c->species[m->prod].dev.st : nullptr;
  ISKRA_CUDA(c, launch_pdl(k_append_begin, 1, 1, 0, c->stream, s.dev.st, pst));
  rc = queue_mcc_phases(c, mid, M, 1, s.dview, pd, nullptr, nullptr, c->E32, c->nn, blocks, (MccWork *)c->mcc_work,
                        c->mcc_nwork, c->mcc_work_cap, d_step, c->d_err, c->stream);
  if (rc) return rc;
  ISKRA_CUDA(c, launch_pdl(k_append_end, 1, 1, 0, c->stream, s.dev.st, s.cap));
  if (m->prod >= 0)
    ISKRA_CUDA(c, launch_pdl(k_append_end, 1, 1, 0, c->stream, c->species[m->prod].dev.st, c->species[m->prod].cap));
  ISKRA_CUDA(c, cudaGetLastError());
  // appended particles are not in the deposit accumulators
  for (int sid : {m->src, m->prod}) {
    if (sid < 0) continue;
    Species &sp = c->species[sid];
    if (sp.acc_valid) sp.acc_zero = false;
    sp.acc_valid = false;
    sp.n_valid = false;
  }
  return ISKRA_OK;
}

// Ensemble launch of MCC set mid of the template context over R runs:
// per-run stores (src/prod views), keys (2 words per run), counters (R x N)
// and node fields (R x nn); work list of cap_work entries.
int launch_mcc_runs(Ctx *c, int mid, double dt, int R, const SpeciesDev *src, const SpeciesDev *prod,
                    const uint2 *keys, unsigned long long *counts, const float2 *E32, int nn, int blocks_per_run,
                    void *work, unsigned long long *nwork, unsigned long long cap_work,
                    const unsigned long long *d_step, int *err, cudaStream_t st, int phases) {
  MccDev M;
  int rc = mcc_params(c, mid, dt, 0, M);
  if (rc) return rc;
  return queue_mcc_phases(c, mid, M, R, src, prod, keys, counts, E32, nn, blocks_per_run, (MccWork *)work, nwork,
                          cap_work, d_step, err, st, phases);
}

// The selection draw of MCC set mid for time step dt, for a push that makes
// the set's next work list (keys, list and counters are the caller's).
int mcc_push_select(Ctx *c, int mid, double dt, PushSelect *S) {
  MccDev M;
  int rc = mcc_params(c, mid, dt, 0, M);
  if (rc) return rc;
  S->lam = M.lam;
  return ISKRA_OK;
}

size_t mcc_work_bytes(size_t R, size_t cap) { return R * cap * sizeof(MccWork) + R * hit_words(cap) * sizeof(unsigned); }

// Work list sized for the largest species; called where no stream capture can
// be active (MCC set and species creation).
int ensure_mcc_work(Ctx *c) {
  if (c->mccs.empty()) return ISKRA_OK;
  long long cap = 1;
  for (auto &sp : c->species) cap = std::max(cap, sp.cap);
  if (c->mcc_work && c->mcc_work_cap >= (unsigned long long)cap) return ISKRA_OK;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  cudaFree(c->mcc_work);
  c->mcc_work = nullptr;
  c->mcc_work_cap = 0;
  ISKRA_CUDA(c, cudaMalloc(&c->mcc_work, mcc_work_bytes(1, (size_t)cap)));
  if (!c->mcc_nwork) ISKRA_CUDA(c, cudaMalloc(&c->mcc_nwork, sizeof(unsigned long long)));
  c->mcc_work_cap = (unsigned long long)cap;
  return ISKRA_OK;
}

// CrossSection lookups exactly as the MCC kernels make them (FP32 table,
// sigma_at with the set's log-uniform bracket guess), for a list of energies.
__global__ void k_mcc_sigma(const float *__restrict__ e, const float *__restrict__ s, int n, int logu, float le0,
                            float idl, const double *__restrict__ x, long long m, double *__restrict__ out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
    out[k] = (double)sigma_at(e, s, n, (float)x[k], logu, le0, idl);
}

// Accepted collisions per node and process since the previous call (the
// "nuMCC" record of perform!, mcc.jl:234,283,287, which counts one step):
// out[node N + k]; the device counters restart from zero.  Synchronous.
int mcc_download_nu(Ctx *c, int mid, unsigned *out) {
  Mcc *m = c->mccs[mid];
  const size_t bytes = (size_t)c->nn * m->N * sizeof(unsigned);
  ISKRA_CUDA(c, cudaMemcpyAsync(out, m->nu, bytes, cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(m->nu, 0, bytes, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  return ISKRA_OK;
}

int mcc_nproc(Ctx *c, int mid) { return c->mccs[mid]->N; }
int mcc_src(Ctx *c, int mid) { return c->mccs[mid]->src; }
int mcc_prod(Ctx *c, int mid) { return c->mccs[mid]->prod; }
int mcc_set_index(Ctx *c, int mid) { return c->mccs[mid]->set_index; }

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_mcc_create(iskra_ctx *h, int src, int nproc, const int *types, const double *energies, const int32_t *off,
                     const double *eps, const double *sigma, double gas_mass, double gas_T, double gas_q,
                     const double *gas_n, int prod, double *max_sigma_g, int *mid) {
  if (!h || !types || !energies || !off || !eps || !sigma || !gas_n || !mid) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (src < 0 || src >= (int)c->species.size()) return set_err(c, ISKRA_EINVAL, "bad source species");
  if (prod >= (int)c->species.size()) return set_err(c, ISKRA_EINVAL, "bad product species");
  if (nproc < 1 || nproc > kMaxProc) return set_err(c, ISKRA_EINVAL, "1..8 processes per set");
  if ((int)c->mccs.size() >= kMaxMcc) return set_err(c, ISKRA_EINVAL, "too many MCC sets");
  if (!(gas_mass > 0) || !(gas_T >= 0)) return set_err(c, ISKRA_EINVAL, "bad gas mass / temperature");
  if (off[0] != 0 || off[nproc] > kMaxTable) return set_err(c, ISKRA_EINVAL, "bad table offsets");
  for (int k = 0; k < nproc; k++) {
    if (types[k] < 0 || types[k] > 4) return set_err(c, ISKRA_EINVAL, "bad process type");
    if (off[k + 1] - off[k] < 1) return set_err(c, ISKRA_EINVAL, "empty cross-section table");
    for (int t = off[k] + 1; t < off[k + 1]; t++)
      if (!(eps[t] > eps[t - 1])) return set_err(c, ISKRA_EINVAL, "table energies must increase");
  }
  Mcc *m = new Mcc();
  m->src = src;
  m->prod = prod;
  m->N = nproc;
  m->types.assign(types, types + nproc);
  m->energies.assign(energies, energies + nproc);
  m->off.assign(off, off + nproc + 1);
  m->eps_h.assign(eps, eps + off[nproc]);
  m->sig_h.assign(sigma, sigma + off[nproc]);
  m->gas_mass = gas_mass;
  m->gas_T = gas_T;
  m->gas_q = gas_q;
  m->set_index = (int)c->mccs.size();
  // tables on a log-uniform energy grid get an O(1) bracket guess
  m->logu.assign(nproc, 0);
  m->log_e0.assign(nproc, 0.f);
  m->inv_dlog.assign(nproc, 0.f);
  for (int k = 0; k < nproc; k++) {
    const double *E = eps + off[k];
    const int n = off[k + 1] - off[k];
    if (n < 3 || !(E[0] > 0)) continue;
    const double d = std::log(E[n - 1] / E[0]) / (n - 1);
    bool uni = d > 0;
    for (int t = 1; t < n && uni; t++) uni = std::fabs(std::log(E[t] / E[t - 1]) - d) <= 1e-6 * d;
    if (!uni) continue;
    m->logu[k] = 1;
    m->log_e0[k] = (float)std::log((double)(float)E[0]);
    m->inv_dlog[k] = (float)(1.0 / d);
  }
  // MonteCarloCollisions constructor (mcc.jl:27-51): max over the union of
  // table energies (plus 0) of Σ_k σ_k(ε) v(ε), v = sqrt(2ε/m_eV)
  std::vector<double> e = {0.0};
  e.insert(e.end(), eps, eps + off[nproc]);
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  const double ms = c->species[src].m / 1.60217646e-19;
  const double alpha = std::sqrt(2.0 / ms);
  double best = 0;
  for (size_t a = 0; a < e.size(); a++) {
    const double v = alpha * std::sqrt(e[a]);
    double s = 0;
    for (int k = 0; k < nproc; k++) {
      const double *E = eps + off[k], *S = sigma + off[k];
      const int n = off[k + 1] - off[k];
      double sg;
      if (e[a] <= E[0]) sg = S[0];
      else if (e[a] >= E[n - 1]) sg = S[n - 1];
      else {
        int lo = 0, hi = n - 1;
        while (hi - lo > 1) {
          int mid2 = (lo + hi) >> 1;
          if (E[mid2] <= e[a]) lo = mid2; else hi = mid2;
        }
        const double t = (e[a] - E[lo]) / (E[hi] - E[lo]);
        sg = (1.0 - t) * S[lo] + t * S[hi];
      }
      s += sg * v;
    }
    if (a == 0 || s > best) best = s;
  }
  m->max_sigma_g = best;
  double mx = gas_n[0];
  for (int k = 1; k < c->nn; k++) mx = gas_n[k] > mx ? gas_n[k] : mx;
  m->max_n = mx;
  std::vector<float> ef(eps, eps + off[nproc]), sf(sigma, sigma + off[nproc]), nf(gas_n, gas_n + c->nn);
  bool ok = cudaMalloc(&m->eps, ef.size() * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->sig, sf.size() * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->gas_n, nf.size() * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->counts, kMaxProc * sizeof(unsigned long long)) == cudaSuccess &&
            cudaMalloc(&m->nu, (size_t)c->nn * nproc * sizeof(unsigned int)) == cudaSuccess;
  if (!ok) {
    mcc_destroy(m);
    return set_err(c, ISKRA_ENOMEM, "MCC tables");
  }
  cudaMemcpy(m->eps, ef.data(), ef.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(m->sig, sf.data(), sf.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(m->gas_n, nf.data(), nf.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(m->counts, 0, kMaxProc * sizeof(unsigned long long));
  cudaMemset(m->nu, 0, (size_t)c->nn * nproc * sizeof(unsigned int));
  c->mccs.push_back(m);
  *mid = (int)c->mccs.size() - 1;
  if (max_sigma_g) *max_sigma_g = best;
  invalidate_graphs(c);
  return ensure_mcc_work(c);
}

int iskra_mcc_perform(iskra_ctx *h, int mid, double dt, uint64_t seed, uint64_t step) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (mid < 0 || mid >= (int)c->mccs.size()) return set_err(c, ISKRA_EINVAL, "bad MCC id");
  if (!(dt > 0)) return set_err(c, ISKRA_EINVAL, "dt must be positive");
  unsigned long long st = step;
  ISKRA_CUDA(c, cudaMemcpyAsync(c->d_step, &st, sizeof(st), cudaMemcpyHostToDevice, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->d_step_known = ~0ull;
  return launch_mcc(c, mid, dt, seed, c->d_step, step);
}

int iskra_mcc_counts(iskra_ctx *h, int mid, int64_t *counts) {
  if (!h || !counts) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (mid < 0 || mid >= (int)c->mccs.size()) return set_err(c, ISKRA_EINVAL, "bad MCC id");
  Mcc *m = c->mccs[mid];
  unsigned long long tmp[kMaxProc];
  ISKRA_CUDA(c, cudaMemcpyAsync(tmp, m->counts, sizeof(tmp), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(m->counts, 0, sizeof(tmp), c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < m->N; k++) counts[k] = (int64_t)tmp[k];
  return collect_device_errors(c);
}

int iskra_mcc_sigma(iskra_ctx *h, int mid, int process, const double *energies, int64_t n, double *sigma_out) {
  if (!h || (n > 0 && (!energies || !sigma_out)) || n < 0) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (mid < 0 || mid >= (int)c->mccs.size()) return set_err(c, ISKRA_EINVAL, "bad MCC id");
  Mcc *m = c->mccs[mid];
  if (process < 0 || process >= m->N) return set_err(c, ISKRA_EINVAL, "bad process index");
  if (n == 0) return ISKRA_OK;
  double *d = nullptr;
  ISKRA_CUDA(c, cudaMalloc(&d, 2 * (size_t)n * sizeof(double)));
  int rc = ISKRA_OK;
  cudaError_t e = cudaMemcpyAsync(d, energies, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    const int k = process, len = m->off[k + 1] - m->off[k];
    const long long blocks = std::min<long long>((n + 255) / 256, 1024);
    k_mcc_sigma<<<(unsigned)blocks, 256, 0, c->stream>>>(m->eps + m->off[k], m->sig + m->off[k], len, m->logu[k],
                                                         m->log_e0[k], m->inv_dlog[k], d, n, d + n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sigma_out, d + n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) rc = cuda_check(c, e, "iskra_mcc_sigma");
  cudaFree(d);
  return rc;
}

}  // extern "C"
