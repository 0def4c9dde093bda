// source.cu -- particle sources: sample!(::MaxwellianSource, species, Δt)
// (ParticleInCell/src/pic/sources.jl:24-34) on the device.  n = min(free
// slots, floor(rate Δt)) particles are appended after the species' live
// slots, x = U(0,1) wx + dx per axis, v = N(0,1) wv + dv per component
// (MaxwellianSource{2,3}, sources.jl:8-22; create_thermalized_beam,
// problem/configuration.jl:89-93, sets wv = sqrt(2 kB T / m)).  Appended
// particles sit in the unsorted tail the push walks.  Randomness: Philox
// keyed by (seed, source, step, particle index), so a run is reproducible.
#include <algorithm>
#include <cmath>
#include <new>

#include "internal.cuh"

namespace iskra {

struct SourceDev {        // device-resident per-source scratch
  long long base;         // first slot of the current sample
  long long n;            // particles in it
  unsigned int id0;       // first identifier
  unsigned int pad;
};

struct Source {
  int sid = 0;
  double rate = 0;
  double wx[2] = {0, 0}, dx[2] = {0, 0};
  double wv[3] = {0, 0, 0}, dv[3] = {0, 0, 0};
  bool every_step = false;
  unsigned long long calls = 0;  // one-off samples so far (a counter word of their keys)
  SourceDev *d = nullptr;
};

struct SourceArgs {
  SpeciesDev s;
  SourceDev *d;
  long long cap, nmax;    // capacity, floor(rate Δt)
  double wx[2], dx[2];    // in cells: wx / Δh, dx / Δh
  float wv[3], dv[3];
  int nx, ny;
  uint32_t k0, k1;        // Philox key (seed)
  uint32_t src;           // source index (a counter word)
  const unsigned long long *step;  // device step counter (a counter word), or nullptr:
  unsigned long long step_value;   //   then this value
};

// reserves the slots: n = min(cap - np, floor(rate Δt)) (sources.jl:30)
__global__ void k_source_reserve(SourceArgs A) {
  pdl_wait();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  SpeciesState &st = *A.s.st;
  long long n = A.cap - st.np;
  if (n > A.nmax) n = A.nmax;
  if (n < 0) n = 0;
  A.d->base = st.np;
  A.d->n = n;
  A.d->id0 = st.next_id;
  st.np += n;
  st.next_id += (unsigned)n;
}

// px = rand() wx + dx, pv = randn() wv + dv (sources.jl:31-32) for slot
// base + k; U(0,1) with 24 random bits, N(0,1) by Box-Muller (both values of
// a pair used)
__global__ void k_source_fill(SourceArgs A, int *err) {
  pdl_wait();
  const long long n = A.d->n, base = A.d->base;
  const unsigned long long step = A.step ? *A.step : A.step_value;
  const int cur = A.s.st->cur;
  float4 *xv = pick(A.s.xv[0], A.s.xv[1], cur);
  float2 *zc = pick(A.s.zc[0], A.s.zc[1], cur);
  uint32_t *id = pick(A.s.id[0], A.s.id[1], cur);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const U4 c0 = {(uint32_t)k, (uint32_t)(k >> 32), (uint32_t)step, A.src};
    const U4 r0 = philox4x32_10(c0, A.k0, A.k1);
    const U4 r1 = philox4x32_10(U4{c0.x, c0.y, c0.z, A.src | 0x80000000u}, A.k0, A.k1 ^ (uint32_t)(step >> 32));
    // x / Δh = U wx / Δh + dx / Δh (FMAs in cell units: no FP64 division here)
    const double fx = fma((double)u01(r0.x), A.wx[0], A.dx[0]);
    const double fy = fma((double)u01(r0.y), A.wx[1], A.dx[1]);
    // Box-Muller: two normals from (r0.z, r0.w), one from (r1.x, r1.y)
    const float a0 = fmaxf(u01(r0.z), 1.0e-12f), a1 = fmaxf(u01(r1.x), 1.0e-12f);
    const float rad0 = sqrtf(-2.0f * logf(a0)), rad1 = sqrtf(-2.0f * logf(a1));
    const float g0 = rad0 * cospif(2.0f * u01(r0.w)), g1 = rad0 * sinpif(2.0f * u01(r0.w));
    const float g2 = rad1 * cospif(2.0f * u01(r1.y));
    const float vx = fmaf(g0, A.wv[0], A.dv[0]), vy = fmaf(g1, A.wv[1], A.dv[1]), vz = fmaf(g2, A.wv[2], A.dv[2]);
    long long ux, uy;
    int cell = cell_of_units(fx, fy, A.nx, A.ny, ux, uy);
    if (cell < 0) atomicOr(err, DERR_DOMAIN);
    const long long p = base + k;
    xv[p] = make_float4((float)ux * kOffInv, (float)uy * kOffInv, vx, vy);
    zc[p] = make_float2(vz, __int_as_float(cell));
    id[p] = A.d->id0 + (uint32_t)k;
  }
}

static std::vector<Source> &sources_of(Ctx *c) {
  return *reinterpret_cast<std::vector<Source> *>(c->sources);
}

int launch_source(Ctx *c, int src, double dt, uint64_t seed, const unsigned long long *step,
                  unsigned long long step_value) {
  Source &S = sources_of(c)[src];
  Species &sp = c->species[S.sid];
  SourceArgs A{};
  A.s = sp.dev;
  A.d = S.d;
  A.cap = sp.cap;
  A.nmax = (long long)std::floor(S.rate * dt);
  if (A.nmax <= 0) return ISKRA_OK;
  const double h[2] = {c->g.dx, c->g.dy};
  for (int a = 0; a < 2; a++) {
    A.wx[a] = S.wx[a] / h[a];
    A.dx[a] = S.dx[a] / h[a];
  }
  for (int a = 0; a < 3; a++) {
    A.wv[a] = (float)S.wv[a];
    A.dv[a] = (float)S.dv[a];
  }
  A.nx = c->nx;
  A.ny = c->ny;
  A.k0 = (uint32_t)seed;
  A.k1 = (uint32_t)(seed >> 32) ^ 0x5EED50u;
  A.src = (uint32_t)src;
  A.step = step;
  A.step_value = step_value;
  ISKRA_CUDA(c, launch_pdl(k_source_reserve, 1, 32, 0, c->stream, A));
  const long long blocks = std::min<long long>((A.nmax + 255) / 256, (long long)c->num_sms * 8);
  ISKRA_CUDA(c, launch_pdl(k_source_fill, (int)std::max(1LL, blocks), 256, 0, c->stream, A, c->d_err));
  ISKRA_CUDA(c, cudaGetLastError());
  sp.acc_valid = false;  // new particles: the density no longer matches
  sp.n_valid = false;
  return ISKRA_OK;
}

// the sources sampled at the start of every iskra_step (the loop of
// ParticleInCell.solve, ParticleInCell.jl:104-106)
int launch_step_sources(Ctx *c, double dt, uint64_t seed) {
  if (!c->sources) return ISKRA_OK;
  auto &v = sources_of(c);
  for (int k = 0; k < (int)v.size(); k++) {
    if (!v[k].every_step) continue;
    int rc = launch_source(c, k, dt, seed, c->d_step, 0);
    if (rc) return rc;
  }
  return ISKRA_OK;
}

void sources_destroy(Ctx *c) {
  if (!c->sources) return;
  for (auto &S : sources_of(c)) cudaFree(S.d);
  delete reinterpret_cast<std::vector<Source> *>(c->sources);
  c->sources = nullptr;
}

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_source_create(iskra_ctx *h, int sid, double rate, const double wx[2], const double dx[2],
                        const double wv[3], const double dv[3], int *src) {
  if (!h || !wx || !wv) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (sid < 0 || sid >= (int)c->species.size()) return set_err(c, ISKRA_EINVAL, "bad species");
  if (!(rate >= 0.0) || !std::isfinite(rate)) return set_err(c, ISKRA_EINVAL, "rate must be finite and >= 0");
  if (!c->sources) {
    c->sources = new (std::nothrow) std::vector<Source>();
    if (!c->sources) return ISKRA_ENOMEM;
  }
  Source S;
  S.sid = sid;
  S.rate = rate;
  for (int a = 0; a < 2; a++) {
    S.wx[a] = wx[a];
    S.dx[a] = dx ? dx[a] : 0.0;
  }
  for (int a = 0; a < 3; a++) {
    S.wv[a] = wv[a];
    S.dv[a] = dv ? dv[a] : 0.0;
  }
  if (cudaMalloc(&S.d, sizeof(SourceDev)) != cudaSuccess) return set_err(c, ISKRA_ENOMEM, "source scratch");
  ISKRA_CUDA(c, cudaMemset(S.d, 0, sizeof(SourceDev)));
  sources_of(c).push_back(S);
  if (src) *src = (int)sources_of(c).size() - 1;
  return ISKRA_OK;
}

int iskra_source_sample(iskra_ctx *h, int src, double dt, uint64_t seed) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->sources || src < 0 || src >= (int)sources_of(c).size()) return set_err(c, ISKRA_EINVAL, "bad source");
  if (!(dt > 0.0)) return set_err(c, ISKRA_EINVAL, "dt must be positive");
  Source &S = sources_of(c)[src];
  // one-off samples take their call number as the step word, with the top
  // bit set so they never share a key with a step's sample
  return launch_source(c, src, dt, seed, nullptr, (1ull << 63) | S.calls++);
}

int iskra_source_set_every_step(iskra_ctx *h, int src, int on) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->sources || src < 0 || src >= (int)sources_of(c).size()) return set_err(c, ISKRA_EINVAL, "bad source");
  sources_of(c)[src].every_step = on != 0;
  invalidate_graphs(c);
  return ISKRA_OK;
}

}  // extern "C"
