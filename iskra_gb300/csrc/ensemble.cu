// ensemble.cu -- batched independent runs of one small discharge setup.
//
// An ensemble copies the configuration of a template context (species,
// boundary rules, MCC sets, the assembled Poisson operator with its driven
// electrodes) and holds R independent runs of it: per run a segment of every
// species store, its own deposit accumulators, ρ, ϕ and E, MCC keys and
// collision counters, and drive amplitudes.  One step of all runs is a
// handful of launches with the run as blockIdx.y (MCC, push) or blockIdx.x
// (field solve), captured in one CUDA graph:
//   MCC set by set (mcc.jl:231-289) -> push of every species with the
//   run's whole E grid and deposit in shared memory (ParticleInCell.jl
//   :102-122) -> per run ρ, FP64 separable Poisson solve and E
//   (generalized_poisson.jl:372-410).
// Each run follows the same algorithm as a single-run context with the same
// seed (MCC keys are formed the same way), so runs compare one to one with
// unbatched execution.  The template context must outlive the ensemble (the
// cross-section tables, gas density and operator tables are shared).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "internal.cuh"

namespace iskra {

struct EnsSpecies {
  long long cap = 0;  // per run
  float4 *xv[2] = {nullptr, nullptr};
  float2 *zc[2] = {nullptr, nullptr};
  uint32_t *id[2] = {nullptr, nullptr};
  SpeciesState *st = nullptr;      // R
  unsigned long long *acc = nullptr;  // R x nn
  unsigned *cnt = nullptr;         // R x nn
  SpeciesDev *views = nullptr;     // R run views (device)
};

struct EnsMcc {
  uint2 *keys = nullptr;                 // R
  unsigned long long *counts = nullptr;  // R x N
  int N = 0;
  MccWork *work = nullptr;               // work list (R x work_cap entries)
  unsigned long long *nwork = nullptr;   // R counters, kNworkStride apart
  // the list is made by the push of the set's source species in the step
  // before (the first set of each source species); otherwise by a selection
  // pass at the start of the step
  bool folded = false;
};

struct Ens {
  Ctx *c = nullptr;  // template
  int R = 0, nn = 0;
  std::vector<EnsSpecies> sp;
  std::vector<EnsMcc> mcc;
  double *rho = nullptr, *x = nullptr;
  float2 *E32 = nullptr;
  double *amp = nullptr;  // R x ngroups
  int ngroups = 0;
  unsigned long long *d_step = nullptr;
  unsigned long long step = 0;
  int *d_err = nullptr, *h_err = nullptr;
  std::vector<uint64_t> seeds;
  bool keys_valid = false;
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0;
  cudaGraphExec_t compact_graph = nullptr;
  int compact_every = 32;
  unsigned long long work_cap = 0;        // MCC work-list entries per run and set
  bool lists_valid = false;               // the folded sets' lists hold the next step's selections
  std::string err;
};

static int ens_err(Ens *e, int code, const std::string &m) {
  e->err = m;
  return code;
}

#define ENS_CUDA(e, call)                                                               \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return ens_err((e), ISKRA_ECUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// per-run state transitions (one thread per run)
enum { kRunsAppendBegin, kRunsAppendEnd, kRunsCompactBegin, kRunsCompactEnd };
__global__ void k_runs_state(SpeciesState *st, int R, long long cap, int op) {
  pdl_wait();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  SpeciesState &s = st[r];
  if (op == kRunsAppendBegin) s.np_new = s.np;
  else if (op == kRunsAppendEnd) s.np = s.np_new > cap ? cap : s.np_new;
  else if (op == kRunsCompactBegin) s.np_new = 0;
  else {
    s.np = s.np_new;
    s.cur ^= 1;
  }
}

// Several of the step's per-run bookkeeping operations in one launch (each a
// few bytes per run; as separate launches they cost more than their work):
// the step counter, state transitions of up to kRunsOpsMax species states in
// order, and zeroed work-list counters.
constexpr int kRunsOpsMax = 8, kRunsZeroMax = 4;
struct RunsOps {
  unsigned long long *d_step;  // incremented when not null
  int n, nzero;
  SpeciesState *st[kRunsOpsMax];
  long long cap[kRunsOpsMax];
  int op[kRunsOpsMax];
  unsigned long long *zero[kRunsZeroMax];  // R counters, kNworkStride apart
};
__global__ void k_runs_ops(RunsOps O, int R) {
  pdl_wait();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (O.d_step && r == 0) *O.d_step += 1ull;
  if (r >= R) return;
  for (int i = 0; i < O.n; i++) {
    SpeciesState &s = O.st[i][r];
    if (O.op[i] == kRunsAppendBegin) s.np_new = s.np;
    else if (O.op[i] == kRunsAppendEnd) s.np = s.np_new > O.cap[i] ? O.cap[i] : s.np_new;
  }
  for (int z = 0; z < O.nzero; z++) O.zero[z][(size_t)r * kNworkStride] = 0ull;
}

// Drop discarded particles of every run: live particles move to the other
// buffer of their run's segment (warp-aggregated slots on the run's cursor).
__global__ void __launch_bounds__(256) k_compact_runs(const SpeciesDev *__restrict__ runs) {
  pdl_wait();
  const unsigned FULL = 0xffffffffu;
  const SpeciesDev s = runs[blockIdx.y];
  const int lane = threadIdx.x & 31;
  const long long np = s.st->np;
  const int cur = s.st->cur;
  const float4 *xv = pick(s.xv[0], s.xv[1], cur);
  const float2 *zc = pick(s.zc[0], s.zc[1], cur);
  const uint32_t *id = pick(s.id[0], s.id[1], cur);
  float4 *xo = pick(s.xv[0], s.xv[1], cur ^ 1);
  float2 *zo = pick(s.zc[0], s.zc[1], cur ^ 1);
  uint32_t *io = pick(s.id[0], s.id[1], cur ^ 1);
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = warp * 32; base < np; base += nwarps * 32) {
    const long long p = base + lane;
    bool live = false;
    float4 a;
    float2 b;
    uint32_t pid = 0;
    if (p < np) {
      b = zc[p];
      live = __float_as_int(b.y) >= 0;
      if (live) {
        a = xv[p];
        pid = id[p];
      }
    }
    const unsigned m = __ballot_sync(FULL, live);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    long long slot = 0;
    if (lane == leader) slot = atomicAdd((unsigned long long *)&s.st->np_new, (unsigned long long)__popc(m));
    slot = __shfl_sync(FULL, slot, leader) + __popc(m & ((1u << lane) - 1u));
    if (live) {
      xo[slot] = a;
      zo[slot] = b;
      io[slot] = pid;
    }
  }
}

static int ens_blocks_per_run(Ens *e) {
  long long cap = 1;
  for (auto &s : e->sp) cap = std::max(cap, s.cap);
  // about 16 k particle slots per block, at most 64 blocks per run
  long long b = (cap + 16383) / 16384;
  return (int)std::max(1LL, std::min(64LL, b));
}

static int ens_queue_step(Ens *e, double dt) {
  Ctx *c = e->c;
  cudaStream_t st = c->stream;
  const int R = e->R, bpr = ens_blocks_per_run(e);
  const int rb = (R + 127) / 128;
  // bookkeeping gathered into one k_runs_ops launch before each MCC set and
  // before the pushes
  RunsOps O{};
  O.d_step = e->d_step;
  auto op = [&](int sp, int kind) -> int {
    if (O.n == kRunsOpsMax) {
      ENS_CUDA(e, launch_pdl(k_runs_ops, rb, 128, 0, st, O, R));
      O = RunsOps{};
    }
    O.st[O.n] = e->sp[sp].st;
    O.cap[O.n] = e->sp[sp].cap;
    O.op[O.n++] = kind;
    return ISKRA_OK;
  };
  auto flush = [&]() -> int {
    if (O.d_step || O.n || O.nzero) ENS_CUDA(e, launch_pdl(k_runs_ops, rb, 128, 0, st, O, R));
    O = RunsOps{};
    return ISKRA_OK;
  };
  for (int m = 0; m < (int)e->mcc.size(); m++) {
    const int src = mcc_src(c, m), prod = mcc_prod(c, m);
    int rc = op(src, kRunsAppendBegin);
    if (!rc && prod >= 0) rc = op(prod, kRunsAppendBegin);
    if (!rc) rc = flush();
    if (rc) return rc;
    rc = launch_mcc_runs(c, m, dt, R, e->sp[src].views, prod >= 0 ? e->sp[prod].views : e->sp[src].views,
                             e->mcc[m].keys, e->mcc[m].counts, e->E32, e->nn, bpr, e->mcc[m].work, e->mcc[m].nwork,
                             e->work_cap, e->d_step, e->d_err, st, e->mcc[m].folded ? kMccCollideOnly : kMccBoth);
    if (rc) return ens_err(e, rc, c->err);
    rc = op(src, kRunsAppendEnd);
    if (!rc && prod >= 0) rc = op(prod, kRunsAppendEnd);
    if (rc) return rc;
  }
  // the pushes make the folded sets' lists for the next step
  for (int m = 0; m < (int)e->mcc.size(); m++) {
    if (!e->mcc[m].folded) continue;
    if (O.nzero == kRunsZeroMax) {
      const int rc = flush();
      if (rc) return rc;
    }
    O.zero[O.nzero++] = e->mcc[m].nwork;
  }
  {
    const int rc = flush();
    if (rc) return rc;
  }
  for (int s = 0; s < (int)e->sp.size(); s++) {
    PushSelect S{};
    bool sel = false;
    for (int m = 0; m < (int)e->mcc.size() && !sel; m++) {
      if (!e->mcc[m].folded || mcc_src(c, m) != s) continue;
      int rc = mcc_push_select(c, m, dt, &S);
      if (rc) return ens_err(e, rc, c->err);
      S.keys = e->mcc[m].keys;
      S.work = e->mcc[m].work;
      S.nwork = e->mcc[m].nwork;
      S.cap_run = e->work_cap;
      S.d_step = e->d_step;
      sel = true;
    }
    int rc = launch_push_runs(c, s, e->sp[s].views, R, e->E32, (float)dt, bpr, e->d_err, st, sel ? &S : nullptr);
    if (rc) return ens_err(e, rc, c->err);
  }
  FieldRunsHost H{};
  H.ns = (int)e->sp.size();
  for (int s = 0; s < H.ns; s++) {
    H.acc[s] = e->sp[s].acc;
    H.cnt[s] = e->sp[s].cnt;
    H.scale[s] = c->species[s].w0 * std::ldexp(1.0, -48);
    H.q[s] = c->species[s].q;
  }
  H.rho = e->rho;
  H.x = e->x;
  H.E32 = e->E32;
  H.amp = e->amp;
  H.d_step = e->d_step;
  H.dt = dt;
  H.err = e->d_err;
  int rc = launch_field_runs(c, R, H, st);
  if (rc) return ens_err(e, rc, c->err);
  return ISKRA_OK;
}

// The folded sets' work lists for the next step, by a selection pass (after
// an upload or a compaction moved the particles the last push selected).
static int ens_queue_select_ahead(Ens *e, double dt) {
  Ctx *c = e->c;
  const int bpr = ens_blocks_per_run(e);
  for (int m = 0; m < (int)e->mcc.size(); m++) {
    if (!e->mcc[m].folded) continue;
    const int src = mcc_src(c, m), prod = mcc_prod(c, m);
    int rc = launch_mcc_runs(c, m, dt, e->R, e->sp[src].views, prod >= 0 ? e->sp[prod].views : e->sp[src].views,
                             e->mcc[m].keys, e->mcc[m].counts, e->E32, e->nn, bpr, e->mcc[m].work,
                             e->mcc[m].nwork, e->work_cap, e->d_step, e->d_err, c->stream, kMccSelectAhead);
    if (rc) return ens_err(e, rc, c->err);
  }
  return ISKRA_OK;
}

static int ens_queue_compact(Ens *e) {
  Ctx *c = e->c;
  cudaStream_t st = c->stream;
  const int R = e->R, rb = (R + 127) / 128;
  for (auto &s : e->sp) {
    ENS_CUDA(e, launch_pdl(k_runs_state, rb, 128, 0, st, s.st, R, s.cap, (int)kRunsCompactBegin));
    ENS_CUDA(e, launch_pdl(k_compact_runs, dim3(ens_blocks_per_run(e), R), 256, 0, st, (const SpeciesDev *)s.views));
    ENS_CUDA(e, launch_pdl(k_runs_state, rb, 128, 0, st, s.st, R, s.cap, (int)kRunsCompactEnd));
  }
  return ISKRA_OK;
}

template <class F>
static int ens_capture(Ens *e, cudaGraphExec_t *out, F fn) {
  cudaStream_t st = e->c->stream;
  cudaGraph_t g;
  ENS_CUDA(e, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int crc = fn();
  cudaError_t ce = cudaStreamEndCapture(st, &g);
  if (crc) {
    if (ce == cudaSuccess) cudaGraphDestroy(g);
    return crc;
  }
  ENS_CUDA(e, ce);
  cudaError_t ie = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  ENS_CUDA(e, ie);
  return ISKRA_OK;
}

static int ens_collect(Ens *e) {
  cudaStream_t st = e->c->stream;
  ENS_CUDA(e, cudaMemcpyAsync(e->h_err, e->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  ENS_CUDA(e, cudaStreamSynchronize(st));
  const int f = *e->h_err;
  if (!f) return ISKRA_OK;
  ENS_CUDA(e, cudaMemsetAsync(e->d_err, 0, sizeof(int), st));
  ENS_CUDA(e, cudaStreamSynchronize(st));
  if (f & DERR_NAN) return ens_err(e, ISKRA_ENAN, "non-finite particle or field value");
  if (f & DERR_PROB) return ens_err(e, ISKRA_EPROB, "MCC collision probability above its bound");
  if (f & DERR_CAPACITY) return ens_err(e, ISKRA_ECAPACITY, "run capacity exceeded; particles dropped");
  if (f & DERR_DOMAIN) return ens_err(e, ISKRA_EDOMAIN, "particle outside the grid on an axis without wrap!/discard!");
  if (f & DERR_OVERFLOW) return ens_err(e, ISKRA_ECAPACITY, "deposit: more than 16383 macroparticles in one cell");
  return ens_err(e, ISKRA_ECUDA, "unknown device error flag");
}

static void ens_free(Ens *e) {
  if (!e || !e->c) return;
  if (e->c->stream) cudaStreamSynchronize(e->c->stream);
  auto &v = e->c->ensembles;
  v.erase(std::remove(v.begin(), v.end(), (void *)e), v.end());
  if (e->graph) cudaGraphExecDestroy(e->graph);
  if (e->compact_graph) cudaGraphExecDestroy(e->compact_graph);
  for (auto &s : e->sp) {
    for (int b = 0; b < 2; b++) {
      cudaFree(s.xv[b]);
      cudaFree(s.zc[b]);
      cudaFree(s.id[b]);
    }
    cudaFree(s.st);
    cudaFree(s.acc);
    cudaFree(s.cnt);
    cudaFree(s.views);
  }
  for (auto &m : e->mcc) {
    cudaFree(m.keys);
    cudaFree(m.counts);
    cudaFree(m.work);
    cudaFree(m.nwork);
  }
  cudaFree(e->rho);
  cudaFree(e->x);
  cudaFree(e->E32);
  cudaFree(e->amp);
  cudaFree(e->d_step);
  cudaFree(e->d_err);
  if (e->h_err) cudaFreeHost(e->h_err);
  *e = Ens{};  // detached: every later call but destroy fails
}

void ensembles_detach(Ctx *c) {
  std::vector<void *> v = c->ensembles;
  for (void *p : v) ens_free((Ens *)p);
  c->ensembles.clear();
}

static int ens_update_keys(Ens *e) {
  if (e->keys_valid) return ISKRA_OK;
  for (int m = 0; m < (int)e->mcc.size(); m++) {
    std::vector<uint2> k(e->R);
    for (int r = 0; r < e->R; r++) mcc_key(e->seeds[r], mcc_set_index(e->c, m), k[r].x, k[r].y);
    ENS_CUDA(e, cudaMemcpy(e->mcc[m].keys, k.data(), e->R * sizeof(uint2), cudaMemcpyHostToDevice));
  }
  e->keys_valid = true;
  return ISKRA_OK;
}

}  // namespace iskra

using namespace iskra;

struct iskra_ens {
  Ens e;
};

extern "C" {

int iskra_ens_create(iskra_ctx *tmpl, int nruns, int64_t cap_per_run, iskra_ens **out) {
  if (!tmpl || !out || nruns < 1 || nruns > 65535 || cap_per_run < 1 || cap_per_run > (1LL << 31) - 1)
    return ISKRA_EINVAL;
  *out = nullptr;
  Ctx *c = &tmpl->c;
  if (c->species.empty()) return set_err(c, ISKRA_EINVAL, "template has no species");
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "template has no Poisson solver");
  if (c->has_circuit) return set_err(c, ISKRA_EINVAL, "ensembles drive electrodes directly (no circuit)");
  if (c->trk) return set_err(c, ISKRA_EINVAL, "ensembles take no surface tracker");
  if (c->sources || c->dsmcs) return set_err(c, ISKRA_EINVAL, "ensembles take no particle sources or DSMC sets");
  if ((c->nx - 1) * (c->ny - 1) > 400) return set_err(c, ISKRA_EINVAL, "ensemble grids hold at most 400 cells");
  if ((double)cap_per_run * nruns > 2.0e9) return set_err(c, ISKRA_EINVAL, "ensemble store above 2e9 slots");
  iskra_ens *h = new (std::nothrow) iskra_ens();
  if (!h) return ISKRA_ENOMEM;
  Ens *e = &h->e;
  e->c = c;
  e->R = nruns;
  e->nn = c->nn;
  const size_t R = nruns, nn = c->nn;
  auto fail = [&](int rc) {
    c->err = e->err.empty() ? c->err : e->err;
    ens_free(e);
    delete h;
    return rc;
  };
#define ENS_ALLOC(ptr, bytes)                                        \
  if (cudaMalloc(&(ptr), (bytes)) != cudaSuccess) {                  \
    e->err = "out of device memory for the ensemble";                \
    return fail(ISKRA_ENOMEM);                                       \
  }
  e->sp.resize(c->species.size());
  for (size_t s = 0; s < c->species.size(); s++) {
    EnsSpecies &q = e->sp[s];
    q.cap = cap_per_run;
    const size_t slots = R * (size_t)cap_per_run;
    for (int b = 0; b < 2; b++) {
      ENS_ALLOC(q.xv[b], slots * sizeof(float4));
      ENS_ALLOC(q.zc[b], slots * sizeof(float2));
      ENS_ALLOC(q.id[b], slots * sizeof(uint32_t));
    }
    ENS_ALLOC(q.st, R * sizeof(SpeciesState));
    ENS_ALLOC(q.acc, R * nn * sizeof(unsigned long long));
    ENS_ALLOC(q.cnt, R * nn * sizeof(unsigned));
    ENS_ALLOC(q.views, R * sizeof(SpeciesDev));
    cudaMemset(q.st, 0, R * sizeof(SpeciesState));
    cudaMemset(q.acc, 0, R * nn * sizeof(unsigned long long));
    cudaMemset(q.cnt, 0, R * nn * sizeof(unsigned));
    std::vector<SpeciesDev> v(R);
    for (size_t r = 0; r < R; r++) {
      SpeciesDev &d = v[r];
      const size_t off = r * (size_t)cap_per_run;
      for (int b = 0; b < 2; b++) {
        d.xv[b] = q.xv[b] + off;
        d.zc[b] = q.zc[b] + off;
        d.id[b] = q.id[b] + off;
      }
      d.st = q.st + r;
      d.acc = q.acc + r * nn;
      d.cnt = q.cnt + r * nn;
      d.cap = cap_per_run;
      d.tile_begin = nullptr;
    }
    cudaMemcpy(q.views, v.data(), R * sizeof(SpeciesDev), cudaMemcpyHostToDevice);
  }
  e->mcc.resize(c->mccs.size());
  for (size_t m = 0; m < c->mccs.size(); m++) {
    e->mcc[m].N = mcc_nproc(c, (int)m);
    ENS_ALLOC(e->mcc[m].keys, R * sizeof(uint2));
    ENS_ALLOC(e->mcc[m].counts, R * e->mcc[m].N * sizeof(unsigned long long));
    cudaMemset(e->mcc[m].counts, 0, R * e->mcc[m].N * sizeof(unsigned long long));
  }
  ENS_ALLOC(e->rho, R * nn * sizeof(double));
  ENS_ALLOC(e->x, R * nn * sizeof(double));
  ENS_ALLOC(e->E32, R * nn * sizeof(float2));
  cudaMemset(e->rho, 0, R * nn * sizeof(double));
  cudaMemset(e->x, 0, R * nn * sizeof(double));
  cudaMemset(e->E32, 0, R * nn * sizeof(float2));
  int rc = poisson_upload_fp64(c);
  if (rc) return fail(rc);
  e->ngroups = poisson_ndrive(c);
  {
    const int ng = std::max(1, e->ngroups);
    ENS_ALLOC(e->amp, R * ng * sizeof(double));
    std::vector<double> a(R * ng, 0.0);
    for (size_t r = 0; r < R; r++)
      for (int g = 0; g < e->ngroups; g++) a[r * ng + g] = poisson_drive_amp(c, g);
    cudaMemcpy(e->amp, a.data(), a.size() * sizeof(double), cudaMemcpyHostToDevice);
  }
  if (!c->mccs.empty()) {
    e->work_cap = (unsigned long long)cap_per_run;  // per run segment
    std::vector<bool> src_folded(c->species.size(), false);
    for (int m = 0; m < (int)e->mcc.size(); m++) {
      ENS_ALLOC(e->mcc[m].work, mcc_work_bytes(R, e->work_cap));
      ENS_ALLOC(e->mcc[m].nwork, (size_t)R * kNworkStride * sizeof(unsigned long long));
      cudaMemset(e->mcc[m].nwork, 0, (size_t)R * kNworkStride * sizeof(unsigned long long));
      const int src = mcc_src(c, m);
      e->mcc[m].folded = !src_folded[src];
      src_folded[src] = true;
    }
  }
  ENS_ALLOC(e->d_step, sizeof(unsigned long long));
  cudaMemset(e->d_step, 0, sizeof(unsigned long long));
  ENS_ALLOC(e->d_err, sizeof(int));
  cudaMemset(e->d_err, 0, sizeof(int));
  if (cudaMallocHost(&e->h_err, sizeof(int)) != cudaSuccess) return fail(ISKRA_ENOMEM);
#undef ENS_ALLOC
  e->seeds.resize(R);
  for (size_t r = 0; r < R; r++) e->seeds[r] = 1000 + r;
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(ISKRA_ECUDA);
  c->ensembles.push_back((void *)e);
  *out = h;
  return ISKRA_OK;
}

int iskra_ens_destroy(iskra_ens *h) {
  if (!h) return ISKRA_OK;
  ens_free(&h->e);
  delete h;
  return ISKRA_OK;
}

const char *iskra_ens_last_error(const iskra_ens *h) { return h ? h->e.err.c_str() : "null ensemble"; }

int iskra_ens_set_seeds(iskra_ens *h, const uint64_t *seeds) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h || !seeds) return ISKRA_EINVAL;
  Ens *e = &h->e;
  e->seeds.assign(seeds, seeds + e->R);
  e->keys_valid = false;
  return ISKRA_OK;
}

int iskra_ens_set_drive_amplitude(iskra_ens *h, int group, const double *amp) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h || !amp) return ISKRA_EINVAL;
  Ens *e = &h->e;
  if (group < 0 || group >= e->ngroups) return ens_err(e, ISKRA_EINVAL, "bad drive group");
  ENS_CUDA(e, cudaStreamSynchronize(e->c->stream));
  std::vector<double> a((size_t)e->R * e->ngroups);
  ENS_CUDA(e, cudaMemcpy(a.data(), e->amp, a.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int r = 0; r < e->R; r++) a[(size_t)r * e->ngroups + group] = amp[r];
  ENS_CUDA(e, cudaMemcpy(e->amp, a.data(), a.size() * sizeof(double), cudaMemcpyHostToDevice));
  return ISKRA_OK;
}

int iskra_ens_upload(iskra_ens *h, int run, int sid, const double *x, const double *v, const uint32_t *id,
                     int64_t np, int64_t ld) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h) return ISKRA_EINVAL;
  Ens *e = &h->e;
  if (run < 0 || run >= e->R || sid < 0 || sid >= (int)e->sp.size()) return ens_err(e, ISKRA_EINVAL, "bad run or species");
  EnsSpecies &q = e->sp[sid];
  if (np < 0 || np > q.cap) return ens_err(e, ISKRA_ECAPACITY, "np exceeds the run capacity");
  if (np > 0 && (!x || !v || ld < np)) return ens_err(e, ISKRA_EINVAL, "bad particle arrays");
  const size_t off = (size_t)run * q.cap;
  e->lists_valid = false;  // new particles: the next step selects from scratch
  int rc = upload_particles(e->c, x, v, id, np, ld, q.xv[0] + off, q.zc[0] + off, q.id[0] + off);
  if (rc) return ens_err(e, rc, e->c->err);
  SpeciesState s0{};
  s0.np = np;
  s0.cur = 0;
  uint32_t maxid = (uint32_t)np;
  if (id)
    for (int64_t p = 0; p < np; p++) maxid = std::max(maxid, id[p]);
  s0.next_id = maxid + 1;
  ENS_CUDA(e, cudaMemcpy(q.st + run, &s0, sizeof(s0), cudaMemcpyHostToDevice));
  return ISKRA_OK;
}

int iskra_ens_count(iskra_ens *h, int run, int sid, int64_t *np) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h || !np) return ISKRA_EINVAL;
  Ens *e = &h->e;
  if (run < 0 || run >= e->R || sid < 0 || sid >= (int)e->sp.size()) return ens_err(e, ISKRA_EINVAL, "bad run or species");
  int rc = ens_collect(e);
  if (rc) return rc;
  // live particles: compact first (cheap next to a download)
  if (!e->compact_graph) {
    rc = ens_capture(e, &e->compact_graph, [&]() { return ens_queue_compact(e); });
    if (rc) return rc;
  }
  ENS_CUDA(e, cudaGraphLaunch(e->compact_graph, e->c->stream));
  e->lists_valid = false;  // the particles moved
  SpeciesState s{};
  ENS_CUDA(e, cudaMemcpyAsync(&s, e->sp[sid].st + run, sizeof(s), cudaMemcpyDeviceToHost, e->c->stream));
  ENS_CUDA(e, cudaStreamSynchronize(e->c->stream));
  *np = s.np;
  return ISKRA_OK;
}

int iskra_ens_download(iskra_ens *h, int run, int sid, double *x, double *v, uint32_t *id, int64_t ld,
                       int64_t *np_out) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h) return ISKRA_EINVAL;
  Ens *e = &h->e;
  int64_t np = 0;
  int rc = iskra_ens_count(h, run, sid, &np);
  if (rc) return rc;
  if (np_out) *np_out = np;
  if (np > ld) return ens_err(e, ISKRA_ECAPACITY, "host arrays too small for the live particles");
  EnsSpecies &q = e->sp[sid];
  SpeciesState s{};
  ENS_CUDA(e, cudaMemcpy(&s, q.st + run, sizeof(s), cudaMemcpyDeviceToHost));
  const size_t off = (size_t)run * q.cap;
  rc = download_particles(e->c, q.xv[s.cur] + off, q.zc[s.cur] + off, q.id[s.cur] + off, np, x, v, id, ld);
  if (rc) return ens_err(e, rc, e->c->err);
  return ISKRA_OK;
}

int iskra_ens_step(iskra_ens *h, double dt, int nsteps) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h) return ISKRA_EINVAL;
  Ens *e = &h->e;
  if (!(dt > 0) || nsteps < 0) return ens_err(e, ISKRA_EINVAL, "bad dt / nsteps");
  if (nsteps == 0) return ISKRA_OK;
  if (!e->keys_valid) e->lists_valid = false;  // selections drawn with other keys
  int rc = ens_update_keys(e);
  if (rc) return rc;
  if (e->graph && e->graph_dt != dt) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  if (e->graph_dt != dt) e->lists_valid = false;  // selections drawn for another Δt
  if (!e->graph) {
    rc = ens_capture(e, &e->graph, [&]() { return ens_queue_step(e, dt); });
    if (rc) return rc;
    e->graph_dt = dt;
  }
  if (!e->compact_graph) {
    rc = ens_capture(e, &e->compact_graph, [&]() { return ens_queue_compact(e); });
    if (rc) return rc;
  }
  for (int n = 0; n < nsteps; n++) {
    if (!e->lists_valid) {
      rc = ens_queue_select_ahead(e, dt);
      if (rc) return rc;
      e->lists_valid = true;
    }
    ENS_CUDA(e, cudaGraphLaunch(e->graph, e->c->stream));
    e->step++;
    if (e->compact_every > 0 && e->step % e->compact_every == 0) {
      ENS_CUDA(e, cudaGraphLaunch(e->compact_graph, e->c->stream));
      e->lists_valid = false;  // the particles moved
    }
  }
  return ISKRA_OK;
}

int iskra_ens_sync(iskra_ens *h) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h) return ISKRA_EINVAL;
  return ens_collect(&h->e);
}

int iskra_ens_mcc_counts(iskra_ens *h, int run, int mid, uint64_t *counts) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h || !counts) return ISKRA_EINVAL;
  Ens *e = &h->e;
  if (run < 0 || run >= e->R || mid < 0 || mid >= (int)e->mcc.size()) return ens_err(e, ISKRA_EINVAL, "bad run or set");
  int rc = ens_collect(e);
  if (rc) return rc;
  const int N = e->mcc[mid].N;
  ENS_CUDA(e, cudaMemcpy(counts, e->mcc[mid].counts + (size_t)run * N, N * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return ISKRA_OK;
}

int iskra_ens_field(iskra_ens *h, int run, int which, double *out) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h || !out) return ISKRA_EINVAL;
  Ens *e = &h->e;
  if (run < 0 || run >= e->R) return ens_err(e, ISKRA_EINVAL, "bad run");
  int rc = ens_collect(e);
  if (rc) return rc;
  const size_t nn = e->nn, o = (size_t)run * nn;
  if (which == ISKRA_FIELD_RHO) {
    ENS_CUDA(e, cudaMemcpy(out, e->rho + o, nn * sizeof(double), cudaMemcpyDeviceToHost));
  } else if (which == ISKRA_FIELD_PHI) {
    ENS_CUDA(e, cudaMemcpy(out, e->x + o, nn * sizeof(double), cudaMemcpyDeviceToHost));
  } else if (which == ISKRA_FIELD_E) {
    std::vector<float2> E(nn);
    ENS_CUDA(e, cudaMemcpy(E.data(), e->E32 + o, nn * sizeof(float2), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < nn; k++) {
      out[k] = E[k].x;
      out[k + nn] = E[k].y;
      out[k + 2 * nn] = 0.0;
    }
  } else {
    return ens_err(e, ISKRA_EINVAL, "bad field selector");
  }
  return ISKRA_OK;
}

int iskra_ens_set_compact_every(iskra_ens *h, int every) {
  if (h && !h->e.c) return ens_err(&h->e, ISKRA_EINVAL, "the ensemble's template context was destroyed");
  if (!h || every < 0) return ISKRA_EINVAL;
  h->e.compact_every = every;
  return ISKRA_OK;
}

}  // extern "C"
