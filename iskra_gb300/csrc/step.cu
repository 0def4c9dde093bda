// step.cu -- the RLC circuit (Circuit/src/Circuit.jl, circuit_coupling.jl) and
// the whole PIC step (the loop body of ParticleInCell.solve,
// ParticleInCell/src/ParticleInCell.jl:102-135) replayed as a CUDA graph.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "internal.cuh"

namespace iskra {

double *poisson_sigma_ptr(Ctx *c);
const double *poisson_x_ptr(Ctx *c);
const float2 *poisson_xd_ptr(Ctx *c);
void poisson_mark_x_stale(Ctx *c);
bool poisson_separable(Ctx *c);
int poisson_solve_blocking(Ctx *c, double rtol, int maxit);
int poisson_solve_graph(Ctx *c, double rtol);

struct CircuitArgs {
  CircuitDev *cd;
  const double *phi;
  const float2 *phid;          // ϕ as double-float pairs (separable solver), else nullptr
  double *sigma;
  int pos_ref, neg_ref;
  int wall;                    // discard wall feeding the floating electrode, -1 none
  int ns;
  SpeciesState *st[kMaxSpecies];
  double qw[kMaxSpecies];      // q * w0 per species
};

// advance!(circuit, ϕ, Δt, config) (circuit_coupling.jl:35-43) with
// advance_circuit! (Circuit.jl:117-136); V_ext = ϕ(positive) - ϕ(negative)
// of the PlasmaDevice (circuit_coupling.jl:18-29); wall-absorbed charge enters
// σ as hit! does (circuit_coupling.jl:45-55).  One thread, FP64.
__global__ void k_circuit(CircuitArgs A, double dt, unsigned long long *seen) {
  pdl_wait();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  CircuitDev &c = *A.cd;
  auto phi_at = [&](int k) { return A.phid ? (double)A.phid[k].x + (double)A.phid[k].y : A.phi[k]; };
  const double vext = phi_at(A.pos_ref) - phi_at(A.neg_ref);
  const double i = c.i, q = c.q, t = c.t;
  const double vsrc = c.amp * sin(2.0 * M_PI * c.freq * t) + c.dc;
  double in = (c.L / dt - c.R / 2) * i + vext - vsrc;
  if (c.C > 0.0) {
    in -= q / c.C;
    in /= (c.L / dt + c.R / 2);
    c.q = q + dt * i;
  } else {
    in /= (c.L / dt + c.R / 2);
  }
  c.i = in;
  c.t = t + dt;
  c.vext = vext;
  double ds = -dt * in / c.area * c.scale;
  if (A.wall >= 0) {
    for (int s = 0; s < A.ns; s++) {
      const unsigned long long now = A.st[s]->absorbed[A.wall];
      const unsigned long long d = now - seen[s];
      seen[s] = now;
      ds += A.qw[s] * (double)d / c.area;
    }
  }
  A.sigma[c.sigma_dof] += ds;
}

__global__ void k_step_begin(unsigned long long *d_step) { pdl_wait(); *d_step += 1ull; }

int launch_circuit(Ctx *c, double dt) {
  if (!c->cir_d) return set_err(c, ISKRA_EINVAL, "no circuit");
  CircuitArgs A{};
  A.cd = c->cir_d;
  A.phi = poisson_x_ptr(c);
  A.phid = poisson_xd_ptr(c);
  A.sigma = poisson_sigma_ptr(c);
  A.pos_ref = c->cir_pos_ref;
  A.neg_ref = c->cir_neg_ref;
  A.wall = c->cir_wall;
  A.ns = (int)c->species.size();
  for (int s = 0; s < A.ns; s++) {
    A.st[s] = c->species[s].dev.st;
    A.qw[s] = c->species[s].q * c->species[s].w0;
  }
  ISKRA_CUDA(c, launch_pdl(k_circuit, 1, 32, 0, c->stream, A, dt, c->cir_seen));
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// queue one PIC step (async; separable Poisson)
static int queue_step(Ctx *c, double dt, uint64_t seed, double rtol, bool blocking_solve) {
  int rc = launch_step_sources(c, dt, seed);  // sample! of every source (ParticleInCell.jl:104-106)
  if (rc) return rc;
  if (!c->mccs.empty()) {  // MCC keys read the step counter first
    ISKRA_CUDA(c, launch_pdl(k_step_begin, 1, 1, 0, c->stream, c->d_step));
    ISKRA_CUDA(c, cudaGetLastError());
    for (int m = 0; m < (int)c->mccs.size(); m++) {
      rc = launch_mcc(c, m, dt, seed, c->d_step, 0);
      if (rc) return rc;
    }
    rc = launch_step_dsmc(c, dt, seed);  // the DSMC sets, after the MCC sets (interactions)
    if (rc) return rc;
    rc = launch_advance_all(c, (float)dt, nullptr, nullptr);
    if (rc) return rc;
  } else {  // the push can advance it (nothing reads it before ρ)
    rc = launch_step_dsmc(c, dt, seed);
    if (rc) return rc;
    bool folded = false;
    rc = launch_advance_all(c, (float)dt, c->d_step, &folded);
    if (rc) return rc;
    if (!folded) {
      ISKRA_CUDA(c, launch_pdl(k_step_begin, 1, 1, 0, c->stream, c->d_step));
      ISKRA_CUDA(c, cudaGetLastError());
    }
  }
  if (c->cir_d) {
    rc = launch_circuit(c, dt);
    if (rc) return rc;
  }
  rc = blocking_solve ? launch_charge_density(c) : launch_step_density(c);
  if (rc) return rc;
  if (blocking_solve) return poisson_solve_blocking(c, rtol, 10000);
  return poisson_solve_graph(c, rtol);
}

// Steps between tile sorts of each species.  Between sorts the push reads E
// from and deposits into its tile's shared-memory window; particles that drift
// more than the kHalo-cell margin off their tile take the slower global path,
// and particles appended by MCC wait in the unsorted tail.  The automatic
// period lets the rms in-plane particle move reach 1.5 kHalo cells, clamped
// to [4, 64] steps.
static int update_sort_periods(Ctx *c, double dt) {
  const double h = std::min(c->g.dx, c->g.dy);
  for (int s = 0; s < (int)c->species.size(); s++) {
    if (c->sort_every >= 0) {
      c->sort_period[s] = c->sort_every;
      continue;
    }
    double v2 = 0;
    int rc = species_speed2(c, s, &v2);
    if (rc) return rc;
    const double cells = std::sqrt(v2) * dt / h;  // rms cells moved per step
    double p = cells > 0 ? 1.5 * kHalo / cells : 64.0;
    p = std::max(4.0, std::min(64.0, std::floor(p)));
    c->sort_period[s] = (int)std::max(2.0, std::min(256.0, std::round(p * c->sort_scale)));
  }
  c->periods_valid = true;
  return ISKRA_OK;
}

// Captures the work queued by fn() on the context stream into an executable
// graph and counts its kernel nodes.
template <class F>
static int capture(Ctx *c, cudaGraphExec_t *out, unsigned long long *kernels, F fn) {
  cudaGraph_t g;
  ISKRA_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int crc = fn();
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (crc) {
    if (e == cudaSuccess) cudaGraphDestroy(g);
    return crc;
  }
  ISKRA_CUDA(c, e);
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
  unsigned long long k = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
  }
  cudaError_t ei = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  ISKRA_CUDA(c, ei);
  *kernels = k;
  return ISKRA_OK;
}

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_circuit_create(iskra_ctx *h, double R, double L, double C, double amp, double freq, double dc,
                         int sigma_dof, const uint8_t *pos_nodes, const uint8_t *neg_nodes, double area,
                         double sigma_scale) {
  if (!h || !pos_nodes || !neg_nodes) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "create the Poisson solver first");
  double sv = 0;
  if (iskra_poisson_get_sigma(h, sigma_dof, &sv)) return set_err(c, ISKRA_EINVAL, "bad σ dof");
  if (!(area > 0) || !(L / 1.0 >= 0) || !(R >= 0)) return set_err(c, ISKRA_EINVAL, "bad circuit values");
  int pos_ref = -1, neg_ref = -1, wall = -1;
  for (int r = 0; r < c->nn && pos_ref < 0; r++)
    if (pos_nodes[r]) pos_ref = r;  // find_reference_node (configuration.jl:59-62)
  for (int r = 0; r < c->nn && neg_ref < 0; r++)
    if (neg_nodes[r]) neg_ref = r;
  if (pos_ref < 0 || neg_ref < 0) return set_err(c, ISKRA_EINVAL, "empty electrode");
  // the wall whose discarded particles land on the floating electrode:
  // 0 x-low (column i=1), 1 x-high (i=nx), 2 y-low (row j=1), 3 y-high (j=ny)
  for (int w = 0; w < 4 && wall < 0; w++) {
    bool all = true;
    const int len = w < 2 ? c->ny : c->nx;
    for (int k = 0; k < len && all; k++) {
      const int i = w == 0 ? 0 : w == 1 ? c->nx - 1 : k;
      const int j = w == 2 ? 0 : w == 3 ? c->ny - 1 : k;
      all = pos_nodes[i + c->nx * j] != 0;
    }
    if (all) wall = w;
  }
  CircuitDev d{};
  d.R = R;
  d.L = L;
  d.C = C;
  d.amp = amp;
  d.freq = freq;
  d.dc = dc;
  d.area = area;
  d.scale = sigma_scale;
  d.sigma_dof = sigma_dof - 1;
  if (!c->cir_d) ISKRA_CUDA(c, cudaMalloc(&c->cir_d, sizeof(CircuitDev)));
  ISKRA_CUDA(c, cudaMemcpy(c->cir_d, &d, sizeof(d), cudaMemcpyHostToDevice));
  c->cir_h = d;
  c->cir_pos_ref = pos_ref;
  c->cir_neg_ref = neg_ref;
  c->cir_wall = wall;
  if (!c->cir_seen) ISKRA_CUDA(c, cudaMalloc(&c->cir_seen, kMaxSpecies * sizeof(unsigned long long)));
  std::vector<unsigned long long> seen(kMaxSpecies, 0);
  for (int s = 0; s < (int)c->species.size(); s++) {
    SpeciesState st{};
    ISKRA_CUDA(c, cudaMemcpy(&st, c->species[s].dev.st, sizeof(st), cudaMemcpyDeviceToHost));
    if (wall >= 0) seen[s] = st.absorbed[wall];
  }
  ISKRA_CUDA(c, cudaMemcpy(c->cir_seen, seen.data(), kMaxSpecies * sizeof(unsigned long long), cudaMemcpyHostToDevice));
  c->has_circuit = true;
  invalidate_graphs(c);
  return ISKRA_OK;
}

int iskra_circuit_advance(iskra_ctx *h, double dt) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!(dt > 0)) return set_err(c, ISKRA_EINVAL, "dt must be positive");
  int rc = poisson_prepare(c);
  if (rc) return rc;
  return launch_circuit(c, dt);
}

int iskra_circuit_state(iskra_ctx *h, double state[5]) {
  if (!h || !state) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->cir_d) return set_err(c, ISKRA_EINVAL, "no circuit");
  CircuitDev d{};
  ISKRA_CUDA(c, cudaMemcpyAsync(&d, c->cir_d, sizeof(d), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  double sv = 0;
  int rc = iskra_poisson_get_sigma(h, d.sigma_dof + 1, &sv);
  if (rc) return rc;
  state[0] = d.t;
  state[1] = d.i;
  state[2] = d.q;
  state[3] = sv;
  state[4] = d.vext;
  return collect_device_errors(c);
}

int iskra_set_sort_every(iskra_ctx *h, int every) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  c->sort_every = every < 0 ? -1 : every;
  c->periods_valid = false;
  return ISKRA_OK;
}

int iskra_step(iskra_ctx *h, double dt, int nsteps, uint64_t seed, double rtol) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!(dt > 0) || nsteps < 0 || !(rtol > 0)) return set_err(c, ISKRA_EINVAL, "bad dt / nsteps / rtol");
  if (nsteps == 0) return ISKRA_OK;
  int rc = poisson_prepare(c);
  if (rc) return rc;
  // bring every accumulator to the consumed state the captured step expects
  bool stale = false;
  for (auto &s : c->species) stale |= s.acc_valid || !s.n_valid;
  if (stale) {
    rc = launch_charge_density(c);
    if (rc) return rc;
  }
  if (c->d_step_known != c->step) {
    c->d_step_host = c->step;
    ISKRA_CUDA(c, cudaMemcpyAsync(c->d_step, &c->d_step_host, sizeof(c->d_step_host), cudaMemcpyHostToDevice,
                                  c->stream));
  }
  c->graph_dt = dt;
  rc = poisson_set_precision(c, rtol);  // (may invalidate the captured step)
  if (rc) return rc;
  if (!c->periods_valid || c->periods_dt != dt) {
    rc = update_sort_periods(c, dt);
    if (rc) return rc;
    c->periods_dt = dt;
  }
  if (!poisson_separable(c)) {
    // eager path: CG needs host-side convergence checks
    for (int n = 0; n < nsteps; n++) {
      rc = queue_step(c, dt, seed, rtol, true);
      if (rc) return rc;
      c->step++;
      c->d_step_known = c->step;
      for (int s = 0; s < (int)c->species.size(); s++) {
        if (c->sort_period[s] > 0 && c->step % c->sort_period[s] == 0) {
          rc = launch_sort(c, s);
          if (rc) return rc;
        }
      }
    }
    return collect_device_errors(c);
  }
  if (c->graph && (c->graph_rtol != rtol || c->graph_seed != seed || c->graph_dt != dt)) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  if (!c->graph) {
    rc = capture(c, &c->graph, &c->graph_kernels, [&]() { return queue_step(c, dt, seed, rtol, false); });
    if (rc) return rc;
    c->graph_rtol = rtol;
    c->graph_seed = seed;
    c->graph_dt = dt;
    // the host flags now describe the state one replay leaves
    c->g_rho64 = c->rho64_valid;
    c->g_rho_df = c->rho_df_valid;
    for (int s = 0; s < (int)c->species.size(); s++) {
      c->g_n64[s] = c->species[s].n64_valid;
      c->g_n_df[s] = c->species[s].n_df_valid;
    }
  }
  for (int s = 0; s < (int)c->species.size(); s++) {
    if (!c->sort_graph[s] && c->sort_period[s] > 0) {
      rc = capture(c, &c->sort_graph[s], &c->sort_graph_kernels[s], [&]() { return launch_sort(c, s); });
      if (rc) return rc;
    }
  }
  c->rho64_valid = c->g_rho64;
  c->rho_df_valid = c->g_rho_df;
  for (int s = 0; s < (int)c->species.size(); s++) {
    c->species[s].n64_valid = c->g_n64[s];
    c->species[s].n_df_valid = c->g_n_df[s];
  }
  for (int n = 0; n < nsteps; n++) {
    ISKRA_CUDA(c, cudaGraphLaunch(c->graph, c->stream));
    c->launches += c->graph_kernels;
    c->e_from_phi = true;
    poisson_mark_x_stale(c);
    c->step++;
    c->d_step_known = c->step;
    for (int s = 0; s < (int)c->species.size(); s++) {
      if (c->sort_period[s] > 0 && c->step % c->sort_period[s] == 0) {
        ISKRA_CUDA(c, cudaGraphLaunch(c->sort_graph[s], c->stream));
        c->launches += c->sort_graph_kernels[s];
      }
    }
  }
  return ISKRA_OK;
}

// Sort-cadence autotuner: runs `trial` steps of the caller's own simulation
// under each factor on the speed-based sort periods (0.5, 1, 2, 4), each trial
// after a sort of every species so that all start from the same order, timed
// with CUDA events on the library stream, and keeps the fastest factor.  The
// sort is a permutation and every per-step result is order-independent, so
// the trials change the run's speed, not its physics.
int iskra_autotune_sort(iskra_ctx *h, double dt, int trial, uint64_t seed, double rtol, double *scale_out,
                        double *ms_out) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (trial < 1) return set_err(c, ISKRA_EINVAL, "trial steps must be >= 1");
  if (c->sort_every >= 0) return set_err(c, ISKRA_EINVAL, "autotuning needs the automatic sort cadence");
  const double factors[] = {0.5, 1.0, 2.0, 4.0};
  double best = 0, best_ms = 0;
  cudaEvent_t e0, e1;
  ISKRA_CUDA(c, cudaEventCreate(&e0));
  ISKRA_CUDA(c, cudaEventCreate(&e1));
  int rc = ISKRA_OK;
  for (double f : factors) {
    c->sort_scale = f;
    c->periods_valid = false;
    for (int s = 0; s < (int)c->species.size() && !rc; s++) rc = launch_sort(c, s);
    if (!rc) rc = iskra_step(h, dt, 1, seed, rtol);  // periods, graphs
    if (rc) break;
    cudaEventRecord(e0, c->stream);
    rc = iskra_step(h, dt, trial, seed, rtol);
    if (rc) break;
    cudaEventRecord(e1, c->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = set_err(c, ISKRA_ECUDA, "autotune timing");
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double per = ms / trial;
    if (best == 0 || per < best_ms) {
      best = f;
      best_ms = per;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  c->sort_scale = best;
  c->periods_valid = false;
  if (scale_out) *scale_out = best;
  if (ms_out) *ms_out = best_ms;
  return collect_device_errors(c);
}

int iskra_set_tile(iskra_ctx *h, int cells) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  const int ts = cells == 8 ? 3 : cells == 16 ? 4 : cells == 32 ? 5 : -1;
  if (ts < 0) return set_err(c, ISKRA_EINVAL, "tile size must be 8, 16 or 32 cells");
  const int rc = set_tile_shift(c, ts);
  if (rc) return rc;
  return collect_device_errors(c);
}

int iskra_get_tile(iskra_ctx *h, int *cells) {
  if (!h || !cells) return ISKRA_EINVAL;
  *cells = 1 << h->c.tile_shift;
  return ISKRA_OK;
}

// Autotuner of the push tile size and the sort cadence: `trial` steps of the
// caller's own simulation per candidate (tiles of 8, 16 and 32 cells x the
// factors 0.5, 1, 2, 4 on the speed-based sort periods), each after a sort of
// every species, timed with CUDA events on the library stream; the fastest
// pair is kept.  Tile size and cadence only decide which block pushes a
// particle and in which order particles sit in memory; every per-particle
// result and the integer deposit are independent of both.  The choice is
// cached for the process by (grid, species, particles per cell, tracker):
// a later context of the same shape takes it without trials.
namespace {
struct TuneKey {
  int nx, ny, ns, ppc_log2, trk;
  bool operator<(const TuneKey &o) const {
    return std::tie(nx, ny, ns, ppc_log2, trk) < std::tie(o.nx, o.ny, o.ns, o.ppc_log2, o.trk);
  }
};
struct TuneVal {
  int ts;
  double scale, ms;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune_cache;
}  // namespace

int iskra_autotune(iskra_ctx *h, double dt, int trial, uint64_t seed, double rtol, int *tile_out, double *scale_out,
                   double *ms_out, double *ms_all, int *cached) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (trial < 1) return set_err(c, ISKRA_EINVAL, "trial steps must be >= 1");
  if (c->sort_every >= 0) return set_err(c, ISKRA_EINVAL, "autotuning needs the automatic sort cadence");
  long long np = 0;
  for (int s = 0; s < (int)c->species.size(); s++) {
    long long n = 0;
    ISKRA_CUDA(c, cudaMemcpyAsync(&n, &c->species[s].dev.st->np, sizeof(long long), cudaMemcpyDeviceToHost,
                                  c->stream));
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
    np += n;
  }
  const double ppc = (double)np / std::max(1, (c->nx - 1) * (c->ny - 1));
  const TuneKey key{c->nx, c->ny, (int)c->species.size(), ppc > 1 ? (int)std::lround(std::log2(ppc)) : 0,
                    c->trk ? 1 : 0};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      int rc = set_tile_shift(c, it->second.ts);
      if (rc) return rc;
      c->sort_scale = it->second.scale;
      c->periods_valid = false;
      if (tile_out) *tile_out = 1 << it->second.ts;
      if (scale_out) *scale_out = it->second.scale;
      if (ms_out) *ms_out = it->second.ms;
      if (cached) *cached = 1;
      return collect_device_errors(c);
    }
  }
  const double factors[] = {0.5, 1.0, 2.0, 4.0};
  double best_ms = 0, best_f = 1.0;
  int best_ts = c->tile_shift;
  cudaEvent_t e0, e1;
  ISKRA_CUDA(c, cudaEventCreate(&e0));
  ISKRA_CUDA(c, cudaEventCreate(&e1));
  int rc = ISKRA_OK, k = 0;
  for (int ts = kTileShiftMin; ts <= kTileShiftMax && !rc; ts++) {
    rc = set_tile_shift(c, ts);
    for (double f : factors) {
      if (rc) break;
      c->sort_scale = f;
      c->periods_valid = false;
      for (int s = 0; s < (int)c->species.size() && !rc; s++) rc = launch_sort(c, s);
      if (!rc) rc = iskra_step(h, dt, 1, seed, rtol);  // periods, graphs
      if (rc) break;
      cudaEventRecord(e0, c->stream);
      rc = iskra_step(h, dt, trial, seed, rtol);
      if (rc) break;
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = set_err(c, ISKRA_ECUDA, "autotune timing");
        break;
      }
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      const double per = ms / trial;
      if (ms_all) ms_all[k] = per;
      k++;
      if (best_ms == 0 || per < best_ms) {
        best_ms = per;
        best_f = f;
        best_ts = ts;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  rc = set_tile_shift(c, best_ts);
  if (rc) return rc;
  c->sort_scale = best_f;
  c->periods_valid = false;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = TuneVal{best_ts, best_f, best_ms};
  }
  if (tile_out) *tile_out = 1 << best_ts;
  if (scale_out) *scale_out = best_f;
  if (ms_out) *ms_out = best_ms;
  if (cached) *cached = 0;
  return collect_device_errors(c);
}

int iskra_kernel_launches(iskra_ctx *h, uint64_t *count) {
  if (!h || !count) return ISKRA_EINVAL;
  *count = h->c.launches;
  return ISKRA_OK;
}

}  // extern "C"
