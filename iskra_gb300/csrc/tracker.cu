// tracker.cu -- the surface tracker (ParticleInCell/src/pic/surfaces/*.jl and
// the electrode surfaces of circuit_coupling.jl:4-16, 45-63): the per-cell
// edge table on the device, the σ credit of floating electrodes inside the
// step, and the C API.  The walk over a particle's path (track! + check! +
// hit!) runs inside the push (track_path, particles.cu).
//
// The reference keys surfaces by ordered pairs of cells (BoundaryCells,
// build.jl:3-4) in a Dict; here every cell holds the surface behind each of
// its four edges (index + 1, one byte each), so the push looks a crossing up
// with one load.  track! (track.jl:39-52) records a particle when its cell is
// either side of some key: that set is kept as one flag byte per cell.
#include <algorithm>
#include <cstring>
#include <new>

#include "internal.cuh"

namespace iskra {

double *poisson_sigma_prepared(Ctx *c);

struct SurfaceChargeArgs {
  const unsigned long long *hits;  // [kMaxSpecies][kMaxSurfaces]
  unsigned long long *seen;
  double *sigma;
  int ns, nsurf;
  double qw[kMaxSpecies];         // q * w0 per species
  int dof[kMaxSurfaces];          // 0-based σ dof, -1: not a floating electrode
  double area[kMaxSurfaces];
};

// hit!(::FloatingPotentialElectrode, ...) (circuit_coupling.jl:45-55): each
// absorbed particle adds q w / area to the electrode's σ.  The push counts
// the hits; this kernel, queued after it and before the field solve, credits
// the ones not credited yet.  Thread f: surface f; FP64.
__global__ void k_surface_charge(SurfaceChargeArgs A) {
  pdl_wait();
  const int f = threadIdx.x;
  if (f >= A.nsurf || A.dof[f] < 0) return;
  double dq = 0.0;
  for (int s = 0; s < A.ns; s++) {
    const unsigned long long now = A.hits[s * kMaxSurfaces + f];
    const unsigned long long d = now - A.seen[s * kMaxSurfaces + f];
    A.seen[s * kMaxSurfaces + f] = now;
    dq += A.qw[s] * (double)d;
  }
  if (dq != 0.0) atomicAdd(&A.sigma[A.dof[f]], dq / A.area[f]);
}

int launch_surface_charge(Ctx *c) {
  Tracker *t = c->trk;
  if (!t || !t->any_floating) return ISKRA_OK;
  SurfaceChargeArgs A{};
  A.hits = t->d_hits;
  A.seen = t->d_seen;
  A.sigma = poisson_sigma_prepared(c);
  if (!A.sigma) return set_err(c, ISKRA_EINVAL, "floating electrode without a Poisson σ dof");
  A.ns = (int)c->species.size();
  A.nsurf = (int)t->kind.size();
  for (int s = 0; s < A.ns; s++) A.qw[s] = c->species[s].q * c->species[s].w0;
  for (int f = 0; f < A.nsurf; f++) {
    A.dof[f] = t->kind[f] == ISKRA_SURF_FLOATING ? t->sigma_dof[f] : -1;
    A.area[f] = t->area[f];
  }
  ISKRA_CUDA(c, launch_pdl(k_surface_charge, 1, kMaxSurfaces, 0, c->stream, A));
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

void tracker_destroy(Ctx *c) {
  Tracker *t = c->trk;
  if (!t) return;
  cudaFree(t->d_edge);
  cudaFree(t->d_cell);
  cudaFree(t->d_kind);
  cudaFree(t->d_hits);
  cudaFree(t->d_seen);
  delete t;
  c->trk = nullptr;
}

static int tracker_upload(Ctx *c) {
  Tracker *t = c->trk;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpy(t->d_edge, t->edge.data(), t->edge.size(), cudaMemcpyHostToDevice));
  ISKRA_CUDA(c, cudaMemcpy(t->d_cell, t->cell.data(), t->cell.size(), cudaMemcpyHostToDevice));
  unsigned char kinds[kMaxSurfaces] = {};
  for (size_t f = 0; f < t->kind.size(); f++) kinds[f] = (unsigned char)t->kind[f];
  ISKRA_CUDA(c, cudaMemcpy(t->d_kind, kinds, kMaxSurfaces, cudaMemcpyHostToDevice));
  invalidate_graphs(c);  // captured pushes hold the tracker pointers (or none)
  return ISKRA_OK;
}

// one edge of 0-based cell (i, j) toward `dir` becomes surface f; both
// cells on its sides are recorded for track! (those inside the grid)
static void set_edge(Tracker *t, const Ctx *c, int i, int j, int dir, int f) {
  t->edge[4 * (size_t)(i + c->nx * j) + dir] = (unsigned char)(f + 1);
  t->cell[i + c->nx * j] = 1;
  int ni = i, nj = j;
  if (dir == kSurfDirXm) ni--;
  if (dir == kSurfDirXp) ni++;
  if (dir == kSurfDirYm) nj--;
  if (dir == kSurfDirYp) nj++;
  if (ni >= 0 && nj >= 0 && ni < c->nx - 1 && nj < c->ny - 1) t->cell[ni + c->nx * nj] = 1;
}

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_tracker_create(iskra_ctx *h, int default_kind) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (default_kind != ISKRA_SURF_ABSORB && default_kind != ISKRA_SURF_REFLECT && default_kind != ISKRA_SURF_PERIODIC)
    return set_err(c, ISKRA_EINVAL, "default surface: absorbing, reflective or periodic");
  if (c->species.size() > (size_t)kMaxSpecies) return set_err(c, ISKRA_EINVAL, "too many species");
  tracker_destroy(c);
  Tracker *t = new (std::nothrow) Tracker();
  if (!t) return ISKRA_ENOMEM;
  c->trk = t;
  t->edge.assign(4 * (size_t)c->nn, 0);
  t->cell.assign((size_t)c->nn, 0);
  auto fail = [&](int rc) {
    tracker_destroy(c);
    return rc;
  };
  if (cudaMalloc(&t->d_edge, t->edge.size()) != cudaSuccess || cudaMalloc(&t->d_cell, t->cell.size()) != cudaSuccess ||
      cudaMalloc(&t->d_kind, kMaxSurfaces) != cudaSuccess ||
      cudaMalloc(&t->d_hits, sizeof(unsigned long long) * kMaxSpecies * kMaxSurfaces) != cudaSuccess ||
      cudaMalloc(&t->d_seen, sizeof(unsigned long long) * kMaxSpecies * kMaxSurfaces) != cudaSuccess) {
    set_err(c, ISKRA_ENOMEM, "out of device memory for the surface tracker");
    return fail(ISKRA_ENOMEM);
  }
  if (cudaMemset(t->d_hits, 0, sizeof(unsigned long long) * kMaxSpecies * kMaxSurfaces) != cudaSuccess ||
      cudaMemset(t->d_seen, 0, sizeof(unsigned long long) * kMaxSpecies * kMaxSurfaces) != cudaSuccess)
    return fail(set_err(c, ISKRA_ECUDA, "cudaMemset failed"));
  // build_default_surface! (build.jl:31-44): the walls, surface 0
  t->kind.push_back(default_kind);
  t->sigma_dof.push_back(-1);
  t->area.push_back(0.0);
  const int cx = c->nx - 1, cy = c->ny - 1;
  for (int i = 0; i < cx; i++) {
    set_edge(t, c, i, 0, kSurfDirYm, 0);
    set_edge(t, c, i, cy - 1, kSurfDirYp, 0);
  }
  for (int j = 0; j < cy; j++) {
    set_edge(t, c, 0, j, kSurfDirXm, 0);
    set_edge(t, c, cx - 1, j, kSurfDirXp, 0);
  }
  int rc = tracker_upload(c);
  if (rc) return fail(rc);
  return ISKRA_OK;
}

int iskra_tracker_add_surface(iskra_ctx *h, const uint8_t *nodes, int kind, int sigma_dof, double area,
                              int *surface) {
  if (!h || !nodes) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  Tracker *t = c->trk;
  if (!t) return set_err(c, ISKRA_EINVAL, "no surface tracker (iskra_tracker_create)");
  if (kind < ISKRA_SURF_ABSORB || kind > ISKRA_SURF_FLOATING) return set_err(c, ISKRA_EINVAL, "bad surface kind");
  if ((int)t->kind.size() >= kMaxSurfaces) return set_err(c, ISKRA_EINVAL, "too many surfaces");
  if (kind == ISKRA_SURF_FLOATING) {
    double sv = 0;
    if (sigma_dof < 1 || iskra_poisson_get_sigma(h, sigma_dof, &sv) != ISKRA_OK)
      return set_err(c, ISKRA_EINVAL, "floating electrode: bad σ dof");
    if (!(area > 0.0)) return set_err(c, ISKRA_EINVAL, "floating electrode: area must be positive");
  }
  const int f = (int)t->kind.size();
  t->kind.push_back(kind);
  t->sigma_dof.push_back(kind == ISKRA_SURF_FLOATING ? sigma_dof - 1 : -1);
  t->area.push_back(kind == ISKRA_SURF_FLOATING ? area : 0.0);
  if (kind == ISKRA_SURF_FLOATING) t->any_floating = true;
  // build_surface_lookup! (build.jl:46-60): corners a (i,j), b (i+1,j),
  // c (i+1,j+1), d (i,j+1) of each cell; an edge with both ends in the node
  // set is a surface seen from this cell
  const int nx = c->nx, cx = c->nx - 1, cy = c->ny - 1;
  for (int i = 0; i < cx; i++) {
    for (int j = 0; j < cy; j++) {
      const bool a = nodes[i + nx * j] != 0, b = nodes[i + 1 + nx * j] != 0;
      const bool cc = nodes[i + 1 + nx * (j + 1)] != 0, d = nodes[i + nx * (j + 1)] != 0;
      if (a && b) set_edge(t, c, i, j, kSurfDirYm, f);
      if (b && cc) set_edge(t, c, i, j, kSurfDirXp, f);
      if (cc && d) set_edge(t, c, i, j, kSurfDirYp, f);
      if (d && a) set_edge(t, c, i, j, kSurfDirXm, f);
    }
  }
  int rc = tracker_upload(c);
  if (rc) return rc;
  if (surface) *surface = f;
  return ISKRA_OK;
}

int iskra_tracker_hits(iskra_ctx *h, int surface, int sid, int64_t *count) {
  if (!h || !count) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  Tracker *t = c->trk;
  if (!t) return set_err(c, ISKRA_EINVAL, "no surface tracker");
  if (surface < 0 || surface >= (int)t->kind.size()) return set_err(c, ISKRA_EINVAL, "bad surface");
  if (sid < 0 || sid >= (int)c->species.size()) return set_err(c, ISKRA_EINVAL, "bad species");
  unsigned long long v = 0;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpy(&v, t->d_hits + (size_t)sid * kMaxSurfaces + surface, sizeof(v), cudaMemcpyDeviceToHost));
  *count = (int64_t)v;
  return collect_device_errors(c);
}

}  // extern "C"
