// ctx.cu -- context, species store, host<->device conversion, error plumbing.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "internal.cuh"

namespace iskra {

int set_err(Ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_check(Ctx *c, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return ISKRA_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return set_err(c, ISKRA_ENOMEM, m);
  return set_err(c, ISKRA_ECUDA, m);
}

int grid_blocks(Ctx *c, int threads, int per_sm) {
  (void)threads;
  return c->num_sms * per_sm;
}

void set_tile_shift_geometry(Ctx *c, int ts) {
  c->tile_shift = ts;
  tile_geometry(c->nx, c->ny, ts, c->tiles_x, c->tiles_y);
  c->ntiles = c->tiles_x * c->tiles_y;
  c->nkeys = c->ntiles << (2 * ts);
}

void invalidate_graphs(Ctx *c) {
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  for (auto &g : c->sort_graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  c->periods_valid = false;
}

int collect_device_errors(Ctx *c) {
  if (c->dl_pending) {  // a synchronising call also completes the non-blocking downloads
    ISKRA_CUDA(c, cudaStreamSynchronize(c->dl_stream));
    c->dl_pending = false;
  }
  ISKRA_CUDA(c, cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  int f = *c->h_err;
  if (!f) return ISKRA_OK;
  ISKRA_CUDA(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (f & DERR_NAN) return set_err(c, ISKRA_ENAN, "non-finite particle or field value");
  if (f & DERR_PROB)
    return set_err(c, ISKRA_EPROB, "MCC collision probability above its bound (mcc.jl:244-246,272-279)");
  if (f & DERR_CAPACITY) return set_err(c, ISKRA_ECAPACITY, "species capacity exceeded; particles dropped");
  if (f & DERR_DOMAIN)
    return set_err(c, ISKRA_EDOMAIN, "particle outside the grid on an axis without wrap!/discard!");
  if (f & DERR_TIMEOUT) return set_err(c, ISKRA_ETIMEDOUT, "bounded device wait gave up");
  if (f & DERR_NOTCONV) return set_err(c, ISKRA_ENOTCONV, "Poisson solve did not reach the tolerance");
  if (f & DERR_OVERFLOW)
    return set_err(c, ISKRA_ECAPACITY, "deposit: more than 16383 macroparticles in one cell (int64 node sums could wrap)");
  return set_err(c, ISKRA_ECUDA, "unknown device error flag");
}

// ---------------------------------------------------------------------------
// upload / download conversion kernels
// ---------------------------------------------------------------------------
// Particle columns of a host array in Julia layout (x, y, vx, vy, vz), each
// either a device staging copy or the page-locked host array itself, which
// the kernel reads or writes over NVLink-C2C (no staging pass).
struct Cols5 {
  const double *c[5];
};
struct OutCols5 {
  double *c[5];
};

// particle_cell (ParticleInCell.jl:28-35) on the upload side: f = 1 + x/Δh,
// i = floor(f), h = f - i, quantised by cell_of_position.  next_id (when
// given) receives max(id) + 1 of the uploaded identifiers (one atomic per
// warp).  Each thread converts kConvIlp particles and issues all their loads
// first: read straight from host memory, the loads cross NVLink-C2C with
// microseconds of latency, and the bytes in flight set the rate.
constexpr int kConvIlp = 4;

__global__ void __launch_bounds__(256) k_upload(Cols5 in, long long np, double dx, double dy, int nx, int ny,
                                                const uint32_t *__restrict__ ids, float4 *xv, float2 *zc,
                                                uint32_t *id, int *err, unsigned *next_id) {
  const long long base = (long long)blockIdx.x * blockDim.x * kConvIlp + threadIdx.x;
  double X[kConvIlp], Y[kConvIlp], VX[kConvIlp], VY[kConvIlp], VZ[kConvIlp];
  uint32_t I[kConvIlp];
#pragma unroll
  for (int u = 0; u < kConvIlp; u++) {
    const long long p = base + (long long)u * blockDim.x;
    if (p < np) {
      X[u] = in.c[0][p];
      Y[u] = in.c[1][p];
      VX[u] = in.c[2][p];
      VY[u] = in.c[3][p];
      VZ[u] = in.c[4][p];
      I[u] = ids ? ids[p] : (uint32_t)(p + 1);
    }
  }
  unsigned mx = 0;
  int flags = 0;
#pragma unroll
  for (int u = 0; u < kConvIlp; u++) {
    const long long p = base + (long long)u * blockDim.x;
    if (p >= np) continue;
    long long ux, uy;
    const int c = cell_of_position(X[u], Y[u], dx, dy, nx, ny, ux, uy);
    int cell = -1;
    const bool finite = isfinite(X[u]) && isfinite(Y[u]) && isfinite(VX[u]) && isfinite(VY[u]) && isfinite(VZ[u]);
    if (!finite) flags |= DERR_NAN;
    else if (c < 0) flags |= DERR_DOMAIN;
    else cell = c;
    xv[p] = make_float4((float)ux * kOffInv, (float)uy * kOffInv, (float)VX[u], (float)VY[u]);
    zc[p] = make_float2((float)VZ[u], __int_as_float(cell));
    id[p] = I[u];
    mx = max(mx, I[u] + 1u);
  }
  if (flags) atomicOr(err, flags);
  if (next_id && ids) {
    const unsigned m = __reduce_max_sync(0xffffffffu, mx);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(next_id, m);
  }
}

__global__ void k_download(OutCols5 out, long long np, double dx, double dy, const float4 *__restrict__ xv,
                           const float2 *__restrict__ zc, const uint32_t *__restrict__ idd,
                           uint32_t *__restrict__ id_out) {
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= np) return;
  float4 a = xv[p];
  float2 b = zc[p];
  int cell = __float_as_int(b.y);
  int i0 = cell & 0xffff, j0 = cell >> 16;
  if (out.c[0]) {
    out.c[0][p] = ((double)i0 + (double)a.x) * dx;
    out.c[1][p] = ((double)j0 + (double)a.y) * dy;
  }
  if (out.c[2]) {
    out.c[2][p] = a.z;
    out.c[3][p] = a.w;
    out.c[4][p] = b.x;
  }
  if (id_out) id_out[p] = idd[p];
}

__global__ void k_upload_E(const double *__restrict__ E, int nx, int ny, float2 *E32, double *E64) {
  const int nn = nx * ny;
  int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  double ex = E[n], ey = E[n + nn], ez = E[n + 2 * nn];
  E32[n] = make_float2((float)ex, (float)ey);
  E64[n] = ex;
  E64[n + nn] = ey;
  E64[n + 2 * nn] = ez;
}

static int ensure_stage(Ctx *c, size_t bytes) {
  if (c->stage_bytes >= bytes) return ISKRA_OK;
  if (c->stage) cudaFree(c->stage);
  c->stage = nullptr;
  c->stage_bytes = 0;
  ISKRA_CUDA(c, cudaMalloc(&c->stage, bytes));
  c->stage_bytes = bytes;
  return ISKRA_OK;
}

static int check_sid(Ctx *c, int sid) {
  if (sid < 0 || sid >= (int)c->species.size()) return set_err(c, ISKRA_EINVAL, "bad species id");
  return ISKRA_OK;
}

// Device address of a host array the GPU can read and write directly
// (page-locked memory registered with CUDA: cudaHostAlloc, cudaHostRegister,
// pinned framework tensors), or nullptr (pageable memory: staged copies).
// On GB300 the kernel then moves the data over NVLink-C2C in the same pass
// that converts it, instead of a copy into a staging buffer followed by a
// conversion pass.
static const void *host_alias(const void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // unregistered pointer: not an error for the caller
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return a.devicePointer;
}

// Host particle arrays (column-major, leading dimension ld) -> one store
// segment: read directly when every array is page-locked and mapped, else
// through the context's staging buffer.  next_id (device, optional) receives
// max(id) + 1 when identifiers are given.  Synchronous: the host arrays are
// free again on return.
int upload_particles(Ctx *c, const double *x, const double *v, const uint32_t *id, int64_t np, int64_t ld,
                     float4 *xv, float2 *zc, uint32_t *idd, unsigned *next_id) {
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (np <= 0) return collect_device_errors(c);
  const double *hx = (const double *)host_alias(x), *hv = (const double *)host_alias(v);
  const uint32_t *hid = id ? (const uint32_t *)host_alias(id) : nullptr;
  Cols5 in{};
  const uint32_t *ids = nullptr;
  if (hx && hv && (!id || hid)) {
    for (int k = 0; k < 2; k++) in.c[k] = hx + k * ld;
    for (int k = 0; k < 3; k++) in.c[2 + k] = hv + k * ld;
    ids = hid;
  } else {
    int rc = ensure_stage(c, (size_t)np * (5 * sizeof(double) + sizeof(uint32_t)));
    if (rc) return rc;
    double *st = c->stage;
    for (int k = 0; k < 2; k++)
      ISKRA_CUDA(c, cudaMemcpyAsync(st + k * np, x + k * ld, np * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    for (int k = 0; k < 3; k++)
      ISKRA_CUDA(c, cudaMemcpyAsync(st + (2 + k) * np, v + k * ld, np * sizeof(double), cudaMemcpyHostToDevice,
                                    c->stream));
    if (id) {
      uint32_t *sid = (uint32_t *)(st + 5 * np);
      ISKRA_CUDA(c, cudaMemcpyAsync(sid, id, np * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
      ids = sid;
    }
    for (int k = 0; k < 5; k++) in.c[k] = st + k * np;
  }
  const long long B = (np + 256 * kConvIlp - 1) / (256 * kConvIlp);
  k_upload<<<(unsigned)B, 256, 0, c->stream>>>(in, np, c->g.dx, c->g.dy, c->nx, c->ny, ids, xv, zc, idd, c->d_err,
                                               next_id);
  ISKRA_CUDA(c, cudaGetLastError());
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  return collect_device_errors(c);
}

// One store segment (np live particles, no holes) -> host arrays (x, v, id
// each optional): written directly when page-locked and mapped, else through
// the staging buffer; synchronous.
int download_particles(Ctx *c, const float4 *xv, const float2 *zc, const uint32_t *idd, long long np, double *x,
                       double *v, uint32_t *id, int64_t ld) {
  if (np == 0) return ISKRA_OK;
  double *hx = x ? (double *)host_alias(x) : nullptr, *hv = v ? (double *)host_alias(v) : nullptr;
  uint32_t *hid = id ? (uint32_t *)host_alias(id) : nullptr;
  const bool direct = (!x || hx) && (!v || hv) && (!id || hid);
  OutCols5 out{};
  if (direct) {
    for (int k = 0; k < 2 && hx; k++) out.c[k] = hx + k * ld;
    for (int k = 0; k < 3 && hv; k++) out.c[2 + k] = hv + k * ld;
  } else {
    int rc = ensure_stage(c, (size_t)np * 5 * sizeof(double));
    if (rc) return rc;
    for (int k = 0; k < 5; k++) out.c[k] = c->stage + k * np;
  }
  const long long B = (np + 255) / 256;
  k_download<<<(unsigned)B, 256, 0, c->stream>>>(out, np, c->g.dx, c->g.dy, xv, zc, idd, direct ? hid : nullptr);
  ISKRA_CUDA(c, cudaGetLastError());
  if (!direct) {
    for (int k = 0; k < 2 && x; k++)
      ISKRA_CUDA(c, cudaMemcpyAsync(x + k * ld, c->stage + k * np, np * sizeof(double), cudaMemcpyDeviceToHost,
                                    c->stream));
    for (int k = 0; k < 3 && v; k++)
      ISKRA_CUDA(c, cudaMemcpyAsync(v + k * ld, c->stage + (2 + k) * np, np * sizeof(double), cudaMemcpyDeviceToHost,
                                    c->stream));
    if (id) ISKRA_CUDA(c, cudaMemcpyAsync(id, idd, np * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  }
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  return ISKRA_OK;
}

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_ctx_create(const iskra_grid_t *g, uint64_t stream, iskra_ctx **out) {
  if (!g || !out) return ISKRA_EINVAL;
  *out = nullptr;
  // a particle's cell is packed as i0 | j0 << 16 in a non-negative int
  if (g->nx < 2 || g->ny < 2 || g->nx > 65535 || g->ny > 32768 || !(g->dx > 0) || !(g->dy > 0))
    return ISKRA_EINVAL;
  if ((long long)g->nx * g->ny > (1LL << 30)) return ISKRA_EINVAL;
  if (g->ox != 0.0 || g->oy != 0.0) return ISKRA_EINVAL;
  iskra_ctx *h = new (std::nothrow) iskra_ctx();
  if (!h) return ISKRA_ENOMEM;
  Ctx *c = &h->c;
  c->g = *g;
  c->nx = g->nx;
  c->ny = g->ny;
  c->nn = g->nx * g->ny;
  for (int ts = kTileShiftMin; ts <= kTileShiftMax; ts++) {  // buffers fit every tile size
    int tx, ty;
    tile_geometry(g->nx, g->ny, ts, tx, ty);
    c->ntiles_cap = std::max(c->ntiles_cap, tx * ty);
    c->nkeys_cap = std::max(c->nkeys_cap, (tx * ty) << (2 * ts));
  }
  set_tile_shift_geometry(c, kTileShiftDefault);
  auto fail = [&](int rc) {
    iskra_ctx_destroy(h);
    return rc;
  };
  if (cudaGetDevice(&c->device) != cudaSuccess) return fail(ISKRA_ECUDA);
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess)
    return fail(ISKRA_ECUDA);
  if (stream) {
    c->stream = (cudaStream_t)(uintptr_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(ISKRA_ECUDA);
    c->own_stream = true;
  }
  size_t nn = (size_t)c->nn;
  bool ok = cudaMalloc(&c->E32, nn * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&c->E64, nn * 3 * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&c->rho, nn * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&c->vol_inv, nn * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&c->rho_df, nn * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&c->vol_inv_df, nn * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&c->d_err, sizeof(int)) == cudaSuccess &&
            cudaMallocHost(&c->h_err, sizeof(int)) == cudaSuccess &&
            cudaMalloc(&c->cell_count, ((size_t)c->nkeys_cap + 1) * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&c->cell_cursor, ((size_t)c->nkeys_cap + 1) * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&c->scan_tmp, ((size_t)c->nkeys_cap / 4096 + 2) * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&c->d_step, sizeof(unsigned long long)) == cudaSuccess &&
            cudaMalloc(&c->d_scratch, 16 * sizeof(double)) == cudaSuccess;
  if (!ok) return fail(ISKRA_ENOMEM);
  cudaMemsetAsync(c->E32, 0, nn * sizeof(float2), c->stream);
  cudaMemsetAsync(c->E64, 0, nn * 3 * sizeof(double), c->stream);
  cudaMemsetAsync(c->rho, 0, nn * sizeof(double), c->stream);
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  cudaMemsetAsync(c->d_step, 0, sizeof(unsigned long long), c->stream);
  // 1/cell_volume (RegularGrids.jl:26-38)
  std::vector<double> vinv(nn);
  double V0 = g->dx * g->dy;
  for (int j = 0; j < c->ny; j++)
    for (int i = 0; i < c->nx; i++) {
      double V = 0.0 + V0;
      if (i == 0 && !g->bc[0]) V *= 0.5;
      if (i == c->nx - 1 && !g->bc[1]) V *= 0.5;
      if (j == 0 && !g->bc[2]) V *= 0.5;
      if (j == c->ny - 1 && !g->bc[3]) V *= 0.5;
      vinv[(size_t)i + (size_t)c->nx * j] = 1.0 / V;
    }
  if (cudaMemcpyAsync(c->vol_inv, vinv.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->stream) !=
      cudaSuccess)
    return fail(ISKRA_ECUDA);
  std::vector<float2> vinv_df(nn);
  for (size_t k = 0; k < nn; k++) vinv_df[k] = df_host(vinv[k]);
  if (cudaMemcpyAsync(c->vol_inv_df, vinv_df.data(), nn * sizeof(float2), cudaMemcpyHostToDevice, c->stream) !=
      cudaSuccess)
    return fail(ISKRA_ECUDA);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(ISKRA_ECUDA);
  *out = h;
  return ISKRA_OK;
}

int iskra_ctx_destroy(iskra_ctx *h) {
  if (!h) return ISKRA_OK;
  Ctx *c = &h->c;
  if (c->stream) cudaStreamSynchronize(c->stream);
  ensembles_detach(c);  // ensembles built on this template lose their device state
  lws_destroy_ctx(c);
  tracker_destroy(c);
  sources_destroy(c);
  dsmc_destroy(c);
  invalidate_graphs(c);
  for (auto &s : c->species) {
    for (int b = 0; b < 2; b++) {
      cudaFree(s.dev.xv[b]);
      cudaFree(s.dev.zc[b]);
      cudaFree(s.dev.id[b]);
    }
    cudaFree(s.dev.st);
    cudaFree(s.dev.acc);
    cudaFree(s.dev.cnt);
    cudaFree(s.dev.tile_begin);
    cudaFree(s.dview);
    cudaFree(s.n);
    cudaFree(s.n_df);
  }
  for (auto *m : c->mccs) mcc_destroy(m);
  if (c->ps) poisson_destroy(c->ps);
  cudaFree(c->cir_d);
  cudaFree(c->cir_seen);
  cudaFree(c->E32);
  cudaFree(c->E64);
  cudaFree(c->rho);
  cudaFree(c->rho_bg);
  cudaFree(c->vol_inv);
  cudaFree(c->rho_df);
  cudaFree(c->vol_inv_df);
  cudaFree(c->bg_df);
  cudaFree(c->d_err);
  if (c->h_err) cudaFreeHost(c->h_err);
  cudaFree(c->cell_count);
  cudaFree(c->cell_cursor);
  cudaFree(c->scan_tmp);
  cudaFree(c->stage);
  if (c->dl_stream) cudaStreamSynchronize(c->dl_stream);
  if (c->dl_ready) cudaEventDestroy(c->dl_ready);
  for (int b = 0; b < 2; b++)
    if (c->dl_done[b]) cudaEventDestroy(c->dl_done[b]);
  if (c->dl_stream) cudaStreamDestroy(c->dl_stream);
  cudaFree(c->dl_stage);
  cudaFree(c->d_step);
  cudaFree(c->d_scratch);
  cudaFree(c->mcc_work);
  cudaFree(c->mcc_nwork);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete h;
  return ISKRA_OK;
}

const char *iskra_last_error(const iskra_ctx *h) { return h ? h->c.err.c_str() : "null context"; }

int iskra_sync(iskra_ctx *h) {
  if (!h) return ISKRA_EINVAL;
  return collect_device_errors(&h->c);
}

int iskra_stream(iskra_ctx *h, uint64_t *s) {
  if (!h || !s) return ISKRA_EINVAL;
  *s = (uint64_t)(uintptr_t)h->c.stream;
  return ISKRA_OK;
}

int iskra_species_create(iskra_ctx *h, double q, double m, double w0, int64_t cap, int *sid) {
  if (!h || !sid) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if ((int)c->species.size() >= kMaxSpecies) return set_err(c, ISKRA_EINVAL, "too many species");
  if (cap < 1 || cap > (1LL << 31) - 1) return set_err(c, ISKRA_EINVAL, "capacity out of range");
  if (!(m > 0) || !(w0 > 0) || !std::isfinite(q)) return set_err(c, ISKRA_EINVAL, "bad q/m/w0");
  Species s;
  s.q = q;
  s.m = m;
  s.w0 = w0;
  s.cap = cap;
  s.dev.cap = cap;
  size_t nn = (size_t)c->nn;
  for (int b = 0; b < 2; b++) {
    // kStorePad slots past the capacity: the push's bulk copies read whole
    // 32-record stages (and the 16-byte-aligned record below a stage)
    ISKRA_CUDA(c, cudaMalloc(&s.dev.xv[b], (cap + kStorePad) * sizeof(float4)));
    ISKRA_CUDA(c, cudaMalloc(&s.dev.zc[b], (cap + kStorePad) * sizeof(float2)));
    ISKRA_CUDA(c, cudaMalloc(&s.dev.id[b], cap * sizeof(uint32_t)));
  }
  ISKRA_CUDA(c, cudaMalloc(&s.dev.st, sizeof(SpeciesState)));
  ISKRA_CUDA(c, cudaMalloc(&s.dev.acc, nn * sizeof(unsigned long long)));
  ISKRA_CUDA(c, cudaMalloc(&s.dev.cnt, nn * sizeof(unsigned)));
  ISKRA_CUDA(c, cudaMalloc(&s.dev.tile_begin, ((size_t)c->ntiles_cap + 1) * sizeof(int)));
  ISKRA_CUDA(c, cudaMalloc(&s.dview, sizeof(SpeciesDev)));
  ISKRA_CUDA(c, cudaMemsetAsync(s.dev.tile_begin, 0, ((size_t)c->ntiles_cap + 1) * sizeof(int), c->stream));
  ISKRA_CUDA(c, cudaMalloc(&s.n, nn * sizeof(double)));
  ISKRA_CUDA(c, cudaMalloc(&s.n_df, nn * sizeof(float2)));
  ISKRA_CUDA(c, cudaMemsetAsync(s.dev.st, 0, sizeof(SpeciesState), c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(s.dev.acc, 0, nn * sizeof(unsigned long long), c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(s.dev.cnt, 0, nn * sizeof(unsigned), c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(s.n, 0, nn * sizeof(double), c->stream));
  ISKRA_CUDA(c, cudaMemcpyAsync(s.dview, &s.dev, sizeof(SpeciesDev), cudaMemcpyHostToDevice, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  s.acc_valid = false;
  s.acc_zero = true;
  s.n_valid = true;  // empty species: zero density is current
  c->species.push_back(s);
  *sid = (int)c->species.size() - 1;
  invalidate_graphs(c);
  return ensure_mcc_work(c);
}

int iskra_species_set_boundary(iskra_ctx *h, int sid, int mx, int my) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (check_sid(c, sid)) return ISKRA_EINVAL;
  if (mx < 0 || mx > 2 || my < 0 || my > 2) return set_err(c, ISKRA_EINVAL, "bad boundary mode");
  c->species[sid].bnd[0] = mx;
  c->species[sid].bnd[1] = my;
  invalidate_graphs(c);
  return ISKRA_OK;
}

int iskra_species_upload(iskra_ctx *h, int sid, const double *x, const double *v, const double *wg,
                         const uint32_t *id, int64_t np, int64_t ld) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (check_sid(c, sid)) return ISKRA_EINVAL;
  Species &s = c->species[sid];
  if (np < 0 || np > s.cap) return set_err(c, ISKRA_ECAPACITY, "np exceeds species capacity");
  if (np > 0 && (!x || !v || ld < np)) return set_err(c, ISKRA_EINVAL, "bad particle arrays");
  if (wg) {
    for (int64_t p = 0; p < np; p++)
      if (wg[p] != s.w0)
        return set_err(c, ISKRA_EINVAL, "per-particle weights must all equal w0 on the device store");
  }
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  SpeciesState st0{};
  st0.np = np;
  st0.cur = 0;
  st0.next_id = (uint32_t)np + 1;  // identifiers 1..np, or max(id) + 1 (raised by the upload kernel)
  ISKRA_CUDA(c, cudaMemcpyAsync(s.dev.st, &st0, sizeof(st0), cudaMemcpyHostToDevice, c->stream));
  unsigned *next_id = (unsigned *)((char *)s.dev.st + offsetof(SpeciesState, next_id));
  int rc = upload_particles(c, x, v, id, np, ld, s.dev.xv[0], s.dev.zc[0], s.dev.id[0], next_id);
  if (rc) return rc;
  rc = launch_sort(c, sid);
  if (rc) return rc;
  if (s.acc_valid) s.acc_zero = false;
  s.acc_valid = false;
  s.n_valid = false;
  return ISKRA_OK;
}

int iskra_species_download(iskra_ctx *h, int sid, double *x, double *v, double *wg, uint32_t *id, int64_t ld,
                           int64_t *np_out) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (check_sid(c, sid)) return ISKRA_EINVAL;
  Species &s = c->species[sid];
  int rc = launch_sort(c, sid);  // compacts discarded particles
  if (rc) return rc;
  SpeciesState st{};
  ISKRA_CUDA(c, cudaMemcpyAsync(&st, s.dev.st, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  rc = collect_device_errors(c);
  if (rc) return rc;
  long long np = st.np;
  if (np_out) *np_out = np;
  if (np > ld) return set_err(c, ISKRA_ECAPACITY, "host arrays too small for the live particles");
  if (np == 0) return ISKRA_OK;
  rc = download_particles(c, s.dev.xv[st.cur], s.dev.zc[st.cur], s.dev.id[st.cur], np, x, v, id, ld);
  if (rc) return rc;
  if (wg)
    for (long long p = 0; p < np; p++) wg[p] = s.w0;
  return ISKRA_OK;
}

int iskra_species_count(iskra_ctx *h, int sid, int64_t *np) {
  if (!h || !np) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (check_sid(c, sid)) return ISKRA_EINVAL;
  int rc = launch_sort(c, sid);
  if (rc) return rc;
  SpeciesState st{};
  ISKRA_CUDA(c, cudaMemcpyAsync(&st, c->species[sid].dev.st, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  *np = st.np;
  return collect_device_errors(c);
}

int iskra_species_absorbed(iskra_ctx *h, int sid, int64_t counts[4]) {
  if (!h || !counts) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (check_sid(c, sid)) return ISKRA_EINVAL;
  SpeciesState st{};
  SpeciesState *d = c->species[sid].dev.st;
  ISKRA_CUDA(c, cudaMemcpyAsync(&st, d, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaMemsetAsync(&d->absorbed[0], 0, sizeof(st.absorbed), c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 4; k++) counts[k] = (int64_t)st.absorbed[k];
  return collect_device_errors(c);
}

int iskra_species_sort(iskra_ctx *h, int sid) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (check_sid(c, sid)) return ISKRA_EINVAL;
  return launch_sort(c, sid);
}

int iskra_field_upload_E(iskra_ctx *h, const double *E) {
  if (!h || !E) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  int rc = ensure_stage(c, (size_t)c->nn * 3 * sizeof(double));
  if (rc) return rc;
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpyAsync(c->stage, E, (size_t)c->nn * 3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  k_upload_E<<<(c->nn + 255) / 256, 256, 0, c->stream>>>(c->stage, c->nx, c->ny, c->E32, c->E64);
  c->e_from_phi = false;
  ISKRA_CUDA(c, cudaGetLastError());
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  return ISKRA_OK;
}

int iskra_set_background(iskra_ctx *h, const double *rho_bg) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!rho_bg) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->rho_bg);
    cudaFree(c->bg_df);
    c->rho_bg = nullptr;
    c->bg_df = nullptr;
  } else {
    if (!c->rho_bg) ISKRA_CUDA(c, cudaMalloc(&c->rho_bg, (size_t)c->nn * sizeof(double)));
    if (!c->bg_df) ISKRA_CUDA(c, cudaMalloc(&c->bg_df, (size_t)c->nn * sizeof(float2)));
    std::vector<float2> bdf(c->nn);
    for (int k = 0; k < c->nn; k++) bdf[k] = df_host(rho_bg[k]);
    ISKRA_CUDA(c, cudaMemcpyAsync(c->rho_bg, rho_bg, (size_t)c->nn * sizeof(double), cudaMemcpyHostToDevice,
                                  c->stream));
    ISKRA_CUDA(c, cudaMemcpyAsync(c->bg_df, bdf.data(), (size_t)c->nn * sizeof(float2), cudaMemcpyHostToDevice,
                                  c->stream));
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  invalidate_graphs(c);
  return ISKRA_OK;
}

}  // extern "C"
