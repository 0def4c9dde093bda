// poisson.cu -- FP64 Poisson solve on the reference's assembled operator.
//
// Host side: the operator is assembled row by row exactly as
// FiniteDifferenceMethod/src/generalized_poisson.jl does it
// (create_generalized_poisson_solver :34-68, apply_dirichlet :205-215,
// add_new_dof :217-230, apply_neumann :235-269, apply_periodic :286-324),
// kept in a 7-slot row form per node: self, (i-1,j), (i+1,j), (i,j-1),
// (i,j+1), x-periodic partner, y-periodic partner; plus σ columns.
//
// Device side, per solve of A ϕ = b (b[ρ] = -ρ/ε0, b[Dirichlet] = ϕ0):
//   * rows that are identity (Dirichlet, σ) are fixed values;
//   * the remaining rows are scaled by D so that S = -D A_ff is symmetric
//     positive (semi)definite (Neumann rows of apply_neumann have a different
//     scale than stencil rows);
//   * when S separates into (tridiagonal in x) + (periodic ring in y) -- true
//     for every problem of the reference that uses apply_periodic(solver, 1)
//     with column electrodes -- it is solved exactly by a real FFT along y, one
//     tridiagonal (Thomas / Sherman-Morrison for x-periodic) solve per Fourier
//     mode along x, and an inverse FFT; the residual is then re-evaluated in
//     FP64 and the correction repeated until ||res|| <= rtol ||rhs||;
//   * otherwise Jacobi-preconditioned CG iterates to the same tolerance.
// All-periodic / all-open operators are singular; the solve then uses the
// mean-zero gauge with the right-hand side projected onto the range (the
// reference's dense A\b has no defined answer there; E = -∇ϕ is unaffected).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "internal.cuh"

namespace iskra {

struct RowClass {
  double c0, cW, cE, cS, cN;  // original (unscaled) coefficients
  double d;                   // symmetrising row scale
  double inv_d;               // 1 / d
  double sig_coef;            // coefficient of the σ column
  int sig_dof;                // -1: none
  int fixed;                  // identity row
  int rho;                    // b = -ρ/ε0 (ρ dof) else b = bfix
  float nd32;                 // -d in FP32 (scaling of the FP32 residual)
  float2 c0f, cWf, cEf, cSf, cNf;  // the coefficients as double-float pairs
};

struct DriveGroup {
  std::vector<int> nodes;
  double amp, freq, phase, dc;
};

struct PoissonScal {           // device-resident solver scalars
  double lambda;               // singular case: range projection shift
  double relres;
  double rhs2, res2;
  int iters;
  int done;
  int sweeps;
  unsigned ticket;             // blocks of the running k_residual that have finished
  double rz, rz_new, pap;
  int hist;                    // xh holds the previous step solve's ϕ (warm start)
  int e_pending;               // the first residual pass met rtol but wrote no E
  unsigned hticket;            // blocks of the running k_extrapolate that have finished
};

struct Poisson {
  // ---- host assembly (generalized_poisson.jl) ----
  int nx = 0, ny = 0, nn = 0;
  double dx = 0, dy = 0, eps0 = 0;
  std::vector<double> C;        // nn*7
  std::vector<double> bfix;     // b for non-ρ rows
  std::vector<uint8_t> rho_dof;
  std::vector<std::vector<double>> sig_cols;  // per σ dof: nn column
  std::vector<double> sig_b;
  std::vector<DriveGroup> drives;
  std::vector<double> er;       // (nx+1)*(ny+1) ones
  bool dirty = true;
  int method = 0;               // 0 auto, 1 CG (Jacobi), 2 CG with the multigrid preconditioner
  Mg *mg = nullptr;             // multigrid hierarchy of a non-separable operator (multigrid.cu)
  cudaGraphExec_t pcg_graph = nullptr;  // one multigrid-CG iteration (~70 kernels), replayed
  double pcg_graph_rtol = 0;
  // ---- device representation ----
  bool separable = false, singular = false, cyclic = false;
  int nclass = 0;
  uint16_t *cls = nullptr;      // nn
  RowClass *classes = nullptr;
  double *bfix_d = nullptr;     // nn
  double *sigma_d = nullptr;    // nsig
  int nsig = 0;
  double *x = nullptr;          // ϕ (nn); for separable operators a view refreshed from xd on demand
  float2 *xd = nullptr;         // ϕ as double-float pairs (separable operators: the solver's state)
  float2 *bd = nullptr;         // b of the free rows as double-float pairs (first residual pass)
  void *xh = nullptr;           // previous step solve's ϕ in the state's representation (8 B per node)
  int warm_mode = 1;            // step solves start from 0: ϕ_n, 1: 2 ϕ_n - ϕ_(n-1)
  bool df_mode = false;         // the solver's state is xd (double-float), x a view
  bool x_stale = false;         // (df_mode) x lags xd
  double *r = nullptr, *z = nullptr, *p = nullptr, *ap = nullptr;  // nn
  double *part = nullptr;       // reduction partials (kPartials * 4)
  PoissonScal *scal = nullptr;
  PoissonScal *scal_h = nullptr;  // pinned
  double dsum = 0;              // Σ d over free rows (singular projection)
  // separable solver
  int N = 0, K = 0, logN = 0;   // N = ny, K = N/2+1
  // (FP32 correction: factors computed in FP64 on the host, stored rounded)
  float *r32 = nullptr;         // nn scaled residual, input of the correction
  float2 *spec = nullptr;       // nx*K
  float2 *tw = nullptr;         // N/2 twiddles exp(-2πi m/N)
  float *low = nullptr, *up = nullptr;        // nx
  float *inv = nullptr, *cp = nullptr, *q = nullptr;  // nx*K
  float *gk = nullptr;          // 2K: 1/(1+v.q) and β/γ per mode (x-periodic)
  int cr_levels = 0;            // cyclic reduction: L = floor(log2 nx)
  int cr_nf = 0, cr_nb = 0;     // updated / eliminated rows over all levels
  float2 *cr_fwd = nullptr;     // (α, γ) per mode and updated row
  float2 *cr_back = nullptr;    // (a/b, c/b) per mode and eliminated row
  float *cr_backb = nullptr;    // 1/b per mode and eliminated row
  float *cr_top = nullptr;      // 1/b of the last row per mode
  int pin_k0 = -1;              // pinned column of mode 0 (singular)
  // drives on device
  int ndrive_nodes = 0;
  int *drive_node = nullptr;
  int *drive_group = nullptr;
  double *drive_par = nullptr;  // 4 per group
  int ndrive = 0;
  int blocks = 0;
  int cg_blocks = 0;            // blocks of the multigrid-PCG vector kernels (more per SM: latency bound)
  bool rho_fixed = false;       // some identity row takes its value from ρ (rewritten every solve)
  int last_iters = 0;
  double last_relres = 0;
  // FP64 Thomas factors of the separable operator (host copy; uploaded on
  // demand for the ensemble field solve)
  // FP64 cyclic-reduction coefficients of the ensemble field solve, packed:
  // fwd (K nf pairs), back (K nb pairs), backb (K nb), top (K)
  std::vector<double> cr64;
  double *cr64_d = nullptr;
};

constexpr int kPartials = 1024;
// blocks per SM of the node passes (residuals, conversions); tuned on GB300
#ifndef ISKRA_RES_BLOCKS_PER_SM
#define ISKRA_RES_BLOCKS_PER_SM 2
#endif

void poisson_destroy(Poisson *p) {
  if (!p) return;
  mg_destroy(p->mg);
  if (p->pcg_graph) cudaGraphExecDestroy(p->pcg_graph);
  cudaFree(p->cls);
  cudaFree(p->classes);
  cudaFree(p->bfix_d);
  cudaFree(p->sigma_d);
  cudaFree(p->x);
  cudaFree(p->xd);
  cudaFree(p->bd);
  cudaFree(p->xh);
  cudaFree(p->r);
  cudaFree(p->z);
  cudaFree(p->p);
  cudaFree(p->ap);
  cudaFree(p->part);
  cudaFree(p->scal);
  if (p->scal_h) cudaFreeHost(p->scal_h);
  cudaFree(p->cr64_d);
  cudaFree(p->r32);
  cudaFree(p->spec);
  cudaFree(p->tw);
  cudaFree(p->low);
  cudaFree(p->up);
  cudaFree(p->inv);
  cudaFree(p->cp);
  cudaFree(p->q);
  cudaFree(p->gk);
  cudaFree(p->cr_fwd);
  cudaFree(p->cr_back);
  cudaFree(p->cr_backb);
  cudaFree(p->cr_top);
  cudaFree(p->drive_node);
  cudaFree(p->drive_group);
  cudaFree(p->drive_par);
  delete p;
}

// ===========================================================================
// device kernels
// ===========================================================================
// cls[k] = row class id of node k, with kFixedBit set on identity (fixed) rows
constexpr unsigned kFixedBit = 0x8000u;
constexpr unsigned kClassMask = 0x7fffu;

// (double-float arithmetic: df_* in internal.cuh)

struct OpView {
  const uint16_t *cls;
  const RowClass *classes;
  const double *bfix;
  const double *sigma;
  int nx, ny;
  int nclass;
};

__device__ __forceinline__ void nbr(int k, int nx, int ny, int &w, int &e, int &s, int &n) {
  const int i = k % nx, j = k / nx;
  w = i > 0 ? k - 1 : k + nx - 1;
  e = i < nx - 1 ? k + 1 : k - nx + 1;
  s = j > 0 ? k - nx : k + nx * (ny - 1);
  n = j < ny - 1 ? k + nx : k - nx * (ny - 1);
}

__device__ __forceinline__ double drive_value(const double *par, double t) {
  return par[0] * sin(2.0 * M_PI * par[1] * t + par[2]) + par[3];
}

// fixed-row values: Dirichlet / driven
__global__ void k_set_fixed(OpView op, const int *__restrict__ dnode, const int *__restrict__ dgroup,
                            const double *__restrict__ dpar, int ndn, const unsigned long long *__restrict__ step,
                            double dt, double *__restrict__ bfix_mut, double *__restrict__ x, float2 *__restrict__ xd,
                            const double *__restrict__ rho, double eps0, int nn) {
  pdl_wait();
  // driven groups update bfix (solve of step n uses V((n-2)Δt), n >= 2)
  const unsigned long long n_step = step ? *step : 0ull;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ndn; t += gridDim.x * blockDim.x) {
    const int k = dnode[t];
    if (n_step >= 2) {
      double tt = (double)(n_step - 2) * dt;
      bfix_mut[k] = drive_value(dpar + 4 * dgroup[t], tt);
    }
    x[k] = bfix_mut[k];
    if (xd) xd[k] = df_from(bfix_mut[k]);
  }
}

__global__ void k_fixed_to_x(OpView op, double *__restrict__ x, float2 *__restrict__ xd,
                             const double *__restrict__ rho, double neg_inv_eps0, int nn) {
  pdl_wait();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const unsigned ck = op.cls[k];
    if (ck & kFixedBit) {
      const double v = op.classes[ck & kClassMask].rho ? rho[k] * neg_inv_eps0 : op.bfix[k];
      x[k] = v;
      if (xd) xd[k] = df_from(v);
    }
  }
}

// ϕ conversions between the FP64 view and the double-float state
__global__ void k_df_to_x(const float2 *__restrict__ xd, double *__restrict__ x, int nn) {
  pdl_wait();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) x[k] = df_value(xd[k]);
}
__global__ void k_x_to_df(const double *__restrict__ x, float2 *__restrict__ xd, int nn) {
  pdl_wait();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) xd[k] = df_from(x[k]);
}

// Warm start of a step's solve: the free rows of ϕ extrapolated linearly in
// time from the last two step solutions, ϕ <- 2 ϕ_n - ϕ_(n-1) (a better
// initial guess than ϕ_n while the charge moves smoothly: fewer corrections
// reach the tolerance, which is still tested on the residual); xh <- ϕ_n.
// With no valid history (sc->hist == 0) it only records ϕ_n; the last block
// to finish marks the history valid (every block has read the flag by then).
template <bool DF>
__global__ void k_extrapolate(const uint16_t *__restrict__ cls, void *__restrict__ xv, void *__restrict__ xhv,
                              int nn, PoissonScal *sc) {
  pdl_wait();
  __shared__ int last;
  const bool h = sc->hist != 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const bool upd = h && !(cls[k] & kFixedBit);
    if (DF) {
      float2 *x = (float2 *)xv, *xh = (float2 *)xhv;
      const float2 a = x[k];
      if (upd) x[k] = df_add(make_float2(2.f * a.x, 2.f * a.y), df_neg(xh[k]));
      xh[k] = a;
    } else {
      double *x = (double *)xv, *xh = (double *)xhv;
      const double a = x[k];
      if (upd) x[k] = 2.0 * a - xh[k];
      xh[k] = a;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&sc->hticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    sc->hticket = 0u;
    sc->hist = 1;
  }
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// deterministic sum of partials (every block computes the same value)
__device__ double sum_partials(const double *__restrict__ part, int n, double *sh) {
  double v = 0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) v += __ldcg(part + k);  // written by other blocks
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) sh[32] = t;
  __syncthreads();
  double r = sh[32];
  __syncthreads();
  return r;
}

// Σ d_k b_k over free rows (singular case only: no fixed rows exist)
__global__ void k_sum_db(OpView op, const double *__restrict__ rho, double neg_inv_eps0, int nn,
                         double *__restrict__ part) {
  pdl_wait();
  __shared__ double sh[40];
  double v = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const RowClass &C = op.classes[op.cls[k] & kClassMask];
    if (!C.fixed) {
      double b = C.rho ? rho[k] * neg_inv_eps0 : op.bfix[k];
      if (C.sig_dof >= 0) b -= C.sig_coef * op.sigma[C.sig_dof];
      v += C.d * b;
    }
  }
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_lambda(const double *__restrict__ part, int nparts, double dsum, PoissonScal *sc) {
  pdl_wait();
  __shared__ double sh[40];
  double s = sum_partials(part, nparts, sh);
  if (threadIdx.x == 0) sc->lambda = dsum > 0 ? s / dsum : 0.0;
}

// Optional E = -∇ϕ output of k_residual (generalized_poisson.jl:398-410):
// FP32 node values: the MCC target term and, staged per tile, the gather.
// The node differences are taken in FP64 (ϕ is ~10^2-10^3 V while neighbour
// differences are ~10^-1 V) and scaled in FP32.
struct EOut {
  float2 *E32;
  float idx2, idx1, idy2, idy1;  // 1/(2Δx), 1/Δx, 1/(2Δy), 1/Δy
};

__device__ __forceinline__ void efield_at(const double *__restrict__ x, int k, int i, int j, int nx, int ny,
                                          const EOut &eo) {
  float ex, ey;
  if (i == 0) ex = (float)(x[k] - x[k + 1]) * eo.idx1;
  else if (i == nx - 1) ex = (float)(x[k - 1] - x[k]) * eo.idx1;
  else ex = (float)(x[k - 1] - x[k + 1]) * eo.idx2;
  if (j == 0) ey = (float)(x[k] - x[k + nx]) * eo.idy1;
  else if (j == ny - 1) ey = (float)(x[k - nx] - x[k]) * eo.idy1;
  else ey = (float)(x[k - nx] - x[k + nx]) * eo.idy2;
  eo.E32[k] = make_float2(ex, ey);
}

constexpr int kSmemClasses = 128;  // row-class table held in shared memory up to this size

// res = b - λ - A x over free rows, stored scaled as r = -d * res (FP64 in
// r64 for CG, FP32 in r32 as the input of the FP32 separable correction).
// Block partials of ||res||² (and, in the FIRST pass of a solve, of
// ||rhs_eff||², rhs_eff = b - λ - A_fixed x_fixed) are summed by the last
// block to finish, in block order (deterministic), which updates
// relres/iters and sets sc->done when ||res|| <= rtol ||rhs_eff||.  With
// EOUT, E = -∇ϕ of x is written too.  Passes after the first return at once
// when sc->done is set and count one sweep each.
//
// GB300 runs FP64 at ~1/64 of the FP32 rate, so this pass is built to use few
// FP64 instructions: the sweep form sums the whole stencil in one FMA chain.
// In a step graph the residual of the last sweep flags DERR_NOTCONV (in
// *notconv) when the solve stops above tolerance.
struct SweepLoop {
  int *notconv;
};

// Residual of free row k: res = b - λ - A x, returned scaled as -d res in
// FP32 (r64 != nullptr also receives it in FP64); 0 on fixed rows.  The
// FIRST pass of a solve also accumulates ||rhs_eff||² (rhs_eff = b - λ -
// A_fixed x_fixed).
template <bool FIRST>
__device__ __forceinline__ float residual_node(const OpView &op, const RowClass *__restrict__ CT,
                                               const double *__restrict__ x, const double *__restrict__ rho,
                                               double neg_inv_eps0, double lam, int singular, int k, int i, int j,
                                               double *__restrict__ r64, double &a2, double &b2) {
  const int nx = op.nx, ny = op.ny;
  const unsigned ck = op.cls[k];
  if (ck & kFixedBit) {
    if (r64) r64[k] = 0.0;
    return 0.f;
  }
  const RowClass &C = CT[ck];
  const int w = i > 0 ? k - 1 : k + nx - 1;
  const int e = i < nx - 1 ? k + 1 : k - nx + 1;
  const int s = j > 0 ? k - nx : k + nx * (ny - 1);
  const int n = j < ny - 1 ? k + nx : k - nx * (ny - 1);
  double b = C.rho ? rho[k] * neg_inv_eps0 : op.bfix[k];
  if (singular) b -= lam;
  if (C.sig_dof >= 0) b -= C.sig_coef * op.sigma[C.sig_dof];
  double res;
  if (FIRST) {
    double afix = 0, afree = C.c0 * x[k];
    double t;
    t = C.cW * x[w];
    if (op.cls[w] & kFixedBit) afix += t; else afree += t;
    t = C.cE * x[e];
    if (op.cls[e] & kFixedBit) afix += t; else afree += t;
    t = C.cS * x[s];
    if (op.cls[s] & kFixedBit) afix += t; else afree += t;
    t = C.cN * x[n];
    if (op.cls[n] & kFixedBit) afix += t; else afree += t;
    const double rhs = b - afix;
    res = rhs - afree;
    b2 = fma(rhs, rhs, b2);
  } else {
    // GB300 runs FP64 at ~1/64 of the FP32 rate: one FMA chain over the stencil
    double ax = C.c0 * x[k];
    ax = fma(C.cW, x[w], ax);
    ax = fma(C.cE, x[e], ax);
    ax = fma(C.cS, x[s], ax);
    ax = fma(C.cN, x[n], ax);
    res = b - ax;
  }
  a2 = fma(res, res, a2);
  if (r64) r64[k] = -C.d * res;
  return (float)res * C.nd32;
}

// Block partials of the norms, then the last block to finish sums them in
// block order (deterministic), updates relres/iters and sets sc->done when
// ||res|| <= rtol ||rhs_eff||.  Ends the kernel for every other block.
template <bool FIRST>
__device__ __forceinline__ void finish_norms(PoissonScal *sc, double *__restrict__ part, double a2, double b2,
                                             double rtol2, SweepLoop loop, double *sh, int *last) {
  const double ta = block_sum(a2, sh);
  const double tb = FIRST ? block_sum(b2, sh) : 0.0;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = ta;
    if (FIRST) part[kPartials + blockIdx.x] = tb;
    __threadfence();
    *last = atomicAdd(&sc->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!*last) return;
  __threadfence();
  const double a = sum_partials(part, gridDim.x, sh);
  const double bb = FIRST ? sum_partials(part + kPartials, gridDim.x, sh) : 0.0;
  if (threadIdx.x == 0) {
    sc->ticket = 0u;
    const double rhs2 = FIRST ? bb : sc->rhs2;
    if (FIRST) {
      sc->rhs2 = bb;
      sc->iters = 0;
    } else {
      sc->iters += 1;
    }
    sc->res2 = a;
    sc->relres = rhs2 > 0 ? sqrt(a / rhs2) : sqrt(a);
    const int done = (rhs2 > 0 && a <= rtol2 * rhs2) || a == 0.0;
    sc->done = done;
    if (FIRST) sc->e_pending = done;
    if (loop.notconv && !done) atomicOr(loop.notconv, DERR_NOTCONV);
  }
}

__device__ __forceinline__ const RowClass *stage_classes(const OpView &op, RowClass *cls_sh) {
  const bool sm = op.nclass <= kSmemClasses;
  if (sm)
    for (int t = threadIdx.x; t < op.nclass; t += blockDim.x) cls_sh[t] = op.classes[t];
  __syncthreads();
  return sm ? cls_sh : op.classes;
}

// Residual pass over all nodes (scaled residual to r32 or r64), optionally
// with E = -∇ϕ, and the convergence test.  Passes after the first return at
// once when sc->done is set and count one sweep each.
template <bool FIRST, bool EOUT>
__global__ void __launch_bounds__(256) k_residual(OpView op, const double *__restrict__ x,
                                                  const double *__restrict__ rho, double neg_inv_eps0,
                                                  PoissonScal *sc, double *__restrict__ r64, float *__restrict__ r32,
                                                  double *__restrict__ part, int nn, int singular, double rtol2,
                                                  EOut eo, SweepLoop loop) {
  pdl_wait();
  __shared__ double sh[40];
  __shared__ RowClass cls_sh[kSmemClasses];
  __shared__ int last;
  if (!FIRST && sc->done) return;
  const RowClass *__restrict__ CT = stage_classes(op, cls_sh);
  const double lam = singular ? sc->lambda : 0.0;
  const int nx = op.nx, ny = op.ny;
  double a2 = 0, b2 = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int j = k / nx, i = k - j * nx;
    if (EOUT) efield_at(x, k, i, j, nx, ny, eo);
    const float v = residual_node<FIRST>(op, CT, x, rho, neg_inv_eps0, lam, singular, k, i, j, r64, a2, b2);
    if (r32) r32[k] = v;
  }
  finish_norms<FIRST>(sc, part, a2, b2, rtol2, loop, sh, &last);
}

// E = -∇ϕ at node k from ϕ at the node and its four stencil neighbours
// (double-float pairs, differenced in FP32: the hi parts of neighbours
// subtract exactly when within a factor 2; one-sided at the walls as efield_at)
__device__ __forceinline__ void efield_df5(float2 xk, float2 xw, float2 xe, float2 xs, float2 xn, int k, int i, int j,
                                           int nx, int ny, const EOut &eo) {
  auto dif = [](float2 p, float2 q) { return (p.x - q.x) + (p.y - q.y); };
  float ex, ey;
  if (i == 0) ex = dif(xk, xe) * eo.idx1;
  else if (i == nx - 1) ex = dif(xw, xk) * eo.idx1;
  else ex = dif(xw, xe) * eo.idx2;
  if (j == 0) ey = dif(xk, xn) * eo.idy1;
  else if (j == ny - 1) ey = dif(xs, xk) * eo.idy1;
  else ey = dif(xs, xn) * eo.idy2;
  eo.E32[k] = make_float2(ex, ey);
}

// Residual pass of the separable solver on the double-float ϕ: the stencil
// A x is summed in double-float arithmetic (FP32 pipes); the FIRST pass forms
// b (FP64, then split) for the free rows into bd and the rhs norm, later
// passes reuse bd.  Scaled FP32 residual to r32, E (EOUT), convergence test
// as k_residual (norms in FP64).  A node's loads (its row class, ϕ at the
// five stencil nodes, b) are all issued before its branch on the row class:
// the pass is bound by memory latency, not bandwidth.  In a step graph the
// FIRST pass writes no E (a correction nearly always follows); when it meets
// rtol already, the next pass, otherwise skipped, writes E instead.
// The node loop of k_residual_df over nodes k0, k0 + stride, ... < nn
// (partial norms in a2, b2).
template <bool FIRST, bool EOUT>
__device__ __forceinline__ void residual_df_nodes(const OpView &op, const RowClass *__restrict__ CT,
                                                  const float2 *__restrict__ x, const double *__restrict__ rho,
                                                  const float2 *__restrict__ rho_df, float2 nie_df,
                                                  double neg_inv_eps0, float2 *__restrict__ bd,
                                                  float *__restrict__ r32, int nn, int singular, double lam,
                                                  const EOut &eo, int k0, int stride, double &a2, double &b2) {
  const int nx = op.nx, ny = op.ny;
  for (int k = k0; k < nn; k += stride) {
    const int j = k / nx, i = k - j * nx;
    const int w = i > 0 ? k - 1 : k + nx - 1;
    const int e = i < nx - 1 ? k + 1 : k - nx + 1;
    const int s = j > 0 ? k - nx : k + nx * (ny - 1);
    const int n = j < ny - 1 ? k + nx : k - nx * (ny - 1);
    const unsigned ck = op.cls[k];
    const float2 xk = x[k], xw = x[w], xe = x[e], xs = x[s], xn = x[n];
    double rk = 0.0, fk = 0.0;
    float2 rdk = make_float2(0.f, 0.f);
    unsigned cw = 0, ce = 0, cs = 0, cn = 0;
    float2 b = make_float2(0.f, 0.f);
    if (FIRST) {
      if (rho_df) rdk = rho_df[k];
      else rk = rho[k];
      fk = op.bfix[k];
      cw = op.cls[w];
      ce = op.cls[e];
      cs = op.cls[s];
      cn = op.cls[n];
    } else {
      b = bd[k];
    }
    if (EOUT) efield_df5(xk, xw, xe, xs, xn, k, i, j, nx, ny, eo);
    if (ck & kFixedBit) {
      r32[k] = 0.f;
      continue;
    }
    const RowClass &C = CT[ck];
    float2 res;
    if (FIRST) {
      if (rho_df && C.rho) {  // ρ formed in double-float (no λ, no σ dofs then)
        b = df_mul(rdk, nie_df);
      } else {
        double bv = C.rho ? rk * neg_inv_eps0 : fk;
        if (singular) bv -= lam;
        if (C.sig_dof >= 0) bv -= C.sig_coef * op.sigma[C.sig_dof];
        b = df_from(bv);
      }
      bd[k] = b;
      float2 afix = make_float2(0.f, 0.f), afree = df_mul(C.c0f, xk);
      const float2 t[4] = {df_mul(C.cWf, xw), df_mul(C.cEf, xe), df_mul(C.cSf, xs), df_mul(C.cNf, xn)};
      const unsigned cq[4] = {cw, ce, cs, cn};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (cq[q] & kFixedBit) afix = df_add(afix, t[q]);
        else afree = df_add(afree, t[q]);
      }
      const float2 rhs = df_add(b, df_neg(afix));
      res = df_add(rhs, df_neg(afree));
      // the norms decide convergence to ~1e-7 relative at most: the FP32
      // value of the pair, squared in FP64 (no overflow)
      const double rh = (double)(rhs.x + rhs.y);
      b2 = fma(rh, rh, b2);
    } else {
      float2 ax = df_mul(C.c0f, xk);
      ax = df_add(ax, df_mul(C.cWf, xw));
      ax = df_add(ax, df_mul(C.cEf, xe));
      ax = df_add(ax, df_mul(C.cSf, xs));
      ax = df_add(ax, df_mul(C.cNf, xn));
      res = df_add(b, df_neg(ax));
    }
    const float resf = res.x + res.y;
    r32[k] = resf * C.nd32;
    const double rv = (double)resf;
    a2 = fma(rv, rv, a2);
  }
}

// E = -∇ϕ of the double-float ϕ at every node (a converged first residual
// wrote none)
__device__ __forceinline__ void efield_df_nodes(const float2 *__restrict__ x, int nx, int ny, int nn,
                                                const EOut &eo, int k0, int stride) {
  for (int k = k0; k < nn; k += stride) {
    const int j = k / nx, i = k - j * nx;
    const int w = i > 0 ? k - 1 : k + nx - 1, e = i < nx - 1 ? k + 1 : k - nx + 1;
    const int s = j > 0 ? k - nx : k + nx * (ny - 1), n = j < ny - 1 ? k + nx : k - nx * (ny - 1);
    efield_df5(x[k], x[w], x[e], x[s], x[n], k, i, j, nx, ny, eo);
  }
}

// Residual pass of the separable solver on the double-float ϕ: the stencil
// A x is summed in double-float arithmetic (FP32 pipes); the FIRST pass forms
// b (FP64, then split) for the free rows into bd and the rhs norm, later
// passes reuse bd.  Scaled FP32 residual to r32, E (EOUT), convergence test
// as k_residual (norms in FP64).  A node's loads (its row class, ϕ at the
// five stencil nodes, b) are all issued before its branch on the row class:
// the pass is bound by memory latency, not bandwidth.  In a step graph the
// FIRST pass writes no E (a correction nearly always follows); when it meets
// rtol already, the next pass, otherwise skipped, writes E instead.
template <bool FIRST, bool EOUT>
__global__ void __launch_bounds__(256) k_residual_df(OpView op, const float2 *__restrict__ x,
                                                     const double *__restrict__ rho, const float2 *__restrict__ rho_df,
                                                     float2 nie_df, double neg_inv_eps0,
                                                     float2 *__restrict__ bd, PoissonScal *sc, float *__restrict__ r32,
                                                     double *__restrict__ part, int nn, int singular, double rtol2,
                                                     EOut eo, SweepLoop loop) {
  pdl_wait();
  __shared__ double sh[40];
  __shared__ RowClass cls_sh[kSmemClasses];
  __shared__ int last;
  const int k0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  if (!FIRST && sc->done) {
    if (EOUT && sc->e_pending) efield_df_nodes(x, op.nx, op.ny, nn, eo, k0, stride);
    return;
  }
  const RowClass *__restrict__ CT = stage_classes(op, cls_sh);
  const double lam = singular ? sc->lambda : 0.0;
  double a2 = 0, b2 = 0;
  residual_df_nodes<FIRST, EOUT>(op, CT, x, rho, rho_df, nie_df, neg_inv_eps0, bd, r32, nn, singular, lam, eo, k0,
                                 stride, a2, b2);
  finish_norms<FIRST>(sc, part, a2, b2, rtol2, loop, sh, &last);
}

// mean-zero projection of the double-float ϕ (singular operators)
__global__ void k_sum_xd(const float2 *__restrict__ x, int nn, double *__restrict__ part) {
  pdl_wait();
  __shared__ double sh[40];
  double v = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) v += df_value(x[k]);
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}
__global__ void k_shift_xd(float2 *__restrict__ x, int nn, const double *__restrict__ part, int nparts) {
  pdl_wait();
  __shared__ double sh[40];
  double s = sum_partials(part, nparts, sh);
  const float2 m = df_neg(df_from(s / nn));
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) x[k] = df_add(x[k], m);
}

// ---------------- separable correction: FFT(y) x tridiagonal(x), FP32 ----------------
// One sweep computes δ ≈ S^-1 r in FP32 and adds it to the FP64 ϕ; the FP64
// residual pass that follows decides convergence (iterative refinement), so
// the converged ϕ meets the FP64 tolerance while the transform and the
// tridiagonal solves run on the FP32 pipes.  Two real columns share one
// complex FFT: z = a + i b, A_k = (Z_k + conj Z_{N-k})/2,
// B_k = (Z_k - conj Z_{N-k})/(2i).
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ unsigned bitrev(unsigned v, int bits) { return __brev(v) >> (32 - bits); }

// in-place radix-2 DIT FFT of TP length-N columns held in shared memory with
// column stride S (input in bit-reversed order), twiddles tw (N/2, shared);
// the inverse uses conjugate twiddles and leaves the 1/N to the caller
__device__ void fft_columns(float2 *buf, int TP, int N, int S, int logN, const float2 *tw, bool inverse) {
  const int hlog = logN - 1, hn = N >> 1;
  const int total = TP * hn;
  for (int s = 1; s <= logN; s++) {
    const int half = 1 << (s - 1);
    const int tws = logN - s;  // twiddle index = pos << tws
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
      const int col = b >> hlog;
      const int kk = b & (hn - 1);
      const int pos = kk & (half - 1);
      const int i1 = ((kk >> (s - 1)) << s) + pos, i2 = i1 + half;
      float2 w = tw[pos << tws];
      if (inverse) w.y = -w.y;
      float2 *c = buf + col * S;
      const float2 t = cmulf(w, c[i2]);
      const float2 u = c[i1];
      c[i1] = make_float2(u.x + t.x, u.y + t.y);
      c[i2] = make_float2(u.x - t.x, u.y - t.y);
    }
    __syncthreads();
  }
}

// r (nx, ny) -> spec[i K + k], k = 0..N/2: forward FFT along y of the 2 TP
// columns of work item `item` (columns 2 TP item ...), two per complex
// transform.  fbuf: TP columns of stride N + 1, then N/2 twiddles.  Ends with
// a block barrier (the next item may reuse fbuf).
__device__ __forceinline__ void fft_fwd_item(int item, const float *__restrict__ r, int nx, int N, int logN, int TP,
                                             const float2 *__restrict__ tw, float2 *__restrict__ spec,
                                             float2 *fbuf) {
  const int S = N + 1, W = 2 * TP, K = (N >> 1) + 1;
  const int i0 = item * W;
  float2 *tws = fbuf + TP * S;
  for (int t = threadIdx.x; t < (N >> 1); t += blockDim.x) tws[t] = __ldg(tw + t);
  for (int t = threadIdx.x; t < W * N; t += blockDim.x) {
    const int j = t / W, c = t - j * W;
    const int i = i0 + c;
    const float v = i < nx ? r[i + (size_t)nx * j] : 0.f;
    reinterpret_cast<float *>(fbuf + (c >> 1) * S + bitrev(j, logN))[c & 1] = v;
  }
  __syncthreads();
  fft_columns(fbuf, TP, N, S, logN, tws, false);
  for (int t = threadIdx.x; t < TP * K; t += blockDim.x) {
    const int p = t / K, k = t - p * K;
    const float2 zk = fbuf[p * S + k];
    const float2 zm = fbuf[p * S + ((N - k) & (N - 1))];
    const int ia = i0 + 2 * p;
    if (ia < nx) spec[(size_t)ia * K + k] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
    if (ia + 1 < nx) spec[(size_t)(ia + 1) * K + k] = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_fft_fwd(const float *__restrict__ r, int nx, int N, int logN, int TP,
                                                 const float2 *__restrict__ tw, float2 *__restrict__ spec,
                                                 const PoissonScal *__restrict__ sc) {
  pdl_wait();
  extern __shared__ float2 fbuf[];  // TP columns of stride S, then N/2 twiddles
  if (sc->done) return;
  fft_fwd_item(blockIdx.x, r, nx, N, logN, TP, tw, spec, fbuf);
}

// Per Fourier mode and real/imaginary part (one thread each): Thomas forward
// elimination and back substitution along x with the precomputed factors, in
// place in spec; Sherman-Morrison correction for x-periodic operators.  Used
// when a mode's column does not fit in shared memory for cyclic reduction.
// Rows are fetched in chunks of kTriChunk so that the chunk's loads are in
// flight together instead of one L2 round trip per row of the recurrence.
constexpr int kTriChunk = 16;

__global__ void __launch_bounds__(64) k_tridiag(float *__restrict__ spec, int nx, int K,
                                                const float *__restrict__ low, const float *__restrict__ inv,
                                                const float *__restrict__ cp, const float *__restrict__ q,
                                                const float *__restrict__ gk, int cyclic, int pin0,
                                                const PoissonScal *__restrict__ sc) {
  pdl_wait();
  if (sc->done) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = t >> 1, part = t & 1;
  if (k >= K) return;
  const size_t K2 = 2 * (size_t)K;
  float *__restrict__ col = spec + 2 * (size_t)k + part;  // row i at col[i * K2]
  if (pin0 >= 0 && k == 0) col[(size_t)pin0 * K2] = 0.f;  // pinned row of the singular mode
  float y = 0.f;
  for (int i0 = 0; i0 < nx; i0 += kTriChunk) {
    float r[kTriChunk], iv[kTriChunk], a[kTriChunk];
#pragma unroll
    for (int c = 0; c < kTriChunk; c++) {
      const int i = i0 + c;
      if (i < nx) {
        r[c] = col[i * K2];
        iv[c] = inv[(size_t)i * K + k];
        a[c] = i > 0 ? __ldg(low + i) : 0.f;
      }
    }
#pragma unroll
    for (int c = 0; c < kTriChunk; c++) {
      const int i = i0 + c;
      if (i < nx) {
        y = (r[c] - a[c] * y) * iv[c];
        col[i * K2] = y;
      }
    }
  }
  float xn = y;
  for (int i1 = nx - 2; i1 >= 0; i1 -= kTriChunk) {
    float yv[kTriChunk], cv[kTriChunk];
#pragma unroll
    for (int c = 0; c < kTriChunk; c++) {
      const int i = i1 - c;
      if (i >= 0) {
        yv[c] = col[i * K2];
        cv[c] = cp[(size_t)i * K + k];
      }
    }
#pragma unroll
    for (int c = 0; c < kTriChunk; c++) {
      const int i = i1 - c;
      if (i >= 0) {
        xn = yv[c] - cv[c] * xn;
        col[i * K2] = xn;
      }
    }
  }
  if (cyclic && !(k == 0 && pin0 >= 0)) {
    const float x0 = col[0], xl = col[(size_t)(nx - 1) * K2];
    const float f = (x0 + gk[K + k] * xl) * gk[k];
    for (int i = 0; i < nx; i++) col[i * K2] -= f * q[(size_t)i * K + k];
  }
}

// Cyclic reduction along x for G Fourier modes (2G real columns) held in
// shared memory.  The host factorisation stores each mode's coefficients
// contiguously (fwd: nf (α, γ) pairs, back: nb (a/b, c/b) pairs, backb: nb
// 1/b, then 1/b of the last row), and the block stages them in shared memory
// with the data in one pass, so the 2L dependent levels run on shared memory
// only.  Work item `item` takes modes G item ...; ends with a block barrier.
struct CrArgs {
  float *spec;
  int nx, K, G, L, nf, nb;
  const float2 *fwd, *back;
  const float *backb, *top, *q, *gk;
  int cyclic, pin0;
};

__device__ __forceinline__ void cr_item(int item, const CrArgs &A, float *fsh) {
  const int nx = A.nx, K = A.K, G = A.G, L = A.L, nf = A.nf, nb = A.nb;
  float *__restrict__ spec = A.spec;
  const int k0 = item * G;
  const int g = min(G, K - k0), ncol = 2 * g;
  float2 *cf = reinterpret_cast<float2 *>(fsh + 2 * G * nx);  // [g][nf]
  float2 *cb = cf + (size_t)G * nf;                            // [g][nb]
  float *cbb = reinterpret_cast<float *>(cb + (size_t)G * nb);  // [g][nb]
  for (int t = threadIdx.x; t < g * nf; t += blockDim.x) cf[t] = __ldg(A.fwd + (size_t)k0 * nf + t);
  for (int t = threadIdx.x; t < g * nb; t += blockDim.x) {
    cb[t] = __ldg(A.back + (size_t)k0 * nb + t);
    cbb[t] = __ldg(A.backb + (size_t)k0 * nb + t);
  }
  for (int t = threadIdx.x; t < nx * ncol; t += blockDim.x) {
    const int i = t / ncol, col = t - i * ncol;
    const int k = k0 + (col >> 1);
    float v = spec[((size_t)i * K + k) * 2 + (col & 1)];
    if (A.pin0 >= 0 && k == 0 && i == A.pin0) v = 0.f;  // pinned row of the singular mode
    fsh[col * nx + i] = v;
  }
  __syncthreads();
  int F = 0, B = 0;
  for (int l = 0; l < L; l++) {
    const int s = 1 << l, cnt = nx >> (l + 1);
    for (int t = threadIdx.x; t < cnt * ncol; t += blockDim.x) {
      const int m = t / ncol, col = t - m * ncol;
      const int i = (m + 1) * 2 * s - 1;
      const float2 ag = cf[(col >> 1) * nf + F + m];
      float *dc = fsh + col * nx;
      float v = dc[i] - ag.x * dc[i - s];
      if (i + s < nx) v -= ag.y * dc[i + s];
      dc[i] = v;
    }
    F += cnt;
    B += ((nx >> l) + 1) >> 1;
    __syncthreads();
  }
  const int topr = (1 << L) - 1;
  for (int col = threadIdx.x; col < ncol; col += blockDim.x) fsh[col * nx + topr] *= __ldg(A.top + k0 + (col >> 1));
  __syncthreads();
  for (int l = L - 1; l >= 0; l--) {
    const int s = 1 << l, ecnt = ((nx >> l) + 1) >> 1;
    B -= ecnt;
    for (int t = threadIdx.x; t < ecnt * ncol; t += blockDim.x) {
      const int m = t / ncol, col = t - m * ncol;
      const int j = (2 * m + 1) * s - 1;
      const int o = (col >> 1) * nb + B + m;
      const float2 r = cb[o];
      float *dc = fsh + col * nx;
      float x = cbb[o] * dc[j];
      if (j - s >= 0) x -= r.x * dc[j - s];
      if (j + s < nx) x -= r.y * dc[j + s];
      dc[j] = x;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < nx * ncol; t += blockDim.x) {
    const int i = t / ncol, col = t - i * ncol;
    const int k = k0 + (col >> 1);
    const float *dc = fsh + col * nx;
    float v = dc[i];
    if (A.cyclic && !(k == 0 && A.pin0 >= 0)) v -= (dc[0] + A.gk[K + k] * dc[nx - 1]) * A.gk[k] * A.q[(size_t)i * K + k];
    spec[((size_t)i * K + k) * 2 + (col & 1)] = v;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_tridiag_cr(CrArgs A, const PoissonScal *__restrict__ sc) {
  pdl_wait();
  extern __shared__ float fsh[];  // data [col][nx] (col = 2 (k - k0) + part), then per mode fwd, back, backb
  if (sc->done) return;
  cr_item(blockIdx.x, A, fsh);
}

// spec -> δ (nx, ny) by the inverse of k_fft_fwd for work item `item`; x +=
// δ on free rows.  Ends with a block barrier.
template <bool DF>
__device__ __forceinline__ void fft_inv_item(int item, const float2 *__restrict__ spec, int nx, int N, int logN,
                                             int TP, const float2 *__restrict__ tw, const uint16_t *__restrict__ cls,
                                             float2 *__restrict__ xd, double *__restrict__ x64, float2 *fbuf) {
  const int S = N + 1, W = 2 * TP, K = (N >> 1) + 1;
  const int i0 = item * W;
  float2 *tws = fbuf + TP * S;
  for (int t = threadIdx.x; t < (N >> 1); t += blockDim.x) tws[t] = __ldg(tw + t);
  // the update's ϕ values and row classes, fetched before the transform
  constexpr int kPre = 8;
  float2 xp[kPre];
  double xq[kPre];
  bool freep[kPre];
#pragma unroll
  for (int u = 0; u < kPre; u++) {
    const int t = threadIdx.x + u * blockDim.x;
    const int j = t / W, c = t - j * W;
    const int i = i0 + c;
    freep[u] = false;
    xp[u] = make_float2(0.f, 0.f);
    xq[u] = 0.0;
    if (t < W * N && i < nx) {
      const size_t kk = i + (size_t)nx * j;
      freep[u] = !(cls[kk] & kFixedBit);
      if (freep[u]) {
        if (DF) xp[u] = xd[kk];
        else xq[u] = x64[kk];
      }
    }
  }
  for (int t = threadIdx.x; t < TP * N; t += blockDim.x) {
    const int p = t >> logN, k = t & (N - 1);
    const int ia = i0 + 2 * p;
    const bool hi = k >= K;
    const int kk = hi ? N - k : k;
    float2 a = make_float2(0.f, 0.f), b = a;
    if (ia < nx) a = spec[(size_t)ia * K + kk];
    if (ia + 1 < nx) b = spec[(size_t)(ia + 1) * K + kk];
    if (hi) {
      a.y = -a.y;
      b.y = -b.y;
    }
    fbuf[p * S + bitrev(k, logN)] = make_float2(a.x - b.y, a.y + b.x);
  }
  __syncthreads();
  fft_columns(fbuf, TP, N, S, logN, tws, true);
  const float invN = 1.f / (float)N;  // N is a power of two: exact
#pragma unroll
  for (int u = 0; u < kPre; u++) {
    const int t = threadIdx.x + u * blockDim.x;
    const int j = t / W, c = t - j * W;
    const int i = i0 + c;
    if (freep[u]) {
      const float2 z = fbuf[(c >> 1) * S + j];
      const float dz = (c & 1 ? z.y : z.x) * invN;
      if (DF) xd[i + (size_t)nx * j] = df_add_f(xp[u], dz);
      else x64[i + (size_t)nx * j] = xq[u] + (double)dz;
    }
  }
  for (int t = threadIdx.x + kPre * blockDim.x; t < W * N; t += blockDim.x) {
    const int j = t / W, c = t - j * W;
    const int i = i0 + c;
    if (i < nx) {
      const size_t kk = i + (size_t)nx * j;
      if (!(cls[kk] & kFixedBit)) {
        const float2 z = fbuf[(c >> 1) * S + j];
        const float dz = (c & 1 ? z.y : z.x) * invN;
        if (DF) xd[kk] = df_add_f(xd[kk], dz);
        else x64[kk] += (double)dz;
      }
    }
  }
  __syncthreads();
}

template <bool DF>
__global__ void __launch_bounds__(256) k_fft_inv_update(const float2 *__restrict__ spec, int nx, int N, int logN,
                                                        int TP, const float2 *__restrict__ tw,
                                                        const uint16_t *__restrict__ cls, float2 *__restrict__ xd,
                                                        double *__restrict__ x64, const PoissonScal *__restrict__ sc) {
  pdl_wait();
  extern __shared__ float2 fbuf[];  // TP columns of stride S, then N/2 twiddles
  if (sc->done) return;
  fft_inv_item<DF>(blockIdx.x, spec, nx, N, logN, TP, tw, cls, xd, x64, fbuf);
}

// mean-zero projection of x over nodes (singular case)
__global__ void k_sum_x(const double *__restrict__ x, int nn, double *__restrict__ part) {
  pdl_wait();
  __shared__ double sh[40];
  double v = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) v += x[k];
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}
__global__ void k_shift_x(double *__restrict__ x, int nn, const double *__restrict__ part, int nparts) {
  pdl_wait();
  __shared__ double sh[40];
  double s = sum_partials(part, nparts, sh);
  const double m = s / nn;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) x[k] -= m;
}

// ---------------- Jacobi-preconditioned CG ----------------
// S p on free rows (p = 0 on fixed rows)
__device__ __forceinline__ double apply_S(const OpView &op, const RowClass &C, const double *__restrict__ v, int k) {
  int w, e, s, n;
  nbr(k, op.nx, op.ny, w, e, s, n);
  double a = C.c0 * v[k] + C.cW * v[w] + C.cE * v[e] + C.cS * v[s] + C.cN * v[n];
  return -C.d * a;
}

__global__ void k_cg_init(OpView op, const double *__restrict__ r, double *__restrict__ z, double *__restrict__ p,
                          double *__restrict__ part, int nn) {
  __shared__ double sh[40];
  double v = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const RowClass &C = op.classes[op.cls[k] & kClassMask];
    double zz = C.fixed ? 0.0 : r[k] / (-C.d * C.c0);
    z[k] = zz;
    p[k] = zz;
    v += r[k] * zz;
  }
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) part[2 * kPartials + blockIdx.x] = t;  // summed by k_cg_rz0
}

// rz of the iteration is held in sc->rz; the kernel that forms the next one
// stores it in sc->rz_new and this kernel (one per iteration, which reads
// neither) moves it to sc->rz: no block of a kernel reads a scalar another
// block of the same kernel writes.
__global__ void k_cg_ap(OpView op, const double *__restrict__ p, double *__restrict__ ap, double *__restrict__ part,
                        int nn, PoissonScal *__restrict__ sc) {
  __shared__ double sh[40];
  if (sc->done) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->rz = sc->rz_new;
  double v = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const RowClass &C = op.classes[op.cls[k] & kClassMask];
    double a = C.fixed ? 0.0 : apply_S(op, C, p, k);
    ap[k] = a;
    v += p[k] * a;
  }
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) part[kPartials + blockIdx.x] = t;
}

// α = rz/pAp; x += αp; r -= αAp; z = r/diag; partial rz_new and ||res||²
__global__ void k_cg_update(OpView op, double *__restrict__ x, double *__restrict__ r, double *__restrict__ z,
                            const double *__restrict__ p, const double *__restrict__ ap, double *__restrict__ part,
                            int nparts, int nn, const PoissonScal *__restrict__ sc) {
  __shared__ double sh[40];
  if (sc->done) return;
  const double rz = sc->rz;
  const double pap = sum_partials(part + kPartials, nparts, sh);
  const double alpha = pap != 0 ? rz / pap : 0.0;
  double v = 0, w2 = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const RowClass &C = op.classes[op.cls[k] & kClassMask];
    if (C.fixed) {
      z[k] = 0.0;
      continue;
    }
    x[k] += alpha * p[k];
    double rr = r[k] - alpha * ap[k];
    r[k] = rr;
    double zz = rr / (-C.d * C.c0);
    z[k] = zz;
    v += rr * zz;
    double res = rr / C.d;
    w2 += res * res;
  }
  double t = block_sum(v, sh);
  double t2 = block_sum(w2, sh);
  if (threadIdx.x == 0) {
    part[2 * kPartials + blockIdx.x] = t;
    part[3 * kPartials + blockIdx.x] = t2;
  }
}

// β = rz_new/rz; p = z + βp; convergence on the unscaled residual
__global__ void k_cg_dir(OpView op, const double *__restrict__ z, double *__restrict__ p, double *__restrict__ part,
                         int nparts, int nn, PoissonScal *sc, double rtol2) {
  __shared__ double sh[40];
  if (sc->done) return;
  const double rz = sc->rz;
  const double rzn = sum_partials(part + 2 * kPartials, nparts, sh);
  const double res2 = sum_partials(part + 3 * kPartials, nparts, sh);
  const double beta = rz != 0 ? rzn / rz : 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) p[k] = z[k] + beta * p[k];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rz_new = rzn;  // moved to sc->rz by the next k_cg_ap
    sc->res2 = res2;
    sc->relres = sc->rhs2 > 0 ? sqrt(res2 / sc->rhs2) : sqrt(res2);
    sc->iters += 1;
    if ((sc->rhs2 > 0 && res2 <= rtol2 * sc->rhs2) || res2 == 0.0) sc->done = 1;
  }
}

// rz of the first iteration (partials of k_cg_init / k_pcg_init in part[2K..])
__global__ void k_cg_rz0(const double *__restrict__ part, int nparts, PoissonScal *sc) {
  __shared__ double sh[40];
  const double t = sum_partials(part + 2 * kPartials, nparts, sh);
  if (threadIdx.x == 0) sc->rz_new = t;
}

// ---- flexible PCG with the multigrid preconditioner (multigrid.cu) ----
// z = M^-1 r comes from a V-cycle between k_pcg_update and k_pcg_dots; the
// direction update is Polak-Ribiere, beta = z_new.(r_new - r_old) / rz_old
// = -alpha z_new.(S p) / rz_old, which tolerates the FP32 rounding of the
// cycle.  Iteration: k_cg_ap, k_pcg_update, cycle, k_pcg_dots, k_pcg_dir.
__global__ void k_pcg_init(OpView op, const double *__restrict__ r, const double *__restrict__ z,
                           double *__restrict__ p, double *__restrict__ part, int nn) {
  __shared__ double sh[40];
  double v = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const double zz = (op.cls[k] & kFixedBit) ? 0.0 : z[k];
    p[k] = zz;
    v += r[k] * zz;
  }
  double t = block_sum(v, sh);
  if (threadIdx.x == 0) part[2 * kPartials + blockIdx.x] = t;
}

// α = rz/pAp; x += αp; r -= αAp; partial ||res||²; α kept for the direction
__global__ void k_pcg_update(OpView op, double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                             const double *__restrict__ ap, double *__restrict__ part, int nparts, int nn,
                             PoissonScal *__restrict__ sc) {
  __shared__ double sh[40];
  if (sc->done) return;
  const double rz = sc->rz;
  const double pap = sum_partials(part + kPartials, nparts, sh);
  const double alpha = pap != 0 ? rz / pap : 0.0;
  double w2 = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const RowClass &C = op.classes[op.cls[k] & kClassMask];
    if (C.fixed) continue;
    x[k] += alpha * p[k];
    const double rr = r[k] - alpha * ap[k];
    r[k] = rr;
    const double res = rr * C.inv_d;
    w2 += res * res;
  }
  double t2 = block_sum(w2, sh);
  if (threadIdx.x == 0) part[3 * kPartials + blockIdx.x] = t2;
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->pap = alpha;
}

// partials of z.r (part[2K..]) and z.Sp (part[K..], after k_pcg_update read pAp)
__global__ void k_pcg_dots(const double *__restrict__ r, const double *__restrict__ z, const double *__restrict__ ap,
                           double *__restrict__ part, int nn, const PoissonScal *__restrict__ sc) {
  __shared__ double sh[40];
  if (sc->done) return;
  double a = 0, b = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    a += z[k] * r[k];
    b += z[k] * ap[k];
  }
  const double ta = block_sum(a, sh), tb = block_sum(b, sh);
  if (threadIdx.x == 0) {
    part[2 * kPartials + blockIdx.x] = ta;
    part[kPartials + blockIdx.x] = tb;
  }
}

// β (Polak-Ribiere), p = z + βp on free rows, convergence on the unscaled residual
__global__ void k_pcg_dir(OpView op, const double *__restrict__ z, double *__restrict__ p, double *__restrict__ part,
                          int nparts, int nn, PoissonScal *sc, double rtol2) {
  __shared__ double sh[40];
  if (sc->done) return;
  const double rz = sc->rz, alpha = sc->pap;
  const double rzn = sum_partials(part + 2 * kPartials, nparts, sh);
  const double zap = sum_partials(part + kPartials, nparts, sh);
  const double res2 = sum_partials(part + 3 * kPartials, nparts, sh);
  const double beta = rz != 0 ? -alpha * zap / rz : 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x)
    p[k] = (op.cls[k] & kFixedBit) ? 0.0 : z[k] + beta * p[k];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rz_new = rzn;
    sc->res2 = res2;
    sc->relres = sc->rhs2 > 0 ? sqrt(res2 / sc->rhs2) : sqrt(res2);
    sc->iters += 1;
    if ((sc->rhs2 > 0 && res2 <= rtol2 * sc->rhs2) || res2 == 0.0) sc->done = 1;
  }
}

// ===========================================================================
// host: assembly
// ===========================================================================
static Poisson *poisson_new(Ctx *c, double eps0) {
  Poisson *P = new Poisson();
  P->nx = c->nx;
  P->ny = c->ny;
  P->nn = c->nn;
  P->dx = c->g.dx;
  P->dy = c->g.dy;
  P->eps0 = eps0;
  const int nx = P->nx, ny = P->ny;
  P->C.assign((size_t)P->nn * 7, 0.0);
  P->bfix.assign(P->nn, 0.0);
  P->rho_dof.assign(P->nn, 1);
  P->er.assign((size_t)(nx + 1) * (ny + 1), 1.0);
  // create_generalized_poisson_solver (:42-61)
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double *R = &P->C[(size_t)(i + nx * j) * 7];
      if (i < nx - 1) { R[0] -= 1.0; R[2] += 1.0; }
      if (i > 0) { R[0] -= 1.0; R[1] += 1.0; }
      if (j < ny - 1) { R[0] -= 1.0; R[4] += 1.0; }
      if (j > 0) { R[0] -= 1.0; R[3] += 1.0; }
    }
  const double h2 = P->dx * P->dx;  // A ./= grid.Δh[1]^2 (:65)
  for (auto &v : P->C) v /= h2;
  return P;
}

static double ER(const Poisson *P, int i1, int j1) {  // εr[i,j] with 1-based indices
  return P->er[(size_t)(i1 - 1) + (size_t)(P->nx + 1) * (j1 - 1)];
}

static void assemble_periodic(Poisson *P, int axis) {
  const int nx = P->nx, ny = P->ny;
  if (axis == 1) {
    const int js[2] = {1, ny};  // Julia iterates the tuple (1, ny)
    for (int t = 0; t < 2; t++) {
      const int j = js[t];
      for (int i = 1; i <= nx; i++) {
        double *R = &P->C[(size_t)((i - 1) + nx * (j - 1)) * 7];
        if (j == ny) {
          double cc = (0.5 * ER(P, i + 1, j + 1) + 0.5 * ER(P, i, j + 1)) / (P->dx * P->dx);
          R[0] -= cc;
          R[6] += cc;
        }
        if (j == 1) {
          double cc = (0.5 * ER(P, i + 1, j) + 0.5 * ER(P, i, j)) / (P->dx * P->dx);
          R[0] -= cc;
          R[6] += cc;
        }
      }
    }
  } else {
    for (int j = 1; j <= ny; j++) {
      const int is[2] = {1, nx};
      for (int t = 0; t < 2; t++) {
        const int i = is[t];
        double *R = &P->C[(size_t)((i - 1) + nx * (j - 1)) * 7];
        if (i == nx) {
          double cc = (0.5 * ER(P, i + 1, j + 1) + 0.5 * ER(P, i + 1, j)) / (P->dy * P->dy);
          R[0] -= cc;
          R[5] += cc;
        }
        if (i == 1) {
          double cc = (0.5 * ER(P, i, j) + 0.5 * ER(P, i, j + 1)) / (P->dy * P->dy);
          R[0] -= cc;
          R[5] += cc;
        }
      }
    }
  }
}

static void assemble_dirichlet(Poisson *P, const uint8_t *nodes, double phi0) {
  for (int r = 0; r < P->nn; r++) {
    if (!nodes[r]) continue;
    double *R = &P->C[(size_t)r * 7];
    for (int s = 0; s < 7; s++) R[s] = 0.0;
    for (auto &col : P->sig_cols) col[r] = 0.0;
    R[0] = 1.0;
    P->bfix[r] = phi0;
    P->rho_dof[r] = 0;
  }
}

// apply_neumann (generalized_poisson.jl:235-269).  gauss = false: the
// reference's rows exactly.  gauss = true: the same rows in the units of the
// stencil rows, i.e. the Gauss law of the electrode node's half (edge) or
// quarter (corner) cell with σ in C/m^2: the edge row is the reference's row
// divided by Δx with the σ coefficient 2/(ε0 Δx) (the reference's 2/Δx
// gradient row against a -ρ/ε0 right-hand side and an undivided σ mixes
// units), the corner row keeps its 1/Δ^2 coefficients and divides the σ
// coefficient by ε0.
static void assemble_neumann(Poisson *P, const uint8_t *nodes, int dof, bool gauss) {
  const int nx = P->nx, ny = P->ny;
  const double dx = P->dx, dy = P->dy;
  // edge-row ϕ divisor: Δx (reference), Δx Δx (Gauss form: 2 εr/(Δx Δx)
  // rounds like the stencil rows' 1/(Δx Δx), so the symmetrising scales stay
  // exact)
  const double ge = gauss ? dx * dx : dx;
  const double gs = gauss ? 1.0 / (P->eps0 * dx) : 1.0;   // edge-row σ scale
  const double gc = gauss ? 1.0 / P->eps0 : 1.0;          // corner-row σ scale
  auto N = [&](int i, int j) { return nodes[i + nx * j] != 0; };  // 0-based
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      if (!N(i, j)) continue;
      const bool a = i > 0 ? N(i - 1, j) : false;
      const bool b = i < nx - 1 ? N(i + 1, j) : false;
      const bool cc = j > 0 ? N(i, j - 1) : true;
      const bool d = j < ny - 1 ? N(i, j + 1) : true;
      const int r = i + nx * j;
      double *R = &P->C[(size_t)r * 7];
      std::vector<double> &S = P->sig_cols[dof - 1];
      if (cc == d && d == true && a == b && b == false) {
        const int ip = i == 0 ? i + 1 : i - 1;
        for (int s = 0; s < 7; s++) R[s] = 0.0;
        for (auto &col : P->sig_cols) col[r] = 0.0;
        R[0] -= 2 * ER(P, i + 1, j + 1) / ge;
        R[ip == i + 1 ? 2 : 1] += 2 * ER(P, ip + 1, j + 1) / ge;
        S[r] += 2 * gs;
      }
      if (cc != d) {
        const int ip = i == 0 ? i + 1 : i - 1;
        const int jp = cc ? j + 1 : j - 1;
        for (int s = 0; s < 7; s++) R[s] = 0.0;
        for (auto &col : P->sig_cols) col[r] = 0.0;
        const double e = ER(P, i + 1, j + 1);
        R[0] -= 4 * e / (3 * dx * dx);
        R[0] -= 4 * e / (3 * dy * dy);
        R[ip == i + 1 ? 2 : 1] += 4 * e / (3 * dx * dx);
        R[jp == j + 1 ? 4 : 3] += 4 * e / (3 * dy * dy);
        S[r] += (2.0 / 3.0) * (dx + dy) / (dx * dy) * gc;
      }
    }
}

// ===========================================================================
// host: device representation, symmetrisation, separable factorisation
// ===========================================================================
struct RowEff {
  double c0, cW, cE, cS, cN;
  int sig_dof;
  double sig_coef;
  bool fixed, rho;
};

static RowEff effective_row(const Poisson *P, int r) {
  const int nx = P->nx, ny = P->ny, i = r % nx, j = r / nx;
  const double *R = &P->C[(size_t)r * 7];
  RowEff e{};
  e.c0 = R[0];
  e.cW = R[1] + (i == 0 ? R[5] : 0.0);
  e.cE = R[2] + (i == nx - 1 ? R[5] : 0.0);
  e.cS = R[3] + (j == 0 ? R[6] : 0.0);
  e.cN = R[4] + (j == ny - 1 ? R[6] : 0.0);
  // nx == 1 / ny == 1 cannot occur (nx, ny >= 2)
  e.sig_dof = -1;
  e.sig_coef = 0;
  int nsig_here = 0;
  for (size_t k = 0; k < P->sig_cols.size(); k++)
    if (P->sig_cols[k][r] != 0.0) {
      e.sig_dof = (int)k;
      e.sig_coef = P->sig_cols[k][r];
      nsig_here++;
    }
  if (nsig_here > 1) e.sig_dof = -2;  // unsupported: flagged by the caller
  e.fixed = e.c0 == 1.0 && e.cW == 0 && e.cE == 0 && e.cS == 0 && e.cN == 0 && e.sig_dof == -1;
  e.rho = P->rho_dof[r] != 0;
  return e;
}

static int fft_smem_attr(Ctx *c, int N);

static int build_device(Ctx *c, Poisson *P) {
  const int nx = P->nx, ny = P->ny, nn = P->nn;
  std::vector<RowEff> rows(nn);
  for (int r = 0; r < nn; r++) {
    rows[r] = effective_row(P, r);
    if (rows[r].sig_dof == -2) return set_err(c, ISKRA_EINVAL, "a row couples to more than one σ dof");
  }
  // neighbor indices (wrapped) for the effective coefficients
  auto nb = [&](int r, int which) {
    const int i = r % nx, j = r / nx;
    switch (which) {
      case 0: return i > 0 ? r - 1 : r + nx - 1;
      case 1: return i < nx - 1 ? r + 1 : r - nx + 1;
      case 2: return j > 0 ? r - nx : r + nx * (ny - 1);
      default: return j < ny - 1 ? r + nx : r - nx * (ny - 1);
    }
  };
  auto coef_to = [&](int r, int col) {  // A[r, col] for a neighbor column
    const RowEff &e = rows[r];
    double a = 0;
    if (nb(r, 0) == col) a += e.cW;
    if (nb(r, 1) == col) a += e.cE;
    if (nb(r, 2) == col) a += e.cS;
    if (nb(r, 3) == col) a += e.cN;
    return a;
  };
  // symmetrising scale by breadth-first propagation over free rows
  std::vector<double> d(nn, 0.0);
  std::vector<int> queue;
  queue.reserve(nn);
  bool any_fixed = false;
  for (int r = 0; r < nn; r++) any_fixed |= rows[r].fixed;
  for (int r0 = 0; r0 < nn; r0++) {
    if (rows[r0].fixed || d[r0] != 0.0) continue;
    d[r0] = 1.0;
    queue.clear();
    queue.push_back(r0);
    for (size_t h = 0; h < queue.size(); h++) {
      const int r = queue[h];
      for (int w = 0; w < 4; w++) {
        const int cidx = nb(r, w);
        if (cidx == r || rows[cidx].fixed) continue;
        const double arc = coef_to(r, cidx), acr = coef_to(cidx, r);
        if (arc == 0.0 && acr == 0.0) continue;
        if (arc == 0.0 || acr == 0.0)
          return set_err(c, ISKRA_EINVAL, "boundary setup gives a non-symmetrizable operator");
        const double want = d[r] * arc / acr;
        if (d[cidx] == 0.0) {
          d[cidx] = want;
          queue.push_back(cidx);
        } else if (std::fabs(d[cidx] - want) > 1e-9 * std::fabs(want)) {
          return set_err(c, ISKRA_EINVAL, "boundary setup gives a non-symmetrizable operator");
        }
      }
    }
  }
  for (int r = 0; r < nn; r++)
    if (!rows[r].fixed && (!(d[r] > 0) || !(-d[r] * rows[r].c0 > 0)))
      return set_err(c, ISKRA_EINVAL, "assembled operator is not definite on its free rows");
  // singular: no fixed row and every free row sums to zero
  bool singular = !any_fixed;
  if (singular) {
    double mx = 0;
    for (int r = 0; r < nn; r++) mx = std::max(mx, std::fabs(rows[r].c0));
    for (int r = 0; r < nn && singular; r++) {
      const RowEff &e = rows[r];
      if (std::fabs(e.c0 + e.cW + e.cE + e.cS + e.cN) > 1e-12 * mx) singular = false;
    }
  }
  P->singular = singular;
  P->dsum = 0;
  for (int r = 0; r < nn; r++)
    if (!rows[r].fixed) P->dsum += d[r];
  // classes
  bool rho_fixed = false;
  std::map<std::vector<double>, int> cmap;
  std::vector<RowClass> classes;
  std::vector<uint16_t> cls(nn);
  for (int r = 0; r < nn; r++) {
    const RowEff &e = rows[r];
    std::vector<double> key = {e.c0, e.cW, e.cE, e.cS, e.cN, e.fixed ? 1.0 : 0.0, e.rho ? 1.0 : 0.0,
                               (double)e.sig_dof, e.sig_coef, e.fixed ? 0.0 : d[r]};
    auto it = cmap.find(key);
    int id;
    if (it == cmap.end()) {
      id = (int)classes.size();
      if (id > (int)kClassMask) return set_err(c, ISKRA_EINVAL, "too many distinct operator rows");
      cmap[key] = id;
      RowClass rc{};
      rc.c0 = e.c0;
      rc.cW = e.cW;
      rc.cE = e.cE;
      rc.cS = e.cS;
      rc.cN = e.cN;
      rc.d = e.fixed ? 1.0 : d[r];
      rc.inv_d = 1.0 / rc.d;
      rc.nd32 = (float)(-rc.d);
      auto split = [](double v) {
        const float h = (float)v;
        return make_float2(h, (float)(v - (double)h));
      };
      rc.c0f = split(e.c0);
      rc.cWf = split(e.cW);
      rc.cEf = split(e.cE);
      rc.cSf = split(e.cS);
      rc.cNf = split(e.cN);
      rc.sig_coef = e.sig_coef;
      rc.sig_dof = e.sig_dof;
      rc.fixed = e.fixed;
      rc.rho = e.rho;
      classes.push_back(rc);
    } else {
      id = it->second;
    }
    cls[r] = (uint16_t)(id | (e.fixed ? kFixedBit : 0u));
    rho_fixed |= e.fixed && e.rho;
  }
  P->nclass = (int)classes.size();
  P->rho_fixed = rho_fixed;
  // ---- separability: per column i, every j gives the same scaled row ----
  bool sep = P->method == 0 && ny >= 2 && (ny & (ny - 1)) == 0 && ny <= 4096;
  std::vector<double> s0(nx), sW(nx), sE(nx), ey(nx);
  std::vector<int> colfixed(nx);
  for (int i = 0; i < nx && sep; i++) {
    const RowEff &e0 = rows[i];
    colfixed[i] = e0.fixed;
    for (int j = 1; j < ny && sep; j++) {
      const RowEff &e = rows[i + nx * j];
      if (e.fixed != e0.fixed) sep = false;
      if (!e.fixed && (e.c0 != e0.c0 || e.cW != e0.cW || e.cE != e0.cE || e.cS != e0.cS || e.cN != e0.cN ||
                       d[i + nx * j] != d[i]))
        sep = false;
    }
    if (!sep) break;
    if (!e0.fixed) {
      if (e0.cS != e0.cN) sep = false;
      s0[i] = -d[i] * e0.c0;
      sW[i] = -d[i] * e0.cW;
      sE[i] = -d[i] * e0.cE;
      ey[i] = -d[i] * e0.cS;
    }
  }
  P->separable = sep;
  // ---- multigrid preconditioner of the CG path ----
  mg_destroy(P->mg);
  P->mg = nullptr;
  if (P->pcg_graph) cudaGraphExecDestroy(P->pcg_graph);
  P->pcg_graph = nullptr;
  if (!sep && !singular && P->method != 1) {
    std::vector<double> s0(nn, 0.0), sW(nn, 0.0), sE(nn, 0.0), sS(nn, 0.0), sN(nn, 0.0);
    std::vector<char> free_row(nn, 0);
    int per_x = 0, per_y = 0;
    for (int r = 0; r < nn; r++) {
      per_x |= P->C[(size_t)r * 7 + 5] != 0.0;
      per_y |= P->C[(size_t)r * 7 + 6] != 0.0;
      const RowEff &e = rows[r];
      if (e.fixed) continue;
      free_row[r] = 1;
      s0[r] = -d[r] * e.c0;
      sW[r] = -d[r] * e.cW;
      sE[r] = -d[r] * e.cE;
      sS[r] = -d[r] * e.cS;
      sN[r] = -d[r] * e.cN;
    }
    int rc = mg_build(c, nx, ny, s0, sW, sE, sS, sN, free_row, per_x, per_y, &P->mg);
    if (rc) return rc;
  }
  // ---- device upload ----
  cudaStream_t st = c->stream;
  ISKRA_CUDA(c, cudaStreamSynchronize(st));
  cudaFree(P->cls);
  cudaFree(P->classes);
  P->cls = nullptr;
  P->classes = nullptr;
  ISKRA_CUDA(c, cudaMalloc(&P->cls, nn * sizeof(uint16_t)));
  ISKRA_CUDA(c, cudaMalloc(&P->classes, classes.size() * sizeof(RowClass)));
  ISKRA_CUDA(c, cudaMemcpy(P->cls, cls.data(), nn * sizeof(uint16_t), cudaMemcpyHostToDevice));
  ISKRA_CUDA(c, cudaMemcpy(P->classes, classes.data(), classes.size() * sizeof(RowClass), cudaMemcpyHostToDevice));
  if (!P->bfix_d) ISKRA_CUDA(c, cudaMalloc(&P->bfix_d, nn * sizeof(double)));
  ISKRA_CUDA(c, cudaMemcpy(P->bfix_d, P->bfix.data(), nn * sizeof(double), cudaMemcpyHostToDevice));
  const int nsig = (int)P->sig_b.size();
  if (P->sigma_d && P->nsig > 0) {
    // the device σ values are authoritative (the circuit kernel updates them)
    ISKRA_CUDA(c, cudaMemcpy(P->sig_b.data(), P->sigma_d, std::min(nsig, P->nsig) * sizeof(double),
                             cudaMemcpyDeviceToHost));
  }
  if (nsig != P->nsig) {
    cudaFree(P->sigma_d);
    P->sigma_d = nullptr;
    P->nsig = nsig;
  }
  if (!P->sigma_d) ISKRA_CUDA(c, cudaMalloc(&P->sigma_d, (nsig > 0 ? nsig : 1) * sizeof(double)));
  if (nsig) ISKRA_CUDA(c, cudaMemcpy(P->sigma_d, P->sig_b.data(), nsig * sizeof(double), cudaMemcpyHostToDevice));
  if (P->df_mode && P->x_stale) {  // the FP64 view takes over the double-float state before a rebuild
    k_df_to_x<<<std::max(1, std::min(c->num_sms * 2, (nn + 255) / 256)), 256, 0, c->stream>>>(P->xd, P->x, nn);
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  P->df_mode = false;
  P->x_stale = false;
  if (!P->x) {
    ISKRA_CUDA(c, cudaMalloc(&P->x, nn * sizeof(double)));
    ISKRA_CUDA(c, cudaMemset(P->x, 0, nn * sizeof(double)));
    ISKRA_CUDA(c, cudaMalloc(&P->r, nn * sizeof(double)));
    ISKRA_CUDA(c, cudaMalloc(&P->z, nn * sizeof(double)));
    ISKRA_CUDA(c, cudaMalloc(&P->p, nn * sizeof(double)));
    ISKRA_CUDA(c, cudaMalloc(&P->ap, nn * sizeof(double)));
    ISKRA_CUDA(c, cudaMalloc(&P->part, 4 * kPartials * sizeof(double)));
    ISKRA_CUDA(c, cudaMalloc(&P->scal, sizeof(PoissonScal)));
    ISKRA_CUDA(c, cudaMallocHost(&P->scal_h, sizeof(PoissonScal)));
    ISKRA_CUDA(c, cudaMemset(P->scal, 0, sizeof(PoissonScal)));
  }
  // drives
  cudaFree(P->drive_node);
  cudaFree(P->drive_group);
  cudaFree(P->drive_par);
  P->drive_node = nullptr;
  P->drive_group = nullptr;
  P->drive_par = nullptr;
  {
    std::vector<int> dn, dg;
    std::vector<double> dp;
    for (size_t g = 0; g < P->drives.size(); g++) {
      for (int n : P->drives[g].nodes) {
        dn.push_back(n);
        dg.push_back((int)g);
      }
      dp.insert(dp.end(), {P->drives[g].amp, P->drives[g].freq, P->drives[g].phase, P->drives[g].dc});
    }
    P->ndrive_nodes = (int)dn.size();
    P->ndrive = (int)P->drives.size();
    if (!dn.empty()) {
      ISKRA_CUDA(c, cudaMalloc(&P->drive_node, dn.size() * sizeof(int)));
      ISKRA_CUDA(c, cudaMalloc(&P->drive_group, dg.size() * sizeof(int)));
      ISKRA_CUDA(c, cudaMalloc(&P->drive_par, dp.size() * sizeof(double)));
      ISKRA_CUDA(c, cudaMemcpy(P->drive_node, dn.data(), dn.size() * sizeof(int), cudaMemcpyHostToDevice));
      ISKRA_CUDA(c, cudaMemcpy(P->drive_group, dg.data(), dg.size() * sizeof(int), cudaMemcpyHostToDevice));
      ISKRA_CUDA(c, cudaMemcpy(P->drive_par, dp.data(), dp.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
  }
  P->blocks = std::min(kPartials, std::max(1, std::min(c->num_sms * ISKRA_RES_BLOCKS_PER_SM, (nn + 255) / 256)));
  P->cg_blocks = std::min(kPartials, std::max(1, std::min(c->num_sms * 6, (nn + 255) / 256)));
  // ---- separable factorisation ----
  cudaFree(P->r32);
  cudaFree(P->spec);
  cudaFree(P->tw);
  cudaFree(P->low);
  cudaFree(P->up);
  cudaFree(P->inv);
  cudaFree(P->cp);
  cudaFree(P->q);
  cudaFree(P->gk);
  cudaFree(P->cr_fwd);
  cudaFree(P->cr_back);
  cudaFree(P->cr_backb);
  cudaFree(P->cr_top);
  P->cr_fwd = P->cr_back = nullptr;
  P->cr_backb = P->cr_top = nullptr;
  P->r32 = nullptr;
  P->spec = nullptr;
  P->tw = nullptr;
  P->low = P->up = P->inv = P->cp = P->q = P->gk = nullptr;
  if (sep) {
    const int N = ny, K = N / 2 + 1;
    int logN = 0;
    while ((1 << logN) < N) logN++;
    P->N = N;
    P->K = K;
    P->logN = logN;
    // tridiagonal couplings per column (k-independent); fixed columns decouple
    std::vector<double> lo(nx, 0.0), upv(nx, 0.0);
    double corner_lo = 0.0, corner_up = 0.0;  // T[0][nx-1], T[nx-1][0]
    for (int i = 0; i < nx; i++) {
      if (colfixed[i]) continue;
      const int iw = i > 0 ? i - 1 : nx - 1, ie = i < nx - 1 ? i + 1 : 0;
      double w = colfixed[iw] ? 0.0 : sW[i];
      double e = colfixed[ie] ? 0.0 : sE[i];
      if (i == 0) {
        if (iw == ie) { e += w; w = 0; }  // nx == 2: wrap partner is the east neighbour
        corner_lo = w;
      } else {
        lo[i] = w;
      }
      if (i == nx - 1) {
        if (iw == ie) { lo[i] += e; e = 0; }
        corner_up = e;
      } else {
        upv[i] = e;
      }
    }
    const bool cyclic = corner_lo != 0.0 || corner_up != 0.0;
    P->cyclic = cyclic;
    const int pin = singular ? 0 : -1;  // singular => no fixed column, pin column 0 of mode 0
    P->pin_k0 = pin;
    std::vector<double> inv((size_t)nx * K), cpv((size_t)nx * K), qv(cyclic ? (size_t)nx * K : 1), gkv(2 * K, 0.0);
    int cr_levels = 0;
    while ((2 << cr_levels) <= nx) cr_levels++;  // L = floor(log2 nx)
    size_t cr_nf = 0, cr_nb = 0;
    for (int l = 0; l < cr_levels; l++) {
      cr_nf += nx >> (l + 1);
      cr_nb += ((nx >> l) + 1) >> 1;
    }
    std::vector<double2> cr_fwd(cr_nf * K), cr_back(cr_nb * K);
    std::vector<double> cr_backb(cr_nb * K), cr_top(K);
    for (int k = 0; k < K; k++) {
      double vfac = 0;
      const double ck = std::cos(2.0 * M_PI * k / N);
      std::vector<double> diag(nx), lk(lo), uk(upv);
      for (int i = 0; i < nx; i++) diag[i] = colfixed[i] ? 1.0 : s0[i] + 2.0 * ey[i] * ck;
      const bool pinned = (k == 0 && pin >= 0);
      const bool cyc = cyclic && !pinned;
      double gamma = 0;
      if (cyc) {
        gamma = -diag[0];
        vfac = corner_lo / gamma;  // v = [1, 0, ..., 0, β/γ], β = T[0][nx-1]
        gkv[K + k] = vfac;
        diag[0] -= gamma;
        diag[nx - 1] -= corner_up * corner_lo / gamma;
      }
      // Thomas factors (host: the Sherman-Morrison vector q below)
      double cprev = 0;
      for (int i = 0; i < nx; i++) {
        const size_t o = (size_t)i * K + k;
        if (pinned && i == pin) {
          inv[o] = 0.0;  // y_pin = 0
          cpv[o] = 0.0;
          cprev = 0.0;
          continue;
        }
        const double a = i > 0 ? lk[i] : 0.0;
        const double den = diag[i] - a * cprev;
        if (den == 0.0) return set_err(c, ISKRA_EINVAL, "singular tridiagonal mode in the Poisson factorisation");
        inv[o] = 1.0 / den;
        cprev = (i < nx - 1 ? uk[i] : 0.0) / den;
        cpv[o] = cprev;
      }
      // cyclic-reduction coefficients of T' (device solve).  Level l (stride
      // s = 2^l) updates rows i = (m+1)2s-1 from rows i-s, i+s and eliminates
      // rows j = (2m+1)s-1, which the back substitution recovers from rows j-s,
      // j+s; the last row left is 2^L-1, L = floor(log2 nx).
      {
        std::vector<double> a(nx), b(diag), cc(nx);
        for (int i = 0; i < nx; i++) {
          a[i] = i > 0 ? lk[i] : 0.0;
          cc[i] = i < nx - 1 ? uk[i] : 0.0;
        }
        if (pinned) {  // identity row; the kernel zeroes its right-hand side
          a[pin] = 0.0;
          cc[pin] = 0.0;
          b[pin] = 1.0;
        }
        size_t F = 0, B = 0;
        for (int l = 0; l < cr_levels; l++) {
          const int s = 1 << l;
          const int ecnt = ((nx >> l) + 1) >> 1, cnt = nx >> (l + 1);
          for (int m = 0; m < ecnt; m++) {
            const int j = (2 * m + 1) * s - 1;
            if (b[j] == 0.0) return set_err(c, ISKRA_EINVAL, "singular tridiagonal mode in the Poisson factorisation");
            const size_t o = (size_t)k * cr_nb + B + m;
            cr_back[o] = make_double2(a[j] / b[j], cc[j] / b[j]);
            cr_backb[o] = 1.0 / b[j];
          }
          for (int m = 0; m < cnt; m++) {
            const int i = (m + 1) * 2 * s - 1, im = i - s, ip = i + s;
            const double al = a[i] / b[im];
            const double ga = ip < nx ? cc[i] / b[ip] : 0.0;
            cr_fwd[(size_t)k * cr_nf + F + m] = make_double2(al, ga);
            b[i] = b[i] - al * cc[im] - (ip < nx ? ga * a[ip] : 0.0);
            a[i] = -al * a[im];
            cc[i] = ip < nx ? -ga * cc[ip] : 0.0;
          }
          F += cnt;
          B += ecnt;
        }
        const int top = (1 << cr_levels) - 1;
        if (b[top] == 0.0) return set_err(c, ISKRA_EINVAL, "singular tridiagonal mode in the Poisson factorisation");
        cr_top[k] = 1.0 / b[top];
      }
      if (cyc) {
        // q = T'^{-1} u, u = [γ, 0, ..., 0, α], α = T[nx-1][0]
        std::vector<double> y(nx), u(nx, 0.0);
        u[0] = gamma;
        u[nx - 1] += corner_up;
        for (int i = 0; i < nx; i++) {
          const size_t o = (size_t)i * K + k;
          const double a = i > 0 ? lk[i] : 0.0;
          y[i] = (u[i] - a * (i > 0 ? y[i - 1] : 0.0)) * inv[o];
        }
        for (int i = nx - 2; i >= 0; i--) y[i] -= cpv[(size_t)i * K + k] * y[i + 1];
        for (int i = 0; i < nx; i++) qv[(size_t)i * K + k] = y[i];
        gkv[k] = 1.0 / (1.0 + y[0] + vfac * y[nx - 1]);
      }
    }
    // device tables in FP32 (the correction runs in FP32)
    auto f32 = [](const std::vector<double> &v) { return std::vector<float>(v.begin(), v.end()); };
    auto f32x2 = [](const std::vector<double2> &v) {
      std::vector<float2> o(v.size());
      for (size_t n = 0; n < v.size(); n++) o[n] = make_float2((float)v[n].x, (float)v[n].y);
      return o;
    };
    std::vector<float2> tw(N / 2 > 0 ? N / 2 : 1);
    for (int m = 0; m < N / 2; m++) {
      const double ang = -2.0 * M_PI * m / N;
      tw[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    P->cr64.clear();
    for (const double2 &v : cr_fwd) P->cr64.insert(P->cr64.end(), {v.x, v.y});
    for (const double2 &v : cr_back) P->cr64.insert(P->cr64.end(), {v.x, v.y});
    P->cr64.insert(P->cr64.end(), cr_backb.begin(), cr_backb.end());
    P->cr64.insert(P->cr64.end(), cr_top.begin(), cr_top.end());
    cudaFree(P->cr64_d);
    P->cr64_d = nullptr;
    const std::vector<float> lo32 = f32(lo), up32 = f32(upv), inv32 = f32(inv), cp32 = f32(cpv), gk32 = f32(gkv),
                             q32 = f32(qv), backb32 = f32(cr_backb), top32 = f32(cr_top);
    const std::vector<float2> fwd32 = f32x2(cr_fwd), back32 = f32x2(cr_back);
    ISKRA_CUDA(c, cudaMalloc(&P->r32, nn * sizeof(float)));
    ISKRA_CUDA(c, cudaMalloc(&P->spec, (size_t)nx * K * sizeof(float2)));
    ISKRA_CUDA(c, cudaMalloc(&P->tw, tw.size() * sizeof(float2)));
    ISKRA_CUDA(c, cudaMalloc(&P->low, nx * sizeof(float)));
    ISKRA_CUDA(c, cudaMalloc(&P->up, nx * sizeof(float)));
    ISKRA_CUDA(c, cudaMalloc(&P->inv, (size_t)nx * K * sizeof(float)));
    ISKRA_CUDA(c, cudaMalloc(&P->cp, (size_t)nx * K * sizeof(float)));
    ISKRA_CUDA(c, cudaMalloc(&P->gk, 2 * K * sizeof(float)));
    ISKRA_CUDA(c, cudaMemcpy(P->tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice));
    ISKRA_CUDA(c, cudaMemcpy(P->low, lo32.data(), nx * sizeof(float), cudaMemcpyHostToDevice));
    ISKRA_CUDA(c, cudaMemcpy(P->up, up32.data(), nx * sizeof(float), cudaMemcpyHostToDevice));
    ISKRA_CUDA(c, cudaMemcpy(P->inv, inv32.data(), inv32.size() * sizeof(float), cudaMemcpyHostToDevice));
    ISKRA_CUDA(c, cudaMemcpy(P->cp, cp32.data(), cp32.size() * sizeof(float), cudaMemcpyHostToDevice));
    ISKRA_CUDA(c, cudaMemcpy(P->gk, gk32.data(), 2 * K * sizeof(float), cudaMemcpyHostToDevice));
    P->cr_levels = cr_levels;
    P->cr_nf = (int)cr_nf;
    P->cr_nb = (int)cr_nb;
    ISKRA_CUDA(c, cudaMalloc(&P->cr_fwd, std::max<size_t>(1, fwd32.size()) * sizeof(float2)));
    ISKRA_CUDA(c, cudaMalloc(&P->cr_back, std::max<size_t>(1, back32.size()) * sizeof(float2)));
    ISKRA_CUDA(c, cudaMalloc(&P->cr_backb, std::max<size_t>(1, backb32.size()) * sizeof(float)));
    ISKRA_CUDA(c, cudaMalloc(&P->cr_top, K * sizeof(float)));
    if (!fwd32.empty())
      ISKRA_CUDA(c, cudaMemcpy(P->cr_fwd, fwd32.data(), fwd32.size() * sizeof(float2), cudaMemcpyHostToDevice));
    if (!back32.empty()) {
      ISKRA_CUDA(c, cudaMemcpy(P->cr_back, back32.data(), back32.size() * sizeof(float2), cudaMemcpyHostToDevice));
      ISKRA_CUDA(c, cudaMemcpy(P->cr_backb, backb32.data(), backb32.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    ISKRA_CUDA(c, cudaMemcpy(P->cr_top, top32.data(), K * sizeof(float), cudaMemcpyHostToDevice));
    if (cyclic) {
      ISKRA_CUDA(c, cudaMalloc(&P->q, q32.size() * sizeof(float)));
      ISKRA_CUDA(c, cudaMemcpy(P->q, q32.data(), q32.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
  }
  if (sep) {
    int rc = fft_smem_attr(c, P->N);
    if (rc) return rc;
    if (!P->xd) ISKRA_CUDA(c, cudaMalloc(&P->xd, nn * sizeof(float2)));
    if (!P->bd) ISKRA_CUDA(c, cudaMalloc(&P->bd, nn * sizeof(float2)));
  }
  if (!P->xh) ISKRA_CUDA(c, cudaMalloc(&P->xh, nn * sizeof(double)));
  // a new operator: the next step solve starts from ϕ itself
  ISKRA_CUDA(c, cudaMemset(&P->scal->hist, 0, sizeof(int)));
  P->dirty = false;
  return ISKRA_OK;
}

static int fixed_to_x_now(Ctx *c);

int poisson_prepare(Ctx *c) {
  Poisson *P = c->ps;
  if (!P) return set_err(c, ISKRA_EINVAL, "no Poisson solver: call iskra_poisson_create");
  if (!P->dirty) return ISKRA_OK;
  invalidate_graphs(c);
  int rc = build_device(c, P);
  if (rc) return rc;
  return fixed_to_x_now(c);
}

static OpView opview(Poisson *P) {
  OpView o;
  o.cls = P->cls;
  o.classes = P->classes;
  o.bfix = P->bfix_d;
  o.sigma = P->sigma_d;
  o.nx = P->nx;
  o.ny = P->ny;
  o.nclass = P->nclass;
  return o;
}

static EOut eout(Ctx *c, bool on) {
  EOut e{};
  if (!on) return e;
  e.E32 = c->E32;
  e.idx2 = (float)(1.0 / (2 * c->g.dx));
  e.idx1 = (float)(1.0 / c->g.dx);
  e.idy2 = (float)(1.0 / (2 * c->g.dy));
  e.idy1 = (float)(1.0 / c->g.dy);
  return e;
}

// x at the fixed rows from the fixed values.  Solves rewrite only rows whose
// value can change between solves (driven rows, ρ-valued rows); the others are
// written here, after an operator build or a host update of Dirichlet values.
static int fixed_to_x_now(Ctx *c) {
  Poisson *P = c->ps;
  int rc = sync_rho64(c);  // ρ-valued fixed rows read the FP64 ρ
  if (rc) return rc;
  k_fixed_to_x<<<P->blocks, 256, 0, c->stream>>>(opview(P), P->x, P->xd, c->rho,
                                                  -1.0 / P->eps0, P->nn);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// Column pairs per FFT block: about two blocks per SM (at least one pair),
// at most 64 KB of float2 per block.
static int fft_tp(int N, int nx, int sms) {
  int tp = nx / (4 * sms);
  const int cap = (65536 / (int)sizeof(float2) - N / 2) / (N + 1);
  if (tp > cap) tp = cap;
  if (tp > 16) tp = 16;
  if (tp < 1) tp = 1;
  return tp;
}

static size_t fft_smem(int N, int tp) { return ((size_t)tp * (N + 1) + N / 2) * sizeof(float2); }

// Shared memory of one cyclic-reduction mode: 2 columns of nx floats and its
// coefficients (nf + nb float2, nb float; nf, nb < nx).
static size_t cr_mode_bytes(int nx) { return (size_t)nx * (2 * sizeof(float) + 2 * sizeof(float2) + sizeof(float)); }

// Fourier modes per cyclic-reduction block, about one block per mode up to
// K = 2 x SMs; 0 when one mode does not fit in shared memory (the chunked
// Thomas kernel is used then).
static int cr_modes_per_block(int nx, int K, int sms) {
  if (cr_mode_bytes(nx) > 160 * 1024) return 0;
  int g = K / (2 * sms);
  const int cap = (int)(160 * 1024 / cr_mode_bytes(nx));
  if (g > cap) g = cap;
  if (g > 8) g = 8;
  return g < 1 ? 1 : g;
}

static size_t cr_smem(const Poisson *P, int G) {
  return (size_t)G * (2 * P->nx * sizeof(float) + (P->cr_nf + P->cr_nb) * sizeof(float2) + P->cr_nb * sizeof(float));
}

static int fft_smem_attr(Ctx *c, int N) {
  const int smem = (int)fft_smem(N, fft_tp(N, c->ps->nx, c->num_sms));
  ISKRA_CUDA(c, cudaFuncSetAttribute(k_fft_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  ISKRA_CUDA(c, cudaFuncSetAttribute(k_fft_inv_update<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  ISKRA_CUDA(c, cudaFuncSetAttribute(k_fft_inv_update<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const int G = cr_modes_per_block(c->ps->nx, c->ps->K, c->num_sms);
  const int crsm = (int)cr_smem(c->ps, G);
  if (G && crsm > 48 * 1024)
    ISKRA_CUDA(c, cudaFuncSetAttribute(k_tridiag_cr, cudaFuncAttributeMaxDynamicSharedMemorySize, crsm));
  return ISKRA_OK;
}

static CrArgs cr_args(Poisson *P, int G) {
  CrArgs A;
  A.spec = (float *)P->spec;
  A.nx = P->nx;
  A.K = P->K;
  A.G = G;
  A.L = P->cr_levels;
  A.nf = P->cr_nf;
  A.nb = P->cr_nb;
  A.fwd = P->cr_fwd;
  A.back = P->cr_back;
  A.backb = P->cr_backb;
  A.top = P->cr_top;
  A.q = P->q;
  A.gk = P->gk;
  A.cyclic = (int)P->cyclic;
  A.pin0 = P->pin_k0;
  return A;
}

// Launch shape of the separable correction.
struct SepShape {
  int TP, fb, G;
  size_t smem;
};

static SepShape sep_shape(Ctx *c) {
  Poisson *P = c->ps;
  SepShape sh;
  sh.TP = fft_tp(P->N, P->nx, c->num_sms);
  sh.fb = (P->nx + 2 * sh.TP - 1) / (2 * sh.TP);
  sh.smem = fft_smem(P->N, sh.TP);
  sh.G = cr_modes_per_block(P->nx, P->K, c->num_sms);
  return sh;
}

// First part of a solve: the warm start (step solves of separable
// operators), fixed rows, the singular-case shift and the first residual
// (with E for separable operators), which resets the solver scalars.
static int queue_prologue(Ctx *c, double rtol, double dt_for_drive, SweepLoop loop, bool warm) {
  Poisson *P = c->ps;
  const int nn = P->nn, B = P->blocks, T = 256;
  OpView op = opview(P);
  const double nie = -1.0 / P->eps0;
  const float2 nie_df = df_host(nie);
  cudaStream_t st = c->stream;
  // the first residual takes ρ in double-float when it was formed so; every
  // other reader takes the FP64 copy
  const float2 *rdf = (P->separable && P->df_mode && !P->singular && !P->rho_fixed && c->rho_df_valid)
                          ? c->rho_df : nullptr;
  if (!rdf) {
    int rc = sync_rho64(c);
    if (rc) return rc;
  }
  if (warm && P->separable && P->warm_mode == 1 && c->warm_fused) {
    c->warm_fused = false;  // the step's ρ pass ran it
  } else if (warm && P->separable && P->warm_mode == 1) {
    if (P->df_mode)
      ISKRA_CUDA(c, launch_pdl(k_extrapolate<true>, B, T, 0, st, (const uint16_t *)P->cls, (void *)P->xd, P->xh,
                               nn, P->scal));
    else
      ISKRA_CUDA(c, launch_pdl(k_extrapolate<false>, B, T, 0, st, (const uint16_t *)P->cls, (void *)P->x, P->xh,
                               nn, P->scal));
  }
  if (P->ndrive_nodes)
    ISKRA_CUDA(c, launch_pdl(k_set_fixed, (P->ndrive_nodes + 255) / 256, 256, 0, st, op,
                             (const int *)P->drive_node, (const int *)P->drive_group, (const double *)P->drive_par,
                             P->ndrive_nodes, (const unsigned long long *)c->d_step, dt_for_drive, P->bfix_d, P->x,
                             P->xd, (const double *)c->rho, P->eps0, nn));
  // k_set_fixed wrote the driven rows; ρ-valued identity rows follow ρ
  if (P->rho_fixed)
    ISKRA_CUDA(c, launch_pdl(k_fixed_to_x, B, T, 0, st, op, P->x, P->xd,
                             (const double *)c->rho, nie, nn));
  if (P->singular) {
    ISKRA_CUDA(c, launch_pdl(k_sum_db, B, T, 0, st, op, (const double *)c->rho, nie, nn, P->part));
    ISKRA_CUDA(c, launch_pdl(k_lambda, 1, T, 0, st, (const double *)P->part, B, P->dsum, P->scal));
  }
  if (P->separable && P->df_mode) {
    // (step graphs: E comes from the following pass)
    if (warm)
      ISKRA_CUDA(c, launch_pdl(k_residual_df<true, false>, B, T, 0, st, op, (const float2 *)P->xd,
                               (const double *)c->rho, rdf, nie_df, nie, P->bd, P->scal, P->r32, P->part, nn,
                               (int)P->singular, rtol * rtol, eout(c, false), loop));
    else
      ISKRA_CUDA(c, launch_pdl(k_residual_df<true, true>, B, T, 0, st, op, (const float2 *)P->xd,
                               (const double *)c->rho, rdf, nie_df, nie, P->bd, P->scal, P->r32, P->part, nn,
                               (int)P->singular, rtol * rtol, eout(c, true), loop));
  } else if (P->separable) {
    ISKRA_CUDA(c, launch_pdl(k_residual<true, true>, B, T, 0, st, op, (const double *)P->x, (const double *)c->rho,
                             nie, P->scal, (double *)nullptr, P->r32, P->part, nn, (int)P->singular, rtol * rtol,
                             eout(c, true), loop));
  } else {
    ISKRA_CUDA(c, launch_pdl(k_residual<true, false>, B, T, 0, st, op, (const double *)P->x, (const double *)c->rho,
                             nie, P->scal, P->r, (float *)nullptr, P->part, nn, (int)P->singular, rtol * rtol,
                             eout(c, false), loop));
  }
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// `count` corrections: separable operators run the FP32 FFT, tridiagonal
// solve and inverse FFT, then the FP64 residual (each skipped on the device
// once converged); other operators run CG iterations (the caller loops for
// more).  `loop` applies to the last residual only.
static int queue_sweeps(Ctx *c, double rtol, int count, bool reset_cg, SweepLoop loop) {
  Poisson *P = c->ps;
  const int nn = P->nn, B = P->blocks, T = 256;
  OpView op = opview(P);
  const double nie = -1.0 / P->eps0;
  const double rtol2 = rtol * rtol;
  cudaStream_t st = c->stream;
  const SweepLoop none{};
  if (P->separable) {
    const SepShape sh = sep_shape(c);
    const int N = P->N, K = P->K;
    for (int s = 0; s < count; s++) {
      const bool last = s == count - 1;
      const PoissonScal *sc = P->scal;
      ISKRA_CUDA(c, launch_pdl(k_fft_fwd, sh.fb, 256, sh.smem, st, (const float *)P->r32, P->nx, N, P->logN, sh.TP,
                               (const float2 *)P->tw, P->spec, sc));
      if (sh.G) {
        ISKRA_CUDA(c, launch_pdl(k_tridiag_cr, (K + sh.G - 1) / sh.G, 256, cr_smem(P, sh.G), st, cr_args(P, sh.G),
                                 sc));
      } else {
        ISKRA_CUDA(c, launch_pdl(k_tridiag, (2 * K + 63) / 64, 64, 0, st, (float *)P->spec, P->nx, K,
                                 (const float *)P->low, (const float *)P->inv, (const float *)P->cp,
                                 (const float *)P->q, (const float *)P->gk, (int)P->cyclic, P->pin_k0, sc));
      }
      if (P->df_mode) {
        ISKRA_CUDA(c, launch_pdl(k_fft_inv_update<true>, sh.fb, 256, sh.smem, st, (const float2 *)P->spec, P->nx, N,
                                 P->logN, sh.TP, (const float2 *)P->tw, (const uint16_t *)P->cls, P->xd,
                                 (double *)nullptr, sc));
        ISKRA_CUDA(c, launch_pdl(k_residual_df<false, true>, B, T, 0, st, op, (const float2 *)P->xd,
                                 (const double *)nullptr, (const float2 *)nullptr, make_float2(0.f, 0.f), nie,
                                 P->bd, P->scal, P->r32, P->part, nn,
                                 (int)P->singular, rtol2, eout(c, true), last ? loop : none));
      } else {
        ISKRA_CUDA(c, launch_pdl(k_fft_inv_update<false>, sh.fb, 256, sh.smem, st, (const float2 *)P->spec, P->nx,
                                 N, P->logN, sh.TP, (const float2 *)P->tw, (const uint16_t *)P->cls,
                                 (float2 *)nullptr, P->x, sc));
        ISKRA_CUDA(c, launch_pdl(k_residual<false, true>, B, T, 0, st, op, (const double *)P->x,
                                 (const double *)c->rho, nie, P->scal, (double *)nullptr, P->r32, P->part, nn,
                                 (int)P->singular, rtol2, eout(c, true), last ? loop : none));
      }
    }
  } else if (P->mg) {  // flexible PCG, one multigrid V-cycle per iteration
    const int *skip = &P->scal->done;
    const int G = P->cg_blocks;
    if (reset_cg) {  // rhs2 is already in scal
      int rc = mg_queue_cycle(c, P->mg, P->r, P->z, skip);
      if (rc) return rc;
      k_pcg_init<<<G, T, 0, st>>>(op, P->r, P->z, P->p, P->part, nn);
      k_cg_rz0<<<1, T, 0, st>>>(P->part, G, P->scal);
    }
    for (int s = 0; s < count; s++) {
      k_cg_ap<<<G, T, 0, st>>>(op, P->p, P->ap, P->part, nn, P->scal);
      k_pcg_update<<<G, T, 0, st>>>(op, P->x, P->r, P->p, P->ap, P->part, G, nn, P->scal);
      int rc = mg_queue_cycle(c, P->mg, P->r, P->z, skip);
      if (rc) return rc;
      k_pcg_dots<<<G, T, 0, st>>>(P->r, P->z, P->ap, P->part, nn, P->scal);
      k_pcg_dir<<<G, T, 0, st>>>(op, P->z, P->p, P->part, G, nn, P->scal, rtol2);
    }
  } else {
    if (reset_cg) {  // rhs2 is already in scal
      k_cg_init<<<B, T, 0, st>>>(op, P->r, P->z, P->p, P->part, nn);
      k_cg_rz0<<<1, T, 0, st>>>(P->part, B, P->scal);
    }
    for (int s = 0; s < count; s++) {
      k_cg_ap<<<B, T, 0, st>>>(op, P->p, P->ap, P->part, nn, P->scal);
      k_cg_update<<<B, T, 0, st>>>(op, P->x, P->r, P->z, P->p, P->ap, P->part, B, nn, P->scal);
      k_cg_dir<<<B, T, 0, st>>>(op, P->z, P->p, P->part, B, nn, P->scal, rtol2);
    }
  }
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// Sweeps a step graph runs per solve (each skipped on the device once the
// residual meets rtol): one FP32 correction reduces the residual by about
// 10^-5 (cold start) and the step starts from the previous potential.
static int graph_sweeps(double rtol) {
  const int n = (int)std::ceil(std::log(rtol) / std::log(1e-5));
  return std::max(2, std::min(8, n));
}

static int finish_solve(Ctx *c) {
  Poisson *P = c->ps;
  if (P->singular && P->df_mode) {
    ISKRA_CUDA(c, launch_pdl(k_sum_xd, P->blocks, 256, 0, c->stream, (const float2 *)P->xd, P->nn, P->part));
    ISKRA_CUDA(c, launch_pdl(k_shift_xd, P->blocks, 256, 0, c->stream, P->xd, P->nn, (const double *)P->part,
                             P->blocks));
  } else if (P->singular) {
    ISKRA_CUDA(c, launch_pdl(k_sum_x, P->blocks, 256, 0, c->stream, (const double *)P->x, P->nn, P->part));
    ISKRA_CUDA(c, launch_pdl(k_shift_x, P->blocks, 256, 0, c->stream, P->x, P->nn, (const double *)P->part,
                             P->blocks));
  }
  // the separable path wrote E in its residual passes (the mean shift of the
  // singular case leaves E unchanged); CG computes it here
  c->e_from_phi = true;
  if (P->df_mode) P->x_stale = true;
  if (P->separable) return ISKRA_OK;
  return launch_efield_from(c, P->x);
}

// Solve queued inside a step capture (separable operators).
int poisson_solve_graph(Ctx *c, double rtol) {
  int rc = poisson_prepare(c);
  if (rc) return rc;
  Poisson *P = c->ps;
  if (!P->separable) return set_err(c, ISKRA_EINVAL, "graph solve needs a separable operator");
  const int n = graph_sweeps(rtol);
  const SweepLoop none{}, last{c->d_err};
  rc = queue_prologue(c, rtol, c->graph_dt, none, true);
  if (rc) return rc;
  rc = queue_sweeps(c, rtol, n, false, last);
  if (rc) return rc;
  return finish_solve(c);
}

// Learned warm start of a CG solve: δ = scale y on the free rows (the
// network's predicted correction), applied as ϕ += α δ with the exact line
// search α = δ·r / δ·Sδ in the energy norm of the scaled system S ϕ = c
// (r = c - S ϕ the scaled residual), so the CG error never grows.  Every
// scalar stays on the device: no host round trip inside the solve.
__global__ void k_lws_dir(OpView op, const float *__restrict__ y, const double *__restrict__ scale,
                          const double *__restrict__ r, double *__restrict__ p, double *__restrict__ part, int nn) {
  __shared__ double sh[40];
  const double sc = *scale;
  double v = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const RowClass &C = op.classes[op.cls[k] & kClassMask];
    const double d = C.fixed ? 0.0 : sc * (double)y[k];
    p[k] = d;
    v += d * r[k];
  }
  const double t = block_sum(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// α from the block partials of δ·r (part) and δ·Sδ (part + kPartials); no
// step when the first residual already met the tolerance or α is not a
// positive number
__global__ void __launch_bounds__(256) k_lws_alpha(const double *__restrict__ part, int nb, LwsScal *ls,
                                                   const PoissonScal *sc) {
  __shared__ double sh[40];
  double dr = 0, dsd = 0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    dr += part[b];
    dsd += part[kPartials + b];
  }
  dr = block_sum(dr, sh);
  __syncthreads();
  dsd = block_sum(dsd, sh);
  if (threadIdx.x == 0) {
    double a = dsd > 0 ? dr / dsd : 0.0;
    if (!(a > 0) || !isfinite(a) || sc->done) a = 0.0;
    ls->alpha = a;
    ls->res2_before = sc->res2;
  }
}

__global__ void k_lws_axpy(double *__restrict__ x, const double *__restrict__ p, const LwsScal *__restrict__ ls,
                           int nn) {
  const double alpha = ls->alpha;
  if (alpha == 0.0) return;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) x[k] += alpha * p[k];
}

// after the residual of the corrected ϕ: statistics of the applied step
__global__ void k_lws_stats(LwsScal *ls, const PoissonScal *sc) {
  if (ls->alpha > 0) {
    ls->warm_solves++;
    ls->alpha_sum += ls->alpha;
    ls->ratio_sum += ls->res2_before > 0 ? sqrt(sc->res2 / ls->res2_before) : 0.0;
  }
}

static int lws_line_search(Ctx *c, const float *y, const double *scale) {
  Poisson *P = c->ps;
  const int B = P->blocks, T = 256, nn = P->nn;
  OpView op = opview(P);
  LwsScal *ls = lws_scal(c);
  k_lws_dir<<<B, T, 0, c->stream>>>(op, y, scale, P->r, P->p, P->part, nn);
  k_cg_ap<<<B, T, 0, c->stream>>>(op, P->p, P->ap, P->part, nn, P->scal);
  k_lws_alpha<<<1, 256, 0, c->stream>>>(P->part, B, ls, P->scal);
  k_lws_axpy<<<B, T, 0, c->stream>>>(P->x, P->p, ls, nn);
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

// A solve with host convergence checks (CG; the separable solver outside
// step graphs).  step: the solve of an iskra_step (CG operators), which
// starts from ϕ extrapolated in time like the graph path; other solves
// start from ϕ and end the extrapolation history.
static int solve_sync(Ctx *c, double rtol, int maxit, int *iters, double *relres, bool step = false) {
  int rc = poisson_prepare(c);
  if (rc) return rc;
  rc = poisson_set_precision(c, rtol);
  if (rc) return rc;
  Poisson *P = c->ps;
  if (step && !P->separable && P->warm_mode == 1)
    ISKRA_CUDA(c, launch_pdl(k_extrapolate<false>, P->blocks, 256, 0, c->stream, (const uint16_t *)P->cls,
                             (void *)P->x, P->xh, P->nn, P->scal));
  bool first = true, lws_pending = false;
  int done_it = 0;
  const SweepLoop none{};
  for (;;) {
    const int chunk = std::min(P->separable ? 2 : (P->mg ? 4 : 32), maxit - done_it);
    if (first) {
      rc = queue_prologue(c, rtol, c->graph_dt, none, false);
      if (rc) return rc;
      if (!P->separable && lws_active(c)) {
        // learned warm start: the network's correction from the first
        // residual, then the residual again (CG restarts from the corrected
        // ϕ).  Harvesting reads the first residual's convergence on the host
        // (a solve that needs no iteration gives no training pair); in use
        // mode the device skips the step of an already converged solve.
        bool run = true;
        if (lws_harvesting(c)) {
          ISKRA_CUDA(c, cudaMemcpyAsync(P->scal_h, P->scal, sizeof(PoissonScal), cudaMemcpyDeviceToHost,
                                        c->stream));
          ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
          run = !P->scal_h->done;
        }
        if (run) {
          const float *y = nullptr;
          const double *scale = nullptr;
          lws_pending = true;
          rc = lws_begin(c, P->r, &y, &scale);
          if (rc) return rc;
          rc = lws_mark_start(c, P->x);
          if (rc) return rc;
          if (y) {
            rc = lws_line_search(c, y, scale);
            if (rc) return rc;
            rc = queue_prologue(c, rtol, c->graph_dt, none, false);
            if (rc) return rc;
            k_lws_stats<<<1, 1, 0, c->stream>>>(lws_scal(c), P->scal);
            ISKRA_CUDA(c, cudaGetLastError());
          }
        }
      }
    }
    if (P->mg) {
      // multigrid CG: the start (V-cycle of the first residual) queued, then
      // the iteration's kernels replayed as one graph
      if (first) {
        rc = queue_sweeps(c, rtol, 0, true, none);
        if (rc) return rc;
      }
      if (!P->pcg_graph || P->pcg_graph_rtol != rtol) {
        if (P->pcg_graph) cudaGraphExecDestroy(P->pcg_graph);
        P->pcg_graph = nullptr;
        cudaGraph_t g;
        ISKRA_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int qrc = queue_sweeps(c, rtol, 1, false, none);
        const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
        if (qrc) {
          if (ce == cudaSuccess) cudaGraphDestroy(g);
          return qrc;
        }
        ISKRA_CUDA(c, ce);
        const cudaError_t ie = cudaGraphInstantiate(&P->pcg_graph, g, 0);
        cudaGraphDestroy(g);
        ISKRA_CUDA(c, ie);
        P->pcg_graph_rtol = rtol;
      }
      for (int s = 0; s < chunk; s++) ISKRA_CUDA(c, cudaGraphLaunch(P->pcg_graph, c->stream));
    } else {
      rc = queue_sweeps(c, rtol, chunk, first, none);
      if (rc) return rc;
    }
    first = false;
    ISKRA_CUDA(c, cudaMemcpyAsync(P->scal_h, P->scal, sizeof(PoissonScal), cudaMemcpyDeviceToHost, c->stream));
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
    done_it = P->scal_h->iters;
    if (P->scal_h->done || done_it >= maxit) break;
  }
  rc = finish_solve(c);
  if (rc) return rc;
  if (lws_pending) {
    rc = lws_end(c, P->x, P->scal_h->done != 0);
    if (rc) return rc;
  }
  // ϕ moved outside the step sequence: the next step solve starts from it
  if (!step) ISKRA_CUDA(c, cudaMemsetAsync(&P->scal->hist, 0, sizeof(int), c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  P->last_iters = P->scal_h->iters;
  P->last_relres = P->scal_h->relres;
  if (iters) *iters = P->scal_h->iters;
  if (relres) *relres = P->scal_h->relres;
  if (!P->scal_h->done) return set_err(c, ISKRA_ENOTCONV, "Poisson solve did not reach the tolerance");
  return collect_device_errors(c);
}

double *poisson_sigma_ptr(Ctx *c) { return c->ps ? c->ps->sigma_d : nullptr; }
// the device σ values with the operator built (outside stream capture a
// pending rebuild runs first; a captured step has prepared it already)
double *poisson_sigma_prepared(Ctx *c) {
  if (!c->ps) return nullptr;
  if (c->ps->dirty && poisson_prepare(c) != ISKRA_OK) return nullptr;
  return c->ps->nsig > 0 ? c->ps->sigma_d : nullptr;
}
const double *poisson_x_ptr(Ctx *c) { return c->ps ? c->ps->x : nullptr; }
const float2 *poisson_xd_ptr(Ctx *c) { return c->ps && c->ps->df_mode ? c->ps->xd : nullptr; }
bool poisson_warm_args(Ctx *c, WarmArgs *w) {
  Poisson *P = c->ps;
  if (!P || !P->separable || !P->df_mode || P->warm_mode != 1 || !P->xh || !P->xd) return false;
  w->cls = P->cls;
  w->xd = P->xd;
  w->xh = (float2 *)P->xh;
  w->hist = &P->scal->hist;
  w->ticket = &P->scal->hticket;
  w->fixed_bit = kFixedBit;
  return true;
}

bool poisson_df_rho(Ctx *c) {
  const Poisson *P = c->ps;
  return P && !P->dirty && P->separable && P->df_mode && !P->singular && !P->rho_fixed;
}
void poisson_mark_x_stale(Ctx *c) {
  if (c->ps && c->ps->df_mode) c->ps->x_stale = true;
}

// FP64 view of ϕ brought up to date with the double-float state (stream-ordered)
int poisson_sync_x(Ctx *c) {
  Poisson *P = c->ps;
  if (!P || !P->df_mode || !P->x_stale) return ISKRA_OK;
  k_df_to_x<<<P->blocks, 256, 0, c->stream>>>(P->xd, P->x, P->nn);
  ISKRA_CUDA(c, cudaGetLastError());
  P->x_stale = false;
  return ISKRA_OK;
}

// Precision of the separable solver's state for a tolerance.  Double-float
// keeps ϕ to ~48 bits; its residual floor (~2^-47 |A||x| / ||rhs||, 5e-13
// measured at 512^2) is far below 1e-9, so tolerances from 1e-9 up run on
// the FP32 pipes.  Tighter tolerances and operators with σ dofs (whose rows
// mix 1/Δx and 1/Δx^2 scales) keep the FP64 state.
static bool want_df(const Poisson *P, double rtol) { return P->separable && P->nsig == 0 && rtol >= 1e-9; }

// Switches the authoritative state (outside stream capture; stream-ordered).
int poisson_set_precision(Ctx *c, double rtol) {
  Poisson *P = c->ps;
  if (!P) return ISKRA_OK;
  const bool df = want_df(P, rtol);
  if (df == P->df_mode) return ISKRA_OK;
  if (df) {
    k_x_to_df<<<P->blocks, 256, 0, c->stream>>>(P->x, P->xd, P->nn);
    P->x_stale = false;
  } else {
    if (P->x_stale) k_df_to_x<<<P->blocks, 256, 0, c->stream>>>(P->xd, P->x, P->nn);
    P->x_stale = false;
  }
  ISKRA_CUDA(c, cudaMemsetAsync(&P->scal->hist, 0, sizeof(int), c->stream));  // history in the other representation
  ISKRA_CUDA(c, cudaGetLastError());
  P->df_mode = df;
  invalidate_graphs(c);
  return ISKRA_OK;
}
bool poisson_separable(Ctx *c) { return c->ps && c->ps->separable; }
int poisson_solve_blocking(Ctx *c, double rtol, int maxit) {
  return solve_sync(c, rtol, maxit, nullptr, nullptr, true);
}

// ---------------------------------------------------------------------------
// Ensemble field solve: one block per run forms ρ from the run's deposit,
// sets the fixed rows (drive amplitudes per run), and solves the separable
// operator directly in FP64 -- residual of the previous potential, DFT along
// y (N <= 16, direct), cyclic reduction along x per Fourier mode with the
// host's FP64 coefficients (the single-run solver's, staged in shared memory
// while ρ is formed), inverse DFT -- then writes E.  The same operator as one
// FP64 sweep of the single-run solver, exact to rounding.  Cyclic reduction
// takes 2 log2(nx) dependent levels where a Thomas sweep takes 2 nx dependent
// FP64 steps on one thread per mode (on GB300, whose FP64 rate is ~1/64 of
// FP32, that chain was 2/3 of the kernel).
// ---------------------------------------------------------------------------
struct FieldRuns {
  int ns;
  unsigned long long *acc[kMaxSpecies];  // run 0; run stride nn
  unsigned *cnt[kMaxSpecies];
  double scale[kMaxSpecies];             // w0 2^-48
  double q[kMaxSpecies];
  const double *vol_inv, *bg;
  double *rho, *x;                       // R x nn
  float2 *E32;                           // R x nn
  const double *amp;                     // R x ngroups drive amplitudes
  int ngroups;
  const int *drive_node, *drive_group;
  const double *drive_par;               // 4 per group; par[0] replaced by amp[r][g]
  int ndrive_nodes;
  const unsigned long long *d_step;
  double dt, neg_inv_eps0;
  const double *cr;                      // packed FP64 cyclic-reduction coefficients
  int ncr, L, nf, nb, pin0;              // their count, levels, rows per mode; pinned row of mode 0 (or -1)
  int N, K;
  float idx2, idx1, idy2, idy1;
  int *err;
};

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

__global__ void __launch_bounds__(256) k_field_runs(OpView op, FieldRuns F) {
  extern __shared__ __align__(16) double fsm[];
  __shared__ RowClass cls_sh[kSmemClasses];
  __shared__ double twc[16], tws[16];  // cos, sin of 2π m/N
  const int nx = op.nx, ny = op.ny, nn = nx * ny, N = F.N, K = F.K, ncol = 2 * K;
  // xs, rs: nn each; dsp: column col = 2 k + part of the spectrum (nx each);
  // crs: the coefficients (2 nn + 2 nx K is even: 16-byte aligned pairs)
  double *xs = fsm, *rs = xs + nn, *dsp = rs + nn, *crs = dsp + (size_t)ncol * nx;
  // the coefficients do not depend on the previous kernel: staged before it ends
  for (int t = threadIdx.x; t < F.ncr; t += blockDim.x) cp_async8(crs + t, F.cr + t);
  asm volatile("cp.async.commit_group;" ::: "memory");
  pdl_wait();
  if (threadIdx.x < N) sincospi(2.0 * threadIdx.x / N, &tws[threadIdx.x], &twc[threadIdx.x]);
  const int r = blockIdx.x;
  const size_t o = (size_t)r * nn;
  const RowClass *__restrict__ CT = stage_classes(op, cls_sh);
  int flags = 0;
  // ρ from the run's deposit (consumed); ϕ of the previous step
  for (int k = threadIdx.x; k < nn; k += blockDim.x) {
    const double vi = F.vol_inv[k];
    double rho = 0.0;
    for (int s = 0; s < F.ns; s++) {
      const unsigned long long a = F.acc[s][o + k];
      if (F.cnt[s][o + k] > kMaxCell) flags |= DERR_OVERFLOW;
      F.acc[s][o + k] = 0ull;
      F.cnt[s][o + k] = 0u;
      rho += ((double)a * F.scale[s] * vi) * F.q[s];
    }
    if (F.bg) rho += F.bg[k];
    F.rho[o + k] = rho;
    xs[k] = F.x[o + k];
  }
  __syncthreads();
  // driven rows: V((n-2)Δt) with this run's amplitude, as k_set_fixed
  const unsigned long long n_step = *F.d_step;
  for (int t = threadIdx.x; t < F.ndrive_nodes; t += blockDim.x) {
    const int k = F.drive_node[t], g = F.drive_group[t];
    const double *par = F.drive_par + 4 * g;
    if (n_step >= 2) {
      const double tt = (double)(n_step - 2) * F.dt;
      xs[k] = F.amp[(size_t)r * F.ngroups + g] * sin(2.0 * M_PI * par[1] * tt + par[2]) + par[3];
    } else {
      xs[k] = op.bfix[k];
    }
  }
  __syncthreads();
  // scaled residual of the free rows
  for (int k = threadIdx.x; k < nn; k += blockDim.x) {
    const int j = k / nx, i = k - j * nx;
    const double rhoc = F.rho[o + k];
    const unsigned ck = op.cls[k];
    if (ck & kFixedBit) {
      rs[k] = 0.0;
      continue;
    }
    const RowClass &C = CT[ck];
    const int w = i > 0 ? k - 1 : k + nx - 1;
    const int e = i < nx - 1 ? k + 1 : k - nx + 1;
    const int s = j > 0 ? k - nx : k + nx * (ny - 1);
    const int n = j < ny - 1 ? k + nx : k - nx * (ny - 1);
    const double b = C.rho ? rhoc * F.neg_inv_eps0 : op.bfix[k];
    double ax = C.c0 * xs[k];
    ax = fma(C.cW, xs[w], ax);
    ax = fma(C.cE, xs[e], ax);
    ax = fma(C.cS, xs[s], ax);
    ax = fma(C.cN, xs[n], ax);
    rs[k] = -C.d * (b - ax);
  }
  __syncthreads();
  // DFT along y: column 2k (real) and 2k+1 (imaginary) of mode k,
  // Σ_j r[i, j] e^{-2πi jk/N}; the pinned row of mode 0 is zero
  for (int t = threadIdx.x; t < nx * K; t += blockDim.x) {
    const int i = t / K, k = t - i * K;
    double re = 0, im = 0;
    for (int j = 0; j < N; j++) {
      const int m = (j * k) % N;  // e^{-2πi jk/N}
      const double v = rs[i + nx * j];
      re += v * twc[m];
      im -= v * tws[m];
    }
    if (k == 0 && i == F.pin0) re = im = 0.0;
    dsp[(2 * k) * nx + i] = re;
    dsp[(2 * k + 1) * nx + i] = im;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  // cyclic reduction (the single-run solver's levels, in FP64)
  const double2 *fwd = reinterpret_cast<const double2 *>(crs);
  const double2 *back = fwd + (size_t)K * F.nf;
  const double *backb = reinterpret_cast<const double *>(back + (size_t)K * F.nb);
  const double *top = backb + (size_t)K * F.nb;
  int Fo = 0, Bo = 0;
  for (int l = 0; l < F.L; l++) {
    const int s = 1 << l, cnt = nx >> (l + 1);
    for (int t = threadIdx.x; t < cnt * ncol; t += blockDim.x) {
      const int m = t / ncol, col = t - m * ncol;
      const int i = (m + 1) * 2 * s - 1;
      const double2 ag = fwd[(size_t)(col >> 1) * F.nf + Fo + m];
      double *dc = dsp + (size_t)col * nx;
      double v = dc[i] - ag.x * dc[i - s];
      if (i + s < nx) v -= ag.y * dc[i + s];
      dc[i] = v;
    }
    Fo += cnt;
    Bo += ((nx >> l) + 1) >> 1;
    __syncthreads();
  }
  const int topr = (1 << F.L) - 1;
  for (int col = threadIdx.x; col < ncol; col += blockDim.x) dsp[(size_t)col * nx + topr] *= top[col >> 1];
  __syncthreads();
  for (int l = F.L - 1; l >= 0; l--) {
    const int s = 1 << l, ecnt = ((nx >> l) + 1) >> 1;
    Bo -= ecnt;
    for (int t = threadIdx.x; t < ecnt * ncol; t += blockDim.x) {
      const int m = t / ncol, col = t - m * ncol;
      const int j = (2 * m + 1) * s - 1;
      const size_t q = (size_t)(col >> 1) * F.nb + Bo + m;
      const double2 rr = back[q];
      double *dc = dsp + (size_t)col * nx;
      double x = backb[q] * dc[j];
      if (j - s >= 0) x -= rr.x * dc[j - s];
      if (j + s < nx) x -= rr.y * dc[j + s];
      dc[j] = x;
    }
    __syncthreads();
  }
  // inverse DFT (Hermitian spectrum) and update of the free rows
  const bool pow2N = (N & (N - 1)) == 0;
  const double invN = 1.0 / N;
  for (int k = threadIdx.x; k < nn; k += blockDim.x) {
    if (op.cls[k] & kFixedBit) continue;
    const int j = k / nx, i = k - j * nx;
    double v = 0;
    for (int m = 0; m < N; m++) {
      const int mm = m < K ? m : N - m;
      const double re = dsp[(2 * mm) * nx + i];
      const double im = m < K ? dsp[(2 * mm + 1) * nx + i] : -dsp[(2 * mm + 1) * nx + i];
      const int q = (j * m) % N;
      v += re * twc[q] - im * tws[q];
    }
    xs[k] += pow2N ? v * invN : v / N;  // 1/N exact for a power of two
  }
  __syncthreads();
  // ϕ and E = -∇ϕ
  EOut eo;
  eo.E32 = F.E32 + o;
  eo.idx2 = F.idx2;
  eo.idx1 = F.idx1;
  eo.idy2 = F.idy2;
  eo.idy1 = F.idy1;
  for (int k = threadIdx.x; k < nn; k += blockDim.x) {
    const int j = k / nx, i = k - j * nx;
    F.x[o + k] = xs[k];
    efield_at(xs, k, i, j, nx, ny, eo);
  }
  if (flags) atomicOr(F.err, flags);
}

// Ensemble field solve over R runs (separable, non-cyclic, non-singular
// operators with N = ny <= 16 and no σ dof).
int launch_field_runs(Ctx *c, int R, FieldRunsHost &H, cudaStream_t st) {
  int rc = poisson_prepare(c);
  if (rc) return rc;
  Poisson *P = c->ps;
  if (!P->separable || P->cyclic || P->singular || P->N > 16 || P->nsig > 0 || P->rho_fixed)
    return set_err(c, ISKRA_EINVAL, "ensemble field solve needs a separable, non-periodic-x operator with ny <= 16");
  const int nx = P->nx, K = P->K, nn = P->nn;
  if (!P->cr64_d) return set_err(c, ISKRA_EINVAL, "FP64 factors not uploaded (poisson_upload_fp64)");
  FieldRuns F{};
  F.ns = H.ns;
  for (int s = 0; s < H.ns; s++) {
    F.acc[s] = H.acc[s];
    F.cnt[s] = H.cnt[s];
    F.scale[s] = H.scale[s];
    F.q[s] = H.q[s];
  }
  F.vol_inv = c->vol_inv;
  F.bg = c->rho_bg;
  F.rho = H.rho;
  F.x = H.x;
  F.E32 = H.E32;
  F.amp = H.amp;
  F.ngroups = P->ndrive;
  F.drive_node = P->drive_node;
  F.drive_group = P->drive_group;
  F.drive_par = P->drive_par;
  F.ndrive_nodes = P->ndrive_nodes;
  F.d_step = H.d_step;
  F.dt = H.dt;
  F.neg_inv_eps0 = -1.0 / P->eps0;
  F.cr = P->cr64_d;
  F.ncr = (int)P->cr64.size();
  F.L = P->cr_levels;
  F.nf = P->cr_nf;
  F.nb = P->cr_nb;
  F.pin0 = P->pin_k0;
  F.N = P->N;
  F.K = K;
  const EOut e = eout(c, true);
  F.idx2 = e.idx2;
  F.idx1 = e.idx1;
  F.idy2 = e.idy2;
  F.idy1 = e.idy1;
  F.err = H.err;
  const size_t smem = (2 * (size_t)nn + 2 * (size_t)nx * K + P->cr64.size()) * sizeof(double);
  if (smem > 200 * 1024) return set_err(c, ISKRA_EINVAL, "ensemble grid too large for the per-run field solve");
  ISKRA_CUDA(c, cudaFuncSetAttribute(k_field_runs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  ISKRA_CUDA(c, launch_pdl(k_field_runs, R, 256, smem, st, opview(P), F));
  return ISKRA_OK;
}

// FP64 Thomas factors on the device (outside any stream capture)
int poisson_upload_fp64(Ctx *c) {
  int rc = poisson_prepare(c);
  if (rc) return rc;
  Poisson *P = c->ps;
  if (!P->separable) return set_err(c, ISKRA_EINVAL, "ensemble field solve needs a separable operator");
  if (P->cr64_d) return ISKRA_OK;
  ISKRA_CUDA(c, cudaMalloc(&P->cr64_d, std::max<size_t>(1, P->cr64.size()) * sizeof(double)));
  ISKRA_CUDA(c, cudaMemcpy(P->cr64_d, P->cr64.data(), P->cr64.size() * sizeof(double), cudaMemcpyHostToDevice));
  return ISKRA_OK;
}

int poisson_ndrive(Ctx *c) { return c->ps ? c->ps->ndrive : 0; }
double poisson_drive_amp(Ctx *c, int g) { return c->ps ? c->ps->drives[g].amp : 0.0; }

}  // namespace iskra

using namespace iskra;

extern "C" {

int iskra_poisson_create(iskra_ctx *h, double eps0) {
  if (!h || !(eps0 > 0)) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (c->ps) poisson_destroy(c->ps);
  c->ps = poisson_new(c, eps0);
  return ISKRA_OK;
}

int iskra_poisson_apply_dirichlet(iskra_ctx *h, const uint8_t *nodes, double phi0) {
  if (!h || !nodes) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  Poisson *P = c->ps;
  // value-only update of rows that are already identity rows: no rebuild
  bool structural = false;
  for (int r = 0; r < P->nn && !structural; r++) {
    if (!nodes[r]) continue;
    const double *R = &P->C[(size_t)r * 7];
    bool ident = R[0] == 1.0;
    for (int s = 1; s < 7; s++) ident &= R[s] == 0.0;
    for (auto &col : P->sig_cols) ident &= col[r] == 0.0;
    if (!ident || P->rho_dof[r]) structural = true;
  }
  assemble_dirichlet(P, nodes, phi0);
  if (structural || P->dirty) {
    P->dirty = true;
    return ISKRA_OK;
  }
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpy(P->bfix_d, P->bfix.data(), P->nn * sizeof(double), cudaMemcpyHostToDevice));
  return fixed_to_x_now(c);
}

int iskra_poisson_apply_periodic(iskra_ctx *h, int axis) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  if (axis != 1 && axis != 2) return set_err(c, ISKRA_EINVAL, "axis must be 1 or 2");
  assemble_periodic(c->ps, axis);
  c->ps->dirty = true;
  return ISKRA_OK;
}

int iskra_poisson_add_dof(iskra_ctx *h, int *dof) {
  if (!h || !dof) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  c->ps->sig_cols.emplace_back(c->ps->nn, 0.0);
  c->ps->sig_b.push_back(0.0);
  *dof = (int)c->ps->sig_b.size();
  c->ps->dirty = true;
  return ISKRA_OK;
}

int iskra_poisson_apply_neumann(iskra_ctx *h, const uint8_t *nodes, int dof) {
  if (!h || !nodes) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  if (dof < 1 || dof > (int)c->ps->sig_b.size()) return set_err(c, ISKRA_EINVAL, "bad σ dof");
  assemble_neumann(c->ps, nodes, dof, false);
  c->ps->dirty = true;
  return ISKRA_OK;
}

int iskra_poisson_apply_neumann_gauss(iskra_ctx *h, const uint8_t *nodes, int dof) {
  if (!h || !nodes) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  if (dof < 1 || dof > (int)c->ps->sig_b.size()) return set_err(c, ISKRA_EINVAL, "bad σ dof");
  assemble_neumann(c->ps, nodes, dof, true);
  c->ps->dirty = true;
  return ISKRA_OK;
}

int iskra_poisson_set_sigma(iskra_ctx *h, int dof, double value) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps || dof < 1 || dof > (int)c->ps->sig_b.size()) return set_err(c, ISKRA_EINVAL, "bad σ dof");
  c->ps->sig_b[dof - 1] = value;
  if (c->ps->sigma_d && dof <= c->ps->nsig) {
    ISKRA_CUDA(c, cudaMemcpyAsync(c->ps->sigma_d + (dof - 1), &c->ps->sig_b[dof - 1], sizeof(double),
                                  cudaMemcpyHostToDevice, c->stream));
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return ISKRA_OK;
}

int iskra_poisson_get_sigma(iskra_ctx *h, int dof, double *value) {
  if (!h || !value) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps || dof < 1 || dof > (int)c->ps->sig_b.size()) return set_err(c, ISKRA_EINVAL, "bad σ dof");
  if (c->ps->sigma_d && dof <= c->ps->nsig) {
    ISKRA_CUDA(c, cudaMemcpyAsync(&c->ps->sig_b[dof - 1], c->ps->sigma_d + (dof - 1), sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  *value = c->ps->sig_b[dof - 1];
  return ISKRA_OK;
}

int iskra_poisson_drive_dirichlet(iskra_ctx *h, const uint8_t *nodes, double amp, double freq, double phase,
                                  double dc) {
  if (!h || !nodes) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  DriveGroup g;
  for (int r = 0; r < c->ps->nn; r++) {
    if (!nodes[r]) continue;
    const double *R = &c->ps->C[(size_t)r * 7];
    bool ident = R[0] == 1.0 && !c->ps->rho_dof[r];
    for (int s = 1; s < 7; s++) ident &= R[s] == 0.0;
    if (!ident) return set_err(c, ISKRA_EINVAL, "driven nodes must be Dirichlet rows (apply_dirichlet first)");
    g.nodes.push_back(r);
  }
  g.amp = amp;
  g.freq = freq;
  g.phase = phase;
  g.dc = dc;
  c->ps->drives.push_back(g);
  c->ps->dirty = true;
  return ISKRA_OK;
}

int iskra_poisson_set_method(iskra_ctx *h, int method, int *active) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  if (method < 0 || method > 2) return set_err(c, ISKRA_EINVAL, "method must be 0, 1 or 2");
  if (c->ps->method != method) {
    c->ps->method = method;
    c->ps->dirty = true;
  }
  int rc = poisson_prepare(c);
  if (rc) return rc;
  if (active) *active = c->ps->separable ? 0 : (c->ps->mg ? 2 : 1);
  return ISKRA_OK;
}

int iskra_poisson_set_warm_start(iskra_ctx *h, int mode) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  if (mode != 0 && mode != 1) return set_err(c, ISKRA_EINVAL, "warm-start mode must be 0 or 1");
  if (c->ps->warm_mode != mode) {
    c->ps->warm_mode = mode;
    invalidate_graphs(c);
    if (c->ps->scal) ISKRA_CUDA(c, cudaMemsetAsync(&c->ps->scal->hist, 0, sizeof(int), c->stream));
  }
  return ISKRA_OK;
}

int iskra_poisson_solve(iskra_ctx *h, double rtol, int maxit, int *iters, double *relres) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!(rtol > 0) || maxit < 1) return set_err(c, ISKRA_EINVAL, "bad tolerance / iteration limit");
  int rc = launch_charge_density(c);
  if (rc) return rc;
  return solve_sync(c, rtol, maxit, iters, relres);
}

int iskra_poisson_solve_host(iskra_ctx *h, const double *f, double rtol, int maxit, double *phi_out, int *iters,
                             double *relres) {
  if (!h || !f) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!(rtol > 0) || maxit < 1) return set_err(c, ISKRA_EINVAL, "bad tolerance / iteration limit");
  // the device ρ holds -f: b[ρ] = f/ε0 = -ρ/ε0
  std::vector<double> negf(c->nn);
  for (int k = 0; k < c->nn; k++) negf[k] = -f[k];
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  ISKRA_CUDA(c, cudaMemcpy(c->rho, negf.data(), c->nn * sizeof(double), cudaMemcpyHostToDevice));
  c->rho64_valid = true;
  c->rho_df_valid = false;
  int rc = solve_sync(c, rtol, maxit, iters, relres);
  if (rc && rc != ISKRA_ENOTCONV) return rc;
  if (phi_out) {
    int rs = poisson_sync_x(c);
    if (rs) return rs;
    ISKRA_CUDA(c, cudaMemcpyAsync(phi_out, c->ps->x, c->nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return rc;
}

int iskra_solve_info(iskra_ctx *h, int *iters, double *relres) {
  if (!h) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps || !c->ps->scal) return set_err(c, ISKRA_EINVAL, "no solve yet");
  ISKRA_CUDA(c, cudaMemcpyAsync(c->ps->scal_h, c->ps->scal, sizeof(PoissonScal), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (iters) *iters = c->ps->scal_h->iters;
  if (relres) *relres = c->ps->scal_h->relres;
  return ISKRA_OK;
}

int iskra_poisson_residual(iskra_ctx *h, const double *f, const double *phi, double *relres) {
  if (!h || !f || !phi || !relres) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  if (!c->ps) return set_err(c, ISKRA_EINVAL, "no Poisson solver");
  int rc = poisson_prepare(c);
  if (rc) return rc;
  Poisson *P = c->ps;
  const int nx = P->nx, ny = P->ny, nn = P->nn;
  // the device copies of the fixed values (driven rows are rewritten there)
  // and of σ (the circuit and the tracker update it) are authoritative
  std::vector<double> bfix(nn), sig(P->sig_b.size());
  ISKRA_CUDA(c, cudaMemcpyAsync(bfix.data(), P->bfix_d, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (!sig.empty() && P->sigma_d)
    ISKRA_CUDA(c, cudaMemcpyAsync(sig.data(), P->sigma_d, std::min<size_t>(sig.size(), P->nsig) * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  // identity rows (Dirichlet values, driven rows): known values, moved to
  // the right-hand side as the solver does; the norms run over the others
  auto identity = [&](int r) {
    const double *R = &P->C[(size_t)r * 7];
    if (R[0] != 1.0) return false;
    for (int q = 1; q < 7; q++)
      if (R[q] != 0.0) return false;
    for (const auto &col : P->sig_cols)
      if (col[r] != 0.0) return false;
    return true;
  };
  std::vector<char> fixed(nn);
  for (int r = 0; r < nn; r++) fixed[r] = identity(r);
  double r2 = 0, b2 = 0;
  for (int r = 0; r < nn; r++) {
    if (fixed[r]) continue;
    const int i = r % nx, j = r / nx;
    const double *R = &P->C[(size_t)r * 7];
    const int col[7] = {r, i > 0 ? r - 1 : r, i < nx - 1 ? r + 1 : r, j > 0 ? r - nx : r, j < ny - 1 ? r + nx : r,
                        i == 0 ? r + nx - 1 : (i == nx - 1 ? r - nx + 1 : r),
                        j == 0 ? r + nx * (ny - 1) : (j == ny - 1 ? r - nx * (ny - 1) : r)};
    double afree = 0, known = 0;
    for (int q = 0; q < 7; q++) {
      if (R[q] == 0.0) continue;
      if (fixed[col[q]]) known += R[q] * phi[col[q]];
      else afree += R[q] * phi[col[q]];
    }
    for (size_t k = 0; k < P->sig_cols.size(); k++)
      if (P->sig_cols[k][r] != 0.0) known += P->sig_cols[k][r] * sig[k];
    const double b = (P->rho_dof[r] ? f[r] / P->eps0 : bfix[r]) - known;
    r2 += (b - afree) * (b - afree);
    b2 += b * b;
  }
  *relres = b2 > 0 ? std::sqrt(r2 / b2) : std::sqrt(r2);
  return ISKRA_OK;
}

}  // extern "C"

// device source of a field download (bringing ϕ and E up to date)
static int field_source(Ctx *c, int which, const double **src, size_t *n) {
  *n = (size_t)c->nn;
  if (which == ISKRA_FIELD_RHO) {
    int rs = sync_rho64(c);
    if (rs) return rs;
    *src = c->rho;
  } else if (which == ISKRA_FIELD_PHI) {
    if (!c->ps || !c->ps->x) return set_err(c, ISKRA_EINVAL, "no potential yet");
    int rs = poisson_sync_x(c);
    if (rs) return rs;
    *src = c->ps->x;
  } else if (which == ISKRA_FIELD_E) {
    if (c->e_from_phi && c->ps && c->ps->x) {
      int rs = poisson_sync_x(c);
      if (rs) return rs;
      int rc = launch_efield64(c, c->ps->x);
      if (rc) return rc;
    }
    *src = c->E64;
    *n *= 3;
  } else {
    return set_err(c, ISKRA_EINVAL, "bad field selector");
  }
  return ISKRA_OK;
}

extern "C" {

int iskra_field_download(iskra_ctx *h, int which, double *out) {
  if (!h || !out) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  const double *src = nullptr;
  size_t n = 0;
  int rc = field_source(c, which, &src, &n);
  if (rc) return rc;
  ISKRA_CUDA(c, cudaMemcpyAsync(out, src, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  ISKRA_CUDA(c, cudaStreamSynchronize(c->stream));
  return collect_device_errors(c);
}

// Non-blocking download: the field as the work queued so far leaves it is
// written to a device staging buffer on the context stream (ϕ of the
// double-float state converted straight into it), then copied to `out` on a
// second stream, so the copy overlaps the next queued steps.  Two staging
// buffers alternate: a download waits only for the copy of the one before
// last.  `out` (pinned host memory for a true overlap) holds the values after
// the next synchronising call.
int iskra_field_download_async(iskra_ctx *h, int which, double *out) {
  if (!h || !out) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  const size_t cap = (size_t)c->nn * 3;
  if (!c->dl_stage) {
    ISKRA_CUDA(c, cudaMalloc(&c->dl_stage, 2 * cap * sizeof(double)));
    ISKRA_CUDA(c, cudaStreamCreateWithFlags(&c->dl_stream, cudaStreamNonBlocking));
    ISKRA_CUDA(c, cudaEventCreateWithFlags(&c->dl_ready, cudaEventDisableTiming));
    for (int b = 0; b < 2; b++) ISKRA_CUDA(c, cudaEventCreateWithFlags(&c->dl_done[b], cudaEventDisableTiming));
  }
  const int b = c->dl_next;
  double *stage = c->dl_stage + (size_t)b * cap;
  size_t n = 0;
  Poisson *P = c->ps;
  if (which == ISKRA_FIELD_PHI && P && P->x && P->df_mode && P->x_stale) {
    if (c->dl_used[b]) ISKRA_CUDA(c, cudaStreamWaitEvent(c->stream, c->dl_done[b], 0));
    k_df_to_x<<<P->blocks, 256, 0, c->stream>>>(P->xd, stage, P->nn);
    ISKRA_CUDA(c, cudaGetLastError());
    n = (size_t)P->nn;
  } else {
    const double *src = nullptr;
    int rc = field_source(c, which, &src, &n);
    if (rc) return rc;
    if (c->dl_used[b]) ISKRA_CUDA(c, cudaStreamWaitEvent(c->stream, c->dl_done[b], 0));
    ISKRA_CUDA(c, cudaMemcpyAsync(stage, src, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  }
  ISKRA_CUDA(c, cudaEventRecord(c->dl_ready, c->stream));
  ISKRA_CUDA(c, cudaStreamWaitEvent(c->dl_stream, c->dl_ready, 0));
  ISKRA_CUDA(c, cudaMemcpyAsync(out, stage, n * sizeof(double), cudaMemcpyDeviceToHost, c->dl_stream));
  ISKRA_CUDA(c, cudaEventRecord(c->dl_done[b], c->dl_stream));
  c->dl_used[b] = true;
  c->dl_next = b ^ 1;
  c->dl_pending = true;
  return ISKRA_OK;
}

}  // extern "C"
