// multigrid.cu -- geometric multigrid V-cycle, the preconditioner of the CG
// Poisson solve for operators the FFT/tridiagonal solve cannot take (internal
// electrodes, non-column boundaries, Neumann rows that break separability).
//
// Replaces the reference's dense A\b (FiniteDifferenceMethod/src/
// generalized_poisson.jl:201-203,372-378) for those operators together with
// the FP64 conjugate-gradient iteration in poisson.cu: CG runs in FP64 on the
// symmetrised operator S = -D A over the free rows and is iterated to the
// requested relative residual; this file supplies z = M^-1 r, one V(2,2)
// cycle in FP32 (the preconditioner needs no FP64 accuracy; GB300 runs FP32
// at ~64x its FP64 rate, and the FP64 residual of the CG iteration decides
// convergence).  CG uses the flexible (Polak-Ribiere) direction update, so
// the FP32 rounding of the cycle does not stall it.
//
// Hierarchy: level 0 is S on the node grid (5-point, periodic wraps as the
// assembled operator has them; identity rows removed: the correction is zero
// there).  Coarser levels halve each axis that has at least 3 nodes (6 when
// periodic): coarse node I sits on fine node 2I, odd fine nodes interpolate
// linearly from their two coarse neighbours (one at an open far end), so
// P = Px (x) Py is bilinear; the coarse operator is the Galerkin product
// P^T S P (9-point), formed on the host in FP64.  Smoother: damped Jacobi
// (omega = 0.7), 2 sweeps before and after the coarse correction; the
// coarsest level (at most kMgCoarsest nodes) is solved exactly with its
// dense inverse.  The cycle is symmetric (same smoother before and after,
// restriction = P^T, exact coarsest solve), so it is a fixed SPD
// preconditioner up to FP32 rounding.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace iskra {

constexpr int kMgCoarsest = 400;  // nodes of the level solved by its dense inverse
constexpr float kMgOmega = 0.7f;
constexpr int kMgSweeps = 2;

struct MgLevel {
  int nx = 0, ny = 0, n = 0;
  int per_x = 0, per_y = 0;   // couplings across the seam exist on this axis
  int cx = 0, cy = 0;          // x / y coarsened towards the next level
  int five = 0;                // no corner couplings (5-point stencil)
  float *coef = nullptr;       // 9 x n: offset o = (dy + 1) 3 + (dx + 1), node-major
  float *dinv = nullptr;       // omega / diagonal, 0 on nodes outside the correction
  float *x = nullptr, *x2 = nullptr, *b = nullptr, *r = nullptr;
};

struct Mg {
  std::vector<MgLevel> lv;
  MgLevel *dlv = nullptr;      // device copy of lv (the single-block bottom reads it)
  int bottom = 0;              // first level of the single-block bottom (0: none)
  float *cinv = nullptr;       // dense inverse of the coarsest level (n x n)
};

void mg_destroy(Mg *m) {
  if (!m) return;
  for (auto &l : m->lv) {
    cudaFree(l.coef);
    cudaFree(l.dinv);
    cudaFree(l.x);
    cudaFree(l.x2);
    cudaFree(l.b);
    cudaFree(l.r);
  }
  cudaFree(m->cinv);
  cudaFree(m->dlv);
  delete m;
}

// ---- interpolation weights along one axis ----------------------------------
// fine index i -> up to two coarse parents with weights (coarsened axis of n
// fine / nc coarse nodes, periodic when per): even i -> i/2 (1); odd i ->
// (i-1)/2 and (i+1)/2 (1/2 each; (i+1)/2 wraps to 0 when periodic, and at an
// open far end the single parent takes 1).  Not coarsened: i -> i (1).
__host__ __device__ __forceinline__ int axis_parents(int i, int n, int nc, int coarsened, int per, int *c, float *w) {
  if (!coarsened) {
    c[0] = i;
    w[0] = 1.f;
    return 1;
  }
  if ((i & 1) == 0) {
    c[0] = i >> 1;
    w[0] = 1.f;
    return 1;
  }
  int hi = (i + 1) >> 1;
  if (hi >= nc) {
    if (per) {
      hi = 0;
    } else {
      c[0] = (i - 1) >> 1;
      w[0] = 1.f;
      return 1;
    }
  }
  c[0] = (i - 1) >> 1;
  w[0] = 0.5f;
  c[1] = hi;
  w[1] = 0.5f;
  return 2;
}

// ---- kernels (FP32) ----------------------------------------------------------
// Node kernels run one thread per node on (32 x 8)-thread blocks over the
// level's grid; every stencil load is issued unconditionally (a zero
// coefficient multiplies a finite x) so that the loads of a node overlap.
// FIVE: the level has no corner couplings (level 0, the 5-point operator):
// the four corner planes are neither read nor multiplied.
constexpr int kMgBx = 32, kMgBy = 8;

__device__ __forceinline__ int wrap_idx(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// (A x)_k with x(m) the iterate at node m
template <bool FIVE, class X>
__device__ __forceinline__ float apply9x(const float *__restrict__ coef, X x, int k, int i, int j, int nx, int ny,
                                         int n) {
  const int iw = wrap_idx(i - 1, nx), ie = wrap_idx(i + 1, nx);
  const int rs = nx * wrap_idx(j - 1, ny), rc = nx * j, rn = nx * wrap_idx(j + 1, ny);
  float a = coef[(size_t)4 * n + k] * x(k);
  a = fmaf(coef[(size_t)1 * n + k], x(i + rs), a);
  a = fmaf(coef[(size_t)3 * n + k], x(iw + rc), a);
  a = fmaf(coef[(size_t)5 * n + k], x(ie + rc), a);
  a = fmaf(coef[(size_t)7 * n + k], x(i + rn), a);
  if (!FIVE) {
    a = fmaf(coef[(size_t)0 * n + k], x(iw + rs), a);
    a = fmaf(coef[(size_t)2 * n + k], x(ie + rs), a);
    a = fmaf(coef[(size_t)6 * n + k], x(iw + rn), a);
    a = fmaf(coef[(size_t)8 * n + k], x(ie + rn), a);
  }
  return a;
}
template <bool FIVE>
__device__ __forceinline__ float apply9(const float *__restrict__ coef, const float *__restrict__ x, int k, int i,
                                        int j, int nx, int ny, int n) {
  return apply9x<FIVE>(coef, [&](int m) { return x[m]; }, k, i, j, nx, ny, n);
}

// One damped-Jacobi sweep at node (i, j): xo = xi + dinv (b - A xi).
// xi == nullptr: the first sweep from x = 0 (xo = dinv b); with r64 given it
// also forms the level-0 right-hand side b = (float) r64 (the FP64 scaled
// residual of the CG iteration).  z64 given: the last sweep of the cycle
// writes the result in FP64 there instead of xo.
template <bool FIVE>
__device__ __forceinline__ void smooth_node(const float *__restrict__ coef, const float *__restrict__ dinv,
                                            const float *__restrict__ xi, float *__restrict__ xo,
                                            float *__restrict__ b, int nx, int ny, int i, int j,
                                            const double *__restrict__ r64, double *__restrict__ z64) {
  const int n = nx * ny, k = i + nx * j;
  const float dk = dinv[k];
  if (!xi) {
    float bk;
    if (r64) {
      bk = (float)r64[k];
      b[k] = bk;
    } else {
      bk = b[k];
    }
    xo[k] = dk * bk;
    return;
  }
  const float ax = apply9<FIVE>(coef, xi, k, i, j, nx, ny, n);
  const float v = dk != 0.f ? xi[k] + dk * (b[k] - ax) : 0.f;
  if (z64) z64[k] = (double)v;
  else xo[k] = v;
}

// The first two sweeps at node (i, j): the first from x = 0 is pointwise
// (x0 = dinv b), so the second forms x0 at the stencil's nodes itself --
// the same products as two sweeps, without the first one's launch and its
// pass over x.  r64 given: level 0, b = (float) r64 (also stored in b).
template <bool FIVE>
__device__ __forceinline__ void smooth01_node(const float *__restrict__ coef, const float *__restrict__ dinv,
                                              float *__restrict__ xo, float *__restrict__ b, int nx, int ny, int i,
                                              int j, const double *__restrict__ r64) {
  const int n = nx * ny, k = i + nx * j;
  auto bval = [&](int m) { return r64 ? (float)r64[m] : b[m]; };
  auto x0 = [&](int m) { return __fmul_rn(dinv[m], bval(m)); };  // as the first sweep stores it
  const float dk = dinv[k], bk = bval(k);
  if (r64) b[k] = bk;
  const float ax = apply9x<FIVE>(coef, x0, k, i, j, nx, ny, n);
  xo[k] = dk != 0.f ? fmaf(dk, bk - ax, __fmul_rn(dk, bk)) : 0.f;
}

// r = b - A x at node (i, j) of the correction's nodes
template <bool FIVE>
__device__ __forceinline__ void residual_node(const float *__restrict__ coef, const float *__restrict__ dinv,
                                              const float *__restrict__ x, const float *__restrict__ b,
                                              float *__restrict__ r, int nx, int ny, int i, int j) {
  const int n = nx * ny, k = i + nx * j;
  const float ax = apply9<FIVE>(coef, x, k, i, j, nx, ny, n);
  r[k] = dinv[k] != 0.f ? b[k] - ax : 0.f;
}

struct MgXfer {
  int nx, ny, ncx, ncy, cx, cy, per_x, per_y;
};

// coarse b = P^T r at coarse node (I, J) (gathered from its fine candidates)
__device__ __forceinline__ void restrict_node(const float *__restrict__ r, float *__restrict__ bc, const MgXfer &T,
                                              int I, int J) {
  float s = 0.f;
  // fine candidates along each axis: 2I-1, 2I, 2I+1 (wrapped), or I itself
  int fi[3], fj[3];
  int ni = 0, nj = 0;
  if (T.cx) {
    for (int d = -1; d <= 1; d++) {
      int f = 2 * I + d;
      if (f < 0 || f >= T.nx) {
        if (!T.per_x) continue;
        f = wrap_idx(f, T.nx);
      }
      fi[ni++] = f;
    }
  } else {
    fi[ni++] = I;
  }
  if (T.cy) {
    for (int d = -1; d <= 1; d++) {
      int f = 2 * J + d;
      if (f < 0 || f >= T.ny) {
        if (!T.per_y) continue;
        f = wrap_idx(f, T.ny);
      }
      fj[nj++] = f;
    }
  } else {
    fj[nj++] = J;
  }
  for (int b2 = 0; b2 < nj; b2++) {
    int cj[2];
    float wj[2];
    const int pj = axis_parents(fj[b2], T.ny, T.ncy, T.cy, T.per_y, cj, wj);
    float wy = 0.f;
    for (int q = 0; q < pj; q++)
      if (cj[q] == J) wy += wj[q];
    if (wy == 0.f) continue;
    for (int a2 = 0; a2 < ni; a2++) {
      int ci[2];
      float wi[2];
      const int pi = axis_parents(fi[a2], T.nx, T.ncx, T.cx, T.per_x, ci, wi);
      float wx = 0.f;
      for (int q = 0; q < pi; q++)
        if (ci[q] == I) wx += wi[q];
      if (wx != 0.f) s = fmaf(wx * wy, r[fi[a2] + T.nx * fj[b2]], s);
    }
  }
  bc[I + T.ncx * J] = s;
}

// x += P xc at fine node (i, j) of the correction's nodes
__device__ __forceinline__ void prolong_node(float *__restrict__ x, const float *__restrict__ dinv,
                                             const float *__restrict__ xc, const MgXfer &T, int i, int j) {
  const int k = i + T.nx * j;
  if (dinv[k] == 0.f) return;
  int ci[2], cj[2];
  float wi[2], wj[2];
  const int pi = axis_parents(i, T.nx, T.ncx, T.cx, T.per_x, ci, wi);
  const int pj = axis_parents(j, T.ny, T.ncy, T.cy, T.per_y, cj, wj);
  float v = 0.f;
  for (int b2 = 0; b2 < pj; b2++)
    for (int a2 = 0; a2 < pi; a2++) v = fmaf(wi[a2] * wj[b2], xc[ci[a2] + T.ncx * cj[b2]], v);
  x[k] += v;
}

template <bool FIVE>
__global__ void __launch_bounds__(kMgBx * kMgBy) k_mg_smooth(const float *__restrict__ coef,
                                                             const float *__restrict__ dinv,
                                                             const float *__restrict__ xi, float *__restrict__ xo,
                                                             float *__restrict__ b, int nx, int ny, const int *skip,
                                                             const double *__restrict__ r64, double *__restrict__ z64) {
  pdl_wait();
  if (*skip) return;
  const int i = blockIdx.x * kMgBx + threadIdx.x, j = blockIdx.y * kMgBy + threadIdx.y;
  if (i < nx && j < ny) smooth_node<FIVE>(coef, dinv, xi, xo, b, nx, ny, i, j, r64, z64);
}

template <bool FIVE>
__global__ void __launch_bounds__(kMgBx * kMgBy) k_mg_smooth01(const float *__restrict__ coef,
                                                               const float *__restrict__ dinv, float *__restrict__ xo,
                                                               float *__restrict__ b, int nx, int ny, const int *skip,
                                                               const double *__restrict__ r64) {
  pdl_wait();
  if (*skip) return;
  const int i = blockIdx.x * kMgBx + threadIdx.x, j = blockIdx.y * kMgBy + threadIdx.y;
  if (i < nx && j < ny) smooth01_node<FIVE>(coef, dinv, xo, b, nx, ny, i, j, r64);
}

template <bool FIVE>
__global__ void __launch_bounds__(kMgBx * kMgBy) k_mg_residual(const float *__restrict__ coef,
                                                               const float *__restrict__ dinv,
                                                               const float *__restrict__ x,
                                                               const float *__restrict__ b, float *__restrict__ r,
                                                               int nx, int ny, const int *skip) {
  pdl_wait();
  if (*skip) return;
  const int i = blockIdx.x * kMgBx + threadIdx.x, j = blockIdx.y * kMgBy + threadIdx.y;
  if (i < nx && j < ny) residual_node<FIVE>(coef, dinv, x, b, r, nx, ny, i, j);
}

__global__ void __launch_bounds__(kMgBx * kMgBy) k_mg_restrict(const float *__restrict__ r, float *__restrict__ bc,
                                                               MgXfer T, const int *skip) {
  pdl_wait();
  if (*skip) return;
  const int I = blockIdx.x * kMgBx + threadIdx.x, J = blockIdx.y * kMgBy + threadIdx.y;
  if (I < T.ncx && J < T.ncy) restrict_node(r, bc, T, I, J);
}

__global__ void __launch_bounds__(kMgBx * kMgBy) k_mg_prolong(float *__restrict__ x, const float *__restrict__ dinv,
                                                              const float *__restrict__ xc, MgXfer T,
                                                              const int *skip) {
  pdl_wait();
  if (*skip) return;
  const int i = blockIdx.x * kMgBx + threadIdx.x, j = blockIdx.y * kMgBy + threadIdx.y;
  if (i < T.nx && j < T.ny) prolong_node(x, dinv, xc, T, i, j);
}

// coarsest level: x = Ainv b (one warp per row)
// (a hierarchy of one level reads r64 and writes z64, the FP64 vectors of the
// CG iteration, directly)
__global__ void __launch_bounds__(256) k_mg_coarse(const float *__restrict__ inv, const float *__restrict__ b,
                                                   float *__restrict__ x, int n, const int *skip,
                                                   const double *__restrict__ r64, double *__restrict__ z64) {
  pdl_wait();
  if (*skip) return;
  const int lane = threadIdx.x & 31;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += (gridDim.x * blockDim.x) >> 5) {
    float s = 0.f;
    for (int c = lane; c < n; c += 32) s = fmaf(inv[(size_t)row * n + c], r64 ? (float)r64[c] : b[c], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
      if (z64) z64[row] = (double)s;
      else x[row] = s;
    }
  }
}

// The smallest levels of the cycle in one block: levels l0 .. L-1 (each of at
// most kMgBottomNodes nodes) get the same sweeps, residuals, transfers and
// coarsest solve as the per-level kernels, separated by block barriers
// instead of launches -- at a few hundred to a thousand nodes a launch
// costs more than the level's work.  Leaves the correction in lv[l0].x.
constexpr int kMgBottomNodes = 1024;
constexpr int kMgBottomThreads = 1024;

__global__ void __launch_bounds__(kMgBottomThreads) k_mg_bottom(const MgLevel *__restrict__ lv, int l0, int L,
                                                                const float *__restrict__ cinv, const int *skip) {
  pdl_wait();
  if (*skip) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  auto xfer = [&](int l) {
    const MgLevel &F = lv[l], &C = lv[l + 1];
    return MgXfer{F.nx, F.ny, C.nx, C.ny, F.cx, F.cy, F.per_x, F.per_y};
  };
  auto smooth = [&](const MgLevel &D, const float *src, float *dst) {
    for (int k = tid; k < D.n; k += nt)
      smooth_node<false>(D.coef, D.dinv, src, dst, D.b, D.nx, D.ny, k % D.nx, k / D.nx, nullptr, nullptr);
    __syncthreads();
  };
  for (int l = l0; l + 1 < L; l++) {
    const MgLevel &D = lv[l];
    for (int s = 0; s < kMgSweeps; s++) smooth(D, s == 0 ? nullptr : ((s & 1) ? D.x2 : D.x), (s & 1) ? D.x : D.x2);
    for (int k = tid; k < D.n; k += nt) residual_node<false>(D.coef, D.dinv, D.x, D.b, D.r, D.nx, D.ny, k % D.nx, k / D.nx);
    __syncthreads();
    const MgLevel &C = lv[l + 1];
    const MgXfer T = xfer(l);
    for (int k = tid; k < C.n; k += nt) restrict_node(D.r, C.b, T, k % C.nx, k / C.nx);
    __syncthreads();
  }
  {
    const MgLevel &C = lv[L - 1];
    const int lane = tid & 31;
    for (int row = tid >> 5; row < C.n; row += nt >> 5) {
      float acc = 0.f;
      for (int c = lane; c < C.n; c += 32) acc = fmaf(cinv[(size_t)row * C.n + c], C.b[c], acc);
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      if (lane == 0) C.x[row] = acc;
    }
    __syncthreads();
  }
  for (int l = L - 2; l >= l0; l--) {
    const MgLevel &D = lv[l];
    const MgXfer T = xfer(l);
    for (int k = tid; k < D.n; k += nt) prolong_node(D.x, D.dinv, lv[l + 1].x, T, k % D.nx, k / D.nx);
    __syncthreads();
    for (int s = 0; s < kMgSweeps; s++) smooth(D, (s & 1) ? D.x2 : D.x, (s & 1) ? D.x : D.x2);
  }
}

// ---- host: hierarchy --------------------------------------------------------
struct HostLevel {
  int nx, ny, per_x, per_y;
  std::vector<double> coef;  // 9 x n (node-major per offset)
  std::vector<char> active;  // node takes part in the correction
};

static bool can_coarsen(int n, int per) { return per ? (n >= 6 && n % 2 == 0) : n >= 3; }

// Galerkin P^T A P of a level onto its coarsening
static HostLevel galerkin(const HostLevel &F, int cx, int cy) {
  HostLevel C;
  C.nx = cx ? (F.per_x ? F.nx / 2 : (F.nx + 1) / 2) : F.nx;
  C.ny = cy ? (F.per_y ? F.ny / 2 : (F.ny + 1) / 2) : F.ny;
  C.per_x = F.per_x;
  C.per_y = F.per_y;
  const int nf = F.nx * F.ny, nc = C.nx * C.ny;
  C.coef.assign((size_t)9 * nc, 0.0);
  auto cdelta = [](int a, int b, int n, int per) {  // b - a in {-1, 0, 1}
    int d = b - a;
    if (per && n > 2) {
      if (d > 1) d -= n;
      if (d < -1) d += n;
    }
    return d;
  };
  for (int k = 0; k < nf; k++) {
    if (!F.active[k]) continue;
    const int j = k / F.nx, i = k - j * F.nx;
    int fci[2], fcj[2];
    float fwi[2], fwj[2];
    const int fpi = axis_parents(i, F.nx, C.nx, cx, C.per_x, fci, fwi);
    const int fpj = axis_parents(j, F.ny, C.ny, cy, C.per_y, fcj, fwj);
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        const double a = F.coef[(size_t)((dy + 1) * 3 + dx + 1) * nf + k];
        if (a == 0.0) continue;
        int gi = i + dx, gj = j + dy;
        gi = gi < 0 ? gi + F.nx : (gi >= F.nx ? gi - F.nx : gi);
        gj = gj < 0 ? gj + F.ny : (gj >= F.ny ? gj - F.ny : gj);
        if (!F.active[gi + F.nx * gj]) continue;
        int gci[2], gcj[2];
        float gwi[2], gwj[2];
        const int gpi = axis_parents(gi, F.nx, C.nx, cx, C.per_x, gci, gwi);
        const int gpj = axis_parents(gj, F.ny, C.ny, cy, C.per_y, gcj, gwj);
        for (int p1 = 0; p1 < fpj; p1++)
          for (int p0 = 0; p0 < fpi; p0++) {
            const int I = fci[p0], J = fcj[p1];
            const double wf = (double)fwi[p0] * (double)fwj[p1];
            for (int q1 = 0; q1 < gpj; q1++)
              for (int q0 = 0; q0 < gpi; q0++) {
                const int ddx = cdelta(I, gci[q0], C.nx, C.per_x), ddy = cdelta(J, gcj[q1], C.ny, C.per_y);
                const double v = wf * a * (double)gwi[q0] * (double)gwj[q1];
                C.coef[(size_t)((ddy + 1) * 3 + ddx + 1) * nc + I + C.nx * J] += v;
              }
          }
      }
  }
  C.active.assign(nc, 0);
  double mx = 0;
  for (int K = 0; K < nc; K++) mx = std::max(mx, std::fabs(C.coef[(size_t)4 * nc + K]));
  for (int K = 0; K < nc; K++) C.active[K] = C.coef[(size_t)4 * nc + K] > 1e-12 * mx;
  for (int K = 0; K < nc; K++)
    if (!C.active[K])
      for (int o = 0; o < 9; o++) C.coef[(size_t)o * nc + K] = 0.0;
  return C;
}

// inverse of the active part of a small SPD level (Gauss-Jordan, FP64)
static std::vector<float> dense_inverse(const HostLevel &L) {
  const int n = L.nx * L.ny;
  std::vector<double> A((size_t)n * n, 0.0), Inv((size_t)n * n, 0.0);
  for (int k = 0; k < n; k++) {
    Inv[(size_t)k * n + k] = 1.0;
    if (!L.active[k]) {
      A[(size_t)k * n + k] = 1.0;
      continue;
    }
    const int j = k / L.nx, i = k - j * L.nx;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        const double a = L.coef[(size_t)((dy + 1) * 3 + dx + 1) * n + k];
        if (a == 0.0) continue;
        int gi = i + dx, gj = j + dy;
        gi = gi < 0 ? gi + L.nx : (gi >= L.nx ? gi - L.nx : gi);
        gj = gj < 0 ? gj + L.ny : (gj >= L.ny ? gj - L.ny : gj);
        const int g = gi + L.nx * gj;
        if (L.active[g]) A[(size_t)k * n + g] += a;
      }
  }
  for (int c = 0; c < n; c++) {
    int piv = c;
    for (int r = c + 1; r < n; r++)
      if (std::fabs(A[(size_t)r * n + c]) > std::fabs(A[(size_t)piv * n + c])) piv = r;
    if (piv != c)
      for (int q = 0; q < n; q++) {
        std::swap(A[(size_t)c * n + q], A[(size_t)piv * n + q]);
        std::swap(Inv[(size_t)c * n + q], Inv[(size_t)piv * n + q]);
      }
    const double d = A[(size_t)c * n + c];
    const double id = d != 0.0 ? 1.0 / d : 0.0;
    for (int q = 0; q < n; q++) {
      A[(size_t)c * n + q] *= id;
      Inv[(size_t)c * n + q] *= id;
    }
    for (int r = 0; r < n; r++) {
      if (r == c) continue;
      const double f = A[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (int q = 0; q < n; q++) {
        A[(size_t)r * n + q] -= f * A[(size_t)c * n + q];
        Inv[(size_t)r * n + q] -= f * Inv[(size_t)c * n + q];
      }
    }
  }
  std::vector<float> out((size_t)n * n);
  for (int r = 0; r < n; r++)
    for (int q = 0; q < n; q++)
      out[(size_t)r * n + q] = (L.active[r] && L.active[q]) ? (float)Inv[(size_t)r * n + q] : 0.f;
  return out;
}

// Builds the hierarchy of the scaled operator S: per node its five
// coefficients s0 (diagonal), sW, sE, sS, sN (to the wrapped neighbours;
// zero where the assembled operator has no coupling) and whether the node is
// free (identity rows are not).  per_x / per_y: some row couples across the
// x / y seam.
int mg_build(Ctx *c, int nx, int ny, const std::vector<double> &s0, const std::vector<double> &sW,
             const std::vector<double> &sE, const std::vector<double> &sS, const std::vector<double> &sN,
             const std::vector<char> &free_row, int per_x, int per_y, Mg **out) {
  *out = nullptr;
  std::vector<HostLevel> H(1);
  HostLevel &L0 = H[0];
  L0.nx = nx;
  L0.ny = ny;
  L0.per_x = per_x;
  L0.per_y = per_y;
  const int n0 = nx * ny;
  L0.coef.assign((size_t)9 * n0, 0.0);
  L0.active = free_row;
  for (int k = 0; k < n0; k++) {
    if (!free_row[k]) continue;
    const int j = k / nx, i = k - j * nx;
    const int w = i > 0 ? k - 1 : k + nx - 1, e = i < nx - 1 ? k + 1 : k - nx + 1;
    const int s = j > 0 ? k - nx : k + nx * (ny - 1), nn_ = j < ny - 1 ? k + nx : k - nx * (ny - 1);
    L0.coef[(size_t)4 * n0 + k] = s0[k];
    if (free_row[w]) L0.coef[(size_t)3 * n0 + k] += sW[k];
    if (free_row[e]) L0.coef[(size_t)5 * n0 + k] += sE[k];
    if (free_row[s]) L0.coef[(size_t)1 * n0 + k] += sS[k];
    if (free_row[nn_]) L0.coef[(size_t)7 * n0 + k] += sN[k];
  }
  std::vector<int> cxs, cys;
  while (H.back().nx * H.back().ny > kMgCoarsest) {
    const HostLevel &F = H.back();
    const int cx = can_coarsen(F.nx, F.per_x), cy = can_coarsen(F.ny, F.per_y);
    if (!cx && !cy) break;
    cxs.push_back(cx);
    cys.push_back(cy);
    H.push_back(galerkin(F, cx, cy));
  }
  if (H.back().nx * H.back().ny > 4096) return set_err(c, ISKRA_EINVAL, "multigrid: coarsest level too large");
  Mg *m = new Mg();
  m->lv.resize(H.size());
  for (size_t l = 0; l < H.size(); l++) {
    MgLevel &D = m->lv[l];
    const HostLevel &S = H[l];
    D.nx = S.nx;
    D.ny = S.ny;
    D.n = S.nx * S.ny;
    D.per_x = S.per_x;
    D.per_y = S.per_y;
    D.cx = l + 1 < H.size() ? cxs[l] : 0;
    D.cy = l + 1 < H.size() ? cys[l] : 0;
    D.five = 1;
    for (int o : {0, 2, 6, 8})
      for (int k = 0; k < D.n && D.five; k++)
        if (S.coef[(size_t)o * D.n + k] != 0.0) D.five = 0;
    std::vector<float> cf(S.coef.begin(), S.coef.end()), dinv(D.n, 0.f);
    for (int k = 0; k < D.n; k++)
      if (S.active[k] && S.coef[(size_t)4 * D.n + k] > 0) dinv[k] = kMgOmega / (float)S.coef[(size_t)4 * D.n + k];
    bool ok = cudaMalloc(&D.coef, cf.size() * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&D.dinv, D.n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&D.x, D.n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&D.x2, D.n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&D.b, D.n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&D.r, D.n * sizeof(float)) == cudaSuccess;
    if (!ok) {
      mg_destroy(m);
      return set_err(c, ISKRA_ENOMEM, "multigrid levels");
    }
    cudaMemcpy(D.coef, cf.data(), cf.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(D.dinv, dinv.data(), D.n * sizeof(float), cudaMemcpyHostToDevice);
  }
  const std::vector<float> inv = dense_inverse(H.back());
  if (cudaMalloc(&m->cinv, inv.size() * sizeof(float)) != cudaSuccess) {
    mg_destroy(m);
    return set_err(c, ISKRA_ENOMEM, "multigrid coarsest inverse");
  }
  cudaMemcpy(m->cinv, inv.data(), inv.size() * sizeof(float), cudaMemcpyHostToDevice);
  // the single-block bottom: the smallest levels (from level 1 on, so that
  // level 0's FP64 conversions stay in its own kernels), if more than the
  // coarsest one qualifies
  const int L = (int)m->lv.size();
  int l0 = L;
  while (l0 > 1 && m->lv[l0 - 1].n <= kMgBottomNodes) l0--;
  if (l0 <= L - 2) {
    if (cudaMalloc(&m->dlv, L * sizeof(MgLevel)) != cudaSuccess) {
      mg_destroy(m);
      return set_err(c, ISKRA_ENOMEM, "multigrid level table");
    }
    cudaMemcpy(m->dlv, m->lv.data(), L * sizeof(MgLevel), cudaMemcpyHostToDevice);
    m->bottom = l0;
  }
  *out = m;
  return ISKRA_OK;
}

int mg_levels(const Mg *m) { return m ? (int)m->lv.size() : 0; }

static dim3 mg_grid2(int nx, int ny) { return dim3((nx + kMgBx - 1) / kMgBx, (ny + kMgBy - 1) / kMgBy); }

static int mg_smooth(Ctx *c, const MgLevel &D, const float *src, float *dst, const int *skip, const double *r64,
                     double *z64) {
  const dim3 g = mg_grid2(D.nx, D.ny), t(kMgBx, kMgBy);
  if (D.five)
    ISKRA_CUDA(c, launch_pdl(k_mg_smooth<true>, g, t, 0, c->stream, (const float *)D.coef, (const float *)D.dinv, src,
                             dst, D.b, D.nx, D.ny, skip, r64, z64));
  else
    ISKRA_CUDA(c, launch_pdl(k_mg_smooth<false>, g, t, 0, c->stream, (const float *)D.coef, (const float *)D.dinv, src,
                             dst, D.b, D.nx, D.ny, skip, r64, z64));
  return ISKRA_OK;
}

// z = M^-1 r: one V(2,2) cycle on the scaled residual r (FP64, free rows);
// every kernel returns at once while *skip is set (a converged solve).  The
// first sweep of level 0 converts r to FP32, the last one writes z in FP64.
int mg_queue_cycle(Ctx *c, Mg *m, const double *r, double *z, const int *skip) {
  cudaStream_t st = c->stream;
  const int L = (int)m->lv.size();
  const dim3 t(kMgBx, kMgBy);
  auto xfer = [&](int l) {
    const MgLevel &F = m->lv[l], &C = m->lv[l + 1];
    return MgXfer{F.nx, F.ny, C.nx, C.ny, F.cx, F.cy, F.per_x, F.per_y};
  };
  // down: smooth from zero (sweeps alternate x2 <- x <- ..., ending in x),
  // residual, restrict
  static_assert(kMgSweeps % 2 == 0, "an even sweep count leaves the iterate in x");
  const int lb = m->bottom ? m->bottom : L - 1;  // first level not run by per-level kernels
  for (int l = 0; l < lb; l++) {
    MgLevel &D = m->lv[l];
    // the first two sweeps in one launch (into x), then the rest alternating
    const double *r64 = l == 0 ? r : nullptr;
    if (D.five)
      ISKRA_CUDA(c, launch_pdl(k_mg_smooth01<true>, mg_grid2(D.nx, D.ny), t, 0, st, (const float *)D.coef,
                               (const float *)D.dinv, D.x, D.b, D.nx, D.ny, skip, r64));
    else
      ISKRA_CUDA(c, launch_pdl(k_mg_smooth01<false>, mg_grid2(D.nx, D.ny), t, 0, st, (const float *)D.coef,
                               (const float *)D.dinv, D.x, D.b, D.nx, D.ny, skip, r64));
    for (int s = 2; s < kMgSweeps; s++) {
      const float *src = (s & 1) ? D.x2 : D.x;
      float *dst = (s & 1) ? D.x : D.x2;
      const int rc = mg_smooth(c, D, src, dst, skip, nullptr, nullptr);
      if (rc) return rc;
    }
    if (D.five)
      ISKRA_CUDA(c, launch_pdl(k_mg_residual<true>, mg_grid2(D.nx, D.ny), t, 0, st, (const float *)D.coef,
                               (const float *)D.dinv, (const float *)D.x, (const float *)D.b, D.r, D.nx, D.ny, skip));
    else
      ISKRA_CUDA(c, launch_pdl(k_mg_residual<false>, mg_grid2(D.nx, D.ny), t, 0, st, (const float *)D.coef,
                               (const float *)D.dinv, (const float *)D.x, (const float *)D.b, D.r, D.nx, D.ny, skip));
    const MgLevel &C = m->lv[l + 1];
    ISKRA_CUDA(c, launch_pdl(k_mg_restrict, mg_grid2(C.nx, C.ny), t, 0, st, (const float *)D.r, C.b, xfer(l), skip));
  }
  if (m->bottom) {
    ISKRA_CUDA(c, launch_pdl(k_mg_bottom, 1, kMgBottomThreads, 0, st, (const MgLevel *)m->dlv, m->bottom, L,
                             (const float *)m->cinv, skip));
  } else {
    MgLevel &C = m->lv[L - 1];
    ISKRA_CUDA(c, launch_pdl(k_mg_coarse, std::max(1, std::min(c->num_sms * 2, (C.n + 7) / 8)), 256, 0, st,
                             (const float *)m->cinv, (const float *)C.b, C.x, C.n, skip, L == 1 ? r : nullptr,
                             L == 1 ? z : nullptr));
  }
  // up: prolong, smooth
  for (int l = lb - 1; l >= 0; l--) {
    MgLevel &D = m->lv[l];
    ISKRA_CUDA(c, launch_pdl(k_mg_prolong, mg_grid2(D.nx, D.ny), t, 0, st, D.x, (const float *)D.dinv,
                             (const float *)m->lv[l + 1].x, xfer(l), skip));
    for (int s = 0; s < kMgSweeps; s++) {
      const float *src = (s & 1) ? D.x2 : D.x;
      float *dst = (s & 1) ? D.x : D.x2;
      const int rc = mg_smooth(c, D, src, dst, skip, nullptr, (l == 0 && s == kMgSweeps - 1) ? z : nullptr);
      if (rc) return rc;
    }
  }
  ISKRA_CUDA(c, cudaGetLastError());
  return ISKRA_OK;
}

}  // namespace iskra
