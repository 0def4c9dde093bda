/*
 * iskra_oracle.c -- FP64 CPU restatement of iskra's electrostatic PIC step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke entry and the CPU-baseline leg of bench.py load it; the product path
 * (libiskra_gpu.so) never links, loads or calls it.
 *
 * Every function restates one function of the Julia reference (bchaber/iskra),
 * cited by file:line relative to the reference project root.  The arithmetic
 * is plain IEEE double in the same operation order as the Julia source.
 * Arrays follow Julia's layout: column-major, node (i,j) of an (nx,ny) grid at
 * offset (i-1) + nx*(j-1); particle matrices are (ld x D) column-major with the
 * first np rows live (KineticSpecies.x / .v, ParticleInCell/src/pic/kinetic.jl:1-12).
 *
 * Pin status (what checks this restatement against the reference itself):
 *   - Poisson/E-field: the reference's own known-answer test (parallel plate
 *     capacitor, FiniteDifferenceMethod/test/runtests.jl:8-22) -- pinned.
 *   - gather/push/wrap/discard/deposit/cell volume/circuit: analytic
 *     known answers only (free streaming, uniform field, CIC partition of
 *     unity, RLC recurrence) -- parity unpinned against reference output,
 *     because Julia is not installed and the reference ships no fixtures.
 *   - MCC: Julia's default RNG stream cannot be reproduced outside Julia, so
 *     this file draws from its own xoshiro256** generator; MCC parity is
 *     statistical -- parity unpinned.
 *   - Cross sections: Interpolations.jl v0.13 LinearInterpolation with Flat()
 *     extrapolation (Chemistry/src/cross_section.jl:8-14), restated from its
 *     published definition -- parity unpinned.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -shared -fPIC).  OpenMP is used only
 * by the *_omp entry points that bench.py times as the CPU baseline.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX2(i, j, nx) ((int64_t)(i) + (int64_t)(nx) * (int64_t)(j))

/* ------------------------------------------------------------------ */
/* Julia floating-point helpers                                        */
/* ------------------------------------------------------------------ */

/* Julia `mod(x, y)` for floats (Base, float.jl): rem, then shift into y's sign. */
static double jl_mod(double x, double y) {
  double r = fmod(x, y);
  if (r == 0.0) return copysign(0.0, y);
  if ((r > 0.0) != (y > 0.0)) return r + y;
  return r;
}

/* Julia `fld(x, y)` for floats: round((x - mod(x, y)) / y). */
static double jl_fld(double x, double y) {
  return nearbyint((x - jl_mod(x, y)) / y);
}

/* ------------------------------------------------------------------ */
/* particle_cell  -- ParticleInCell/src/ParticleInCell.jl:28-35        */
/* 1-based node index of the lower-left node and the in-cell fraction. */
/* The grid origin is not subtracted (as in the reference).            */
/* ------------------------------------------------------------------ */
void orc_particle_cell(double x, double y, double dx, double dy,
                       int64_t *i, int64_t *j, double *hx, double *hy) {
  double fx = 1.0 + x / dx;
  double fy = 1.0 + y / dy;
  double ix = floor(fx), jy = floor(fy);
  *i = (int64_t)ix;
  *j = (int64_t)jy;
  *hx = fx - ix;
  *hy = fy - jy;
}

/* ------------------------------------------------------------------ */
/* cell_volume -- RegularGrids/src/RegularGrids.jl:26-38               */
/* bcs = {left,right,bottom,top}: nonzero = :periodic.                 */
/* ------------------------------------------------------------------ */
void orc_cell_volume(int nx, int ny, double dx, double dy, const int *bcs,
                     double *V) {
  double V0 = dx * dy;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) V[IDX2(i, j, nx)] = 0.0 + V0;
  if (!bcs[0]) for (int j = 0; j < ny; j++) V[IDX2(0, j, nx)] *= 0.5;
  if (!bcs[1]) for (int j = 0; j < ny; j++) V[IDX2(nx - 1, j, nx)] *= 0.5;
  if (!bcs[2]) for (int i = 0; i < nx; i++) V[IDX2(i, 0, nx)] *= 0.5;
  if (!bcs[3]) for (int i = 0; i < nx; i++) V[IDX2(i, ny - 1, nx)] *= 0.5;
}

/* ------------------------------------------------------------------ */
/* grid_to_particle (CIC gather) -- cloud_in_cell.jl:20-36             */
/* E: (nx,ny,3) column-major.  pu: (ldp x 3) column-major.             */
/* Returns 0, or the 1-based index of the first particle whose cell    */
/* lies outside the grid (Julia would raise BoundsError there).        */
/* ------------------------------------------------------------------ */
static inline double node3(const double *E, int nx, int ny, int64_t i,
                           int64_t j, int c) {
  return E[(i - 1) + (int64_t)nx * (j - 1) + (int64_t)nx * ny * c];
}

int64_t orc_grid_to_particle(int nx, int ny, double dx, double dy,
                             const double *E, int64_t np, int64_t ld,
                             const double *x, double *pu, int64_t ldp) {
  int64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(max : bad)
  for (int64_t p = 0; p < np; p++) {
    int64_t i, j;
    double hx, hy;
    orc_particle_cell(x[p], x[p + ld], dx, dy, &i, &j, &hx, &hy);
    if (i < 1 || j < 1 || i + 1 > nx || j + 1 > ny) {
      if (p + 1 > bad) bad = p + 1;
      continue;
    }
    for (int c = 0; c < 3; c++) {
      pu[p + ldp * c] = (1.0 - hx) * (1.0 - hy) * node3(E, nx, ny, i, j, c) +
                        (hx) * (1.0 - hy) * node3(E, nx, ny, i + 1, j, c) +
                        (1.0 - hx) * (hy) * node3(E, nx, ny, i, j + 1, c) +
                        (hx) * (hy) * node3(E, nx, ny, i + 1, j + 1, c);
    }
  }
  return bad;
}

/* ------------------------------------------------------------------ */
/* push_in_cartesian! (Boris) -- ParticleInCell/src/pic/pushers.jl:37-50 */
/* x: (ld x 2), v: (ld x 3), E,B: (ldp x 3).  Same operation order,    */
/* including v' = v- + v- x B (B, not t, as in the reference).         */
/* ------------------------------------------------------------------ */
void orc_push_cartesian(int64_t np, int64_t ld, double *x, double *v,
                        const double *E, const double *B, int64_t ldp,
                        double qm, double dt) {
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < np; p++) {
    double e[3], b[3], vm[3], t[3], vp[3], s[3], vpl[3];
    for (int c = 0; c < 3; c++) {
      e[c] = E[p + ldp * c];
      b[c] = B ? B[p + ldp * c] : 0.0;
    }
    for (int c = 0; c < 3; c++) vm[c] = 0.5 * dt * qm * e[c] + v[p + ld * c];
    for (int c = 0; c < 3; c++) t[c] = 0.5 * dt * qm * b[c];
    double t2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
    /* v' = v- + v- x B */
    vp[0] = vm[0] + (vm[1] * b[2] - vm[2] * b[1]);
    vp[1] = vm[1] + (vm[2] * b[0] - vm[0] * b[2]);
    vp[2] = vm[2] + (vm[0] * b[1] - vm[1] * b[0]);
    for (int c = 0; c < 3; c++) s[c] = 2.0 / (1.0 + t2) * t[c];
    vpl[0] = vm[0] + (vp[1] * s[2] - vp[2] * s[1]);
    vpl[1] = vm[1] + (vp[2] * s[0] - vp[0] * s[2]);
    vpl[2] = vm[2] + (vp[0] * s[1] - vp[1] * s[0]);
    for (int c = 0; c < 3; c++) v[p + ld * c] = dt * e[c] * qm * 0.5 + vpl[c];
    for (int c = 0; c < 2; c++) x[p + ld * c] = dt * v[p + ld * c] + x[p + ld * c];
  }
}

/* ------------------------------------------------------------------ */
/* remove! -- ParticleInCell/src/pic/kinetic.jl:20-27 (swap-remove)    */
/* ------------------------------------------------------------------ */
static void orc_remove(int64_t *np, int64_t ld, double *x, double *v,
                       double *wg, uint32_t *id, double w0, int64_t i) {
  int64_t last = *np - 1;
  for (int c = 0; c < 2; c++) x[i + ld * c] = x[last + ld * c];
  for (int c = 0; c < 3; c++) v[i + ld * c] = v[last + ld * c];
  if (wg) {
    double t = wg[last];
    wg[last] = w0;
    wg[i] = t;
  }
  if (id) {
    uint32_t t = id[last];
    id[last] = id[i];
    id[i] = t;
  }
  *np = last;
}

/* discard! along one dimension -- ParticleInCell/src/pic/surfaces/wrap.jl:1-18.
 * dim is 0 (x) or 1 (y); n = nodes along dim.  Returns the new np.  The
 * number removed per side goes to removed_lo / removed_hi when non-NULL
 * (alpha < 0 / alpha > 0), for wall-charge accounting. */
int64_t orc_discard(int64_t np, int64_t ld, double *x, double *v, double *wg,
                    uint32_t *id, double w0, int dim, int n, double dh,
                    double origin, int64_t *removed_lo, int64_t *removed_hi) {
  double L = (double)(n - 1) * dh;
  for (int64_t p = np - 1; p >= 0; p--) {
    double a = jl_fld(x[p + ld * dim] - origin, L);
    if (a != 0.0) {
      if (a < 0 && removed_lo) (*removed_lo)++;
      if (a > 0 && removed_hi) (*removed_hi)++;
      orc_remove(&np, ld, x, v, wg, id, w0, p);
    }
  }
  return np;
}

/* wrap! along one dimension -- ParticleInCell/src/pic/surfaces/wrap.jl:20-33 */
void orc_wrap(int64_t np, int64_t ld, double *x, int dim, int n, double dh,
              double origin) {
  double L = (double)(n - 1) * dh;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < np; p++) {
    double a = jl_fld(x[p + ld * dim] - origin, L);
    if (a != 0.0) x[p + ld * dim] -= a * L;
  }
}

/* ------------------------------------------------------------------ */
/* particle_to_grid (CIC deposit) -- cloud_in_cell.jl:1-18             */
/* u (nx,ny) is overwritten.  wg may be NULL (uniform weight w0).      */
/* Returns 0 or the 1-based index of a particle outside the grid.      */
/* ------------------------------------------------------------------ */
int64_t orc_particle_to_grid(int nx, int ny, double dx, double dy, int64_t np,
                             int64_t ld, const double *x, const double *wg,
                             double w0, double *u) {
  memset(u, 0, sizeof(double) * (size_t)nx * ny);
  int64_t bad = 0;
  for (int64_t p = 0; p < np; p++) {
    int64_t i, j;
    double hx, hy;
    orc_particle_cell(x[p], x[p + ld], dx, dy, &i, &j, &hx, &hy);
    if (i < 1 || j < 1 || i + 1 > nx || j + 1 > ny) {
      if (!bad) bad = p + 1;
      continue;
    }
    double w = wg ? wg[p] : w0;
    u[IDX2(i - 1, j - 1, nx)] += (1.0 - hx) * (1.0 - hy) * w;
    u[IDX2(i, j - 1, nx)] += (hx) * (1.0 - hy) * w;
    u[IDX2(i - 1, j, nx)] += (1.0 - hx) * (hy) * w;
    u[IDX2(i, j, nx)] += (hx) * (hy) * w;
  }
  return bad;
}

/* Threaded deposit for the CPU baseline: per-thread private grids summed in
 * thread order (deterministic for a fixed thread count). */
int64_t orc_particle_to_grid_omp(int nx, int ny, double dx, double dy,
                                 int64_t np, int64_t ld, const double *x,
                                 double w0, double *u, int nthreads) {
  size_t ng = (size_t)nx * ny;
  memset(u, 0, sizeof(double) * ng);
  if (nthreads < 1) nthreads = 1;
  double *priv = (double *)calloc(ng * (size_t)nthreads, sizeof(double));
  if (!priv) return -1;
  int64_t bad = 0;
#pragma omp parallel num_threads(nthreads) reduction(max : bad)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    double *g = priv + ng * (size_t)t;
#pragma omp for schedule(static)
    for (int64_t p = 0; p < np; p++) {
      int64_t i, j;
      double hx, hy;
      orc_particle_cell(x[p], x[p + ld], dx, dy, &i, &j, &hx, &hy);
      if (i < 1 || j < 1 || i + 1 > nx || j + 1 > ny) {
        if (p + 1 > bad) bad = p + 1;
        continue;
      }
      g[IDX2(i - 1, j - 1, nx)] += (1.0 - hx) * (1.0 - hy) * w0;
      g[IDX2(i, j - 1, nx)] += (hx) * (1.0 - hy) * w0;
      g[IDX2(i - 1, j, nx)] += (1.0 - hx) * (hy) * w0;
      g[IDX2(i, j, nx)] += (hx) * (hy) * w0;
    }
  }
  for (int t = 0; t < nthreads; t++)
    for (size_t k = 0; k < ng; k++) u[k] += priv[ng * (size_t)t + k];
  free(priv);
  return bad;
}

/* ------------------------------------------------------------------ */
/* calculate_electric_field! -- generalized_poisson.jl:398-410         */
/* phi (nx,ny) -> E (nx,ny,3); E_z = 0.                                */
/* ------------------------------------------------------------------ */
void orc_electric_field(int nx, int ny, double dx, double dy, const double *phi,
                        double *E) {
  size_t ng = (size_t)nx * ny;
  memset(E, 0, sizeof(double) * ng * 3);
  for (int j = 0; j < ny; j++) {
    for (int i = 1; i < nx - 1; i++)
      E[IDX2(i, j, nx)] = (phi[IDX2(i - 1, j, nx)] - phi[IDX2(i + 1, j, nx)]) / (2 * dx);
  }
  for (int j = 1; j < ny - 1; j++)
    for (int i = 0; i < nx; i++)
      E[ng + IDX2(i, j, nx)] = (phi[IDX2(i, j - 1, nx)] - phi[IDX2(i, j + 1, nx)]) / (2 * dy);
  for (int j = 0; j < ny; j++) {
    E[IDX2(0, j, nx)] = (phi[IDX2(0, j, nx)] - phi[IDX2(1, j, nx)]) / dx;
    E[IDX2(nx - 1, j, nx)] = (phi[IDX2(nx - 2, j, nx)] - phi[IDX2(nx - 1, j, nx)]) / dx;
  }
  for (int i = 0; i < nx; i++) {
    E[ng + IDX2(i, 0, nx)] = (phi[IDX2(i, 0, nx)] - phi[IDX2(i, 1, nx)]) / dy;
    E[ng + IDX2(i, ny - 1, nx)] = (phi[IDX2(i, ny - 2, nx)] - phi[IDX2(i, ny - 1, nx)]) / dy;
  }
}

/* ------------------------------------------------------------------ */
/* advance_circuit! -- Circuit/src/Circuit.jl:117-136                  */
/* state = {i, q, t}; vsrc = V(t) evaluated by the caller at the old t. */
/* ------------------------------------------------------------------ */
void orc_advance_circuit(double R, double L, double C, double *state,
                         double vext, double vsrc, double dt) {
  double i = state[0], q = state[1];
  double in = (L / dt - R / 2) * i + vext - vsrc;
  if (C > 0.0) {
    in -= q / C;
    in /= (L / dt + R / 2);
    state[1] = q + dt * i;
  } else {
    in /= (L / dt + R / 2);
  }
  state[0] = in;
  state[2] += dt;
}

/* ================================================================== */
/* Monte Carlo collisions -- Chemistry/src/mcc.jl                     */
/* ================================================================== */

/* CrossSection call: Interpolations.jl LinearInterpolation, Flat() extrapolation
 * (Chemistry/src/cross_section.jl:8-14).  eps nodes strictly increasing. */
double orc_sigma(const double *eps, const double *sig, int n, double e) {
  if (n <= 0) return 0.0;
  if (e <= eps[0]) return sig[0];
  if (e >= eps[n - 1]) return sig[n - 1];
  int lo = 0, hi = n - 1; /* eps[lo] <= e < eps[hi] */
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (eps[mid] <= e) lo = mid; else hi = mid;
  }
  double t = (e - eps[lo]) / (eps[hi] - eps[lo]);
  return (1.0 - t) * sig[lo] + t * sig[hi];
}

/* mass() in eV units -- mcc.jl:26 (qe = 1.60217646e-19 there) */
double orc_mass_ev(double m) { return m / 1.60217646e-19; }

/* thermal_speed -- mcc.jl:74-77 (kB = 1.3806503e-23 there) */
double orc_thermal_speed(double T, double m) {
  double kB = 1.3806503e-23;
  return sqrt(2 * kB * T / m);
}

/* MonteCarloCollisions constructor: max over the union energy grid of
 * sum_k sigma_k(eps) * v(eps) -- mcc.jl:27-51.  tables are concatenated:
 * process k owns nodes [off[k], off[k+1]). */
double orc_mcc_max_sigma_g(int N, const int *off, const double *eps,
                           const double *sig, double m_source) {
  int total = off[N];
  double *e = (double *)malloc(sizeof(double) * (size_t)(total + 1));
  int ne = 0;
  e[ne++] = 0.0;
  for (int k = 0; k < total; k++) e[ne++] = eps[k];
  /* sort + unique */
  for (int a = 1; a < ne; a++) {
    double key = e[a];
    int b = a - 1;
    while (b >= 0 && e[b] > key) { e[b + 1] = e[b]; b--; }
    e[b + 1] = key;
  }
  int u = 0;
  for (int a = 0; a < ne; a++)
    if (a == 0 || e[a] != e[u - 1]) e[u++] = e[a];
  double ms = orc_mass_ev(m_source);
  double alpha = sqrt(2.0 / ms);
  double best = 0.0;
  for (int a = 0; a < u; a++) {
    double v = alpha * sqrt(e[a]);
    double s = 0.0;
    for (int k = 0; k < N; k++)
      s += orc_sigma(eps + off[k], sig + off[k], off[k + 1] - off[k], e[a]) * v;
    if (a == 0 || s > best) best = s;
  }
  free(e);
  return best;
}

/* euler_angles -- mcc.jl:89-106 */
static void euler_angles(const double v[3], double *sth, double *cth,
                         double *sph, double *cph) {
  double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  *cth = v[2] / nv;
  *sth = sqrt(1.0 - (*cth) * (*cth));
  if (*sth == 0.0) { /* isapprox(x, 0.0) with default tolerances is x == 0 */
    *cph = 1.0;
    *sph = 0.0;
  } else {
    *cph = v[0] / nv / *sth;
    *sph = v[1] / nv / *sth;
  }
}

/* [sinχcosη sinχsinη cosχ] * unrotated(θ, ϕ) -- mcc.jl:83-87,108-127 */
static void rotate(double sth, double cth, double sph, double cph, double sch,
                   double cch, double seta, double ceta, double out[3]) {
  double a0 = sch * ceta, a1 = sch * seta, a2 = cch;
  out[0] = a0 * (cph * cth) + a1 * (-sph) + a2 * (cph * sth);
  out[1] = a0 * (-sph * cth) + a1 * (cph) + a2 * (sph * sth);
  out[2] = a0 * (-sth) + a1 * 0.0 + a2 * (cth);
}

/* isotropic_scattering(v) with explicit uniforms u1 (χ) and u2 (η) --
 * mcc.jl:53-62,108-113 (χ uniform in [0,2π), as in the reference). */
void orc_isotropic_scattering(const double v[3], double u1, double u2,
                              double out[3]) {
  double sth, cth, sph, cph;
  euler_angles(v, &sth, &cth, &sph, &cph);
  double chi = 2 * M_PI * u1, eta = 2 * M_PI * u2;
  rotate(sth, cth, sph, cph, sin(chi), cos(chi), sin(eta), cos(eta), out);
}

/* diffuse_reflection(v) with explicit uniforms -- mcc.jl:64-72,122-127 */
void orc_diffuse_reflection(const double v[3], double u1, double u2,
                            double out[3]) {
  double sth, cth, sph, cph;
  euler_angles(v, &sth, &cth, &sph, &cph);
  double sch = sqrt(u1);
  double cch = -sqrt(1.0 - sch * sch);
  double eta = 2 * M_PI * u2;
  rotate(sth, cth, sph, cph, sch, cch, sin(eta), cos(eta), out);
}

/* ---- xoshiro256** (Blackman & Vigna) + Box-Muller normals ---------- */
typedef struct { uint64_t s[4]; int has; double spare; } orc_rng;
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t rng_next(orc_rng *r) {
  uint64_t *s = r->s;
  uint64_t res = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t;
  s[3] = rotl(s[3], 45);
  return res;
}
static double rng_uniform(orc_rng *r) { /* [0,1) */
  return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0);
}
static double rng_normal(orc_rng *r) {
  if (r->has) { r->has = 0; return r->spare; }
  double u1, u2;
  do { u1 = rng_uniform(r); } while (u1 <= 0.0);
  u2 = rng_uniform(r);
  double rad = sqrt(-2.0 * log(u1));
  r->spare = rad * sin(2 * M_PI * u2);
  r->has = 1;
  return rad * cos(2 * M_PI * u2);
}
static void rng_seed(orc_rng *r, uint64_t seed) {
  uint64_t z = seed;
  for (int k = 0; k < 4; k++) { /* splitmix64 */
    z += 0x9e3779b97f4a7c15ULL;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    r->s[k] = x ^ (x >> 31);
  }
  r->has = 0;
}

/* Collision types (mcc.jl:4-8) */
enum { ORC_ELASTIC_ISOTROPIC = 0, ORC_ELASTIC_BACKWARD = 1,
       ORC_INELASTIC_BACKWARD = 2, ORC_EXCITATION = 3, ORC_IONIZATION = 4 };

typedef struct {
  /* source species store, (ld x 2) / (ld x 3) column-major */
  double *x, *v;
  int64_t *np;
  int64_t ld;
  double m, q, w0;
  /* ionisation product (ion) store, may be NULL */
  double *px, *pv;
  int64_t *pnp;
  int64_t pld;
  double pw0;
} orc_species_io;

/* mcc.jl:129-229: one collision of process type on particle p. */
static int perform_collision(int type, double energy, orc_species_io *s, int64_t p,
                             double mt, double Tt, orc_rng *r) {
  double sv[3] = {s->v[p], s->v[p + s->ld], s->v[p + 2 * s->ld]};
  if (type == ORC_ELASTIC_ISOTROPIC || type == ORC_ELASTIC_BACKWARD ||
      type == ORC_INELASTIC_BACKWARD) {
    double mr1 = s->m / (s->m + mt), mr2 = mt / (s->m + mt);
    double vth = orc_thermal_speed(Tt, mt);
    double tv[3];
    for (int c = 0; c < 3; c++) tv[c] = rng_normal(r) * vth;
    double vr[3], w[3], dir[3];
    for (int c = 0; c < 3; c++) { vr[c] = sv[c] - tv[c]; w[c] = mr1 * sv[c] + mr2 * tv[c]; }
    double nvr = sqrt(vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]);
    double scale = nvr;
    if (type == ORC_INELASTIC_BACKWARD) scale = rng_uniform(r) * nvr;
    double u1 = rng_uniform(r), u2 = rng_uniform(r);
    if (type == ORC_ELASTIC_ISOTROPIC) orc_isotropic_scattering(vr, u1, u2, dir);
    else orc_diffuse_reflection(vr, u1, u2, dir);
    for (int c = 0; c < 3; c++) s->v[p + s->ld * c] = w[c] + mr2 * (scale * dir[c]);
    return 0;
  }
  double ms = orc_mass_ev(s->m);
  double sE = 0.5 * ms * (sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]) - energy;
  if (sE < 0) return 0;
  if (type == ORC_EXCITATION) {
    double a = sqrt(2 / ms), ev = a * sqrt(sE), dir[3];
    double u1 = rng_uniform(r), u2 = rng_uniform(r);
    orc_isotropic_scattering(sv, u1, u2, dir);
    for (int c = 0; c < 3; c++) s->v[p + s->ld * c] = ev * dir[c];
    return 0;
  }
  /* ionisation, mcc.jl:174-213 */
  double e1E = sE * rng_uniform(r), e2E = sE - e1E;
  double a = sqrt(2.0 / ms), e1v = a * sqrt(e1E), e2v = a * sqrt(e2E);
  double dir[3], nsv[3];
  double u1 = rng_uniform(r), u2 = rng_uniform(r);
  orc_diffuse_reflection(sv, u1, u2, dir);
  for (int c = 0; c < 3; c++) { nsv[c] = e1v * dir[c]; s->v[p + s->ld * c] = nsv[c]; }
  int64_t q = *s->np;
  if (q >= s->ld) return -1; /* capacity */
  u1 = rng_uniform(r); u2 = rng_uniform(r);
  orc_diffuse_reflection(nsv, u1, u2, dir); /* uses the updated sv, as the reference */
  for (int c = 0; c < 2; c++) s->x[q + s->ld * c] = s->x[p + s->ld * c];
  for (int c = 0; c < 3; c++) s->v[q + s->ld * c] = e2v * dir[c];
  *s->np = q + 1;
  if (s->px) {
    double vth = orc_thermal_speed(Tt, mt), tv[3];
    for (int c = 0; c < 3; c++) tv[c] = rng_normal(r) * vth;
    double mp = s->w0 / s->pw0;
    long cnt = lround(mp);
    for (long k = 0; k < cnt; k++) {
      int64_t iq = *s->pnp;
      if (iq >= s->pld) return -1;
      for (int c = 0; c < 2; c++) s->px[iq + s->pld * c] = s->x[p + s->ld * c];
      for (int c = 0; c < 3; c++) s->pv[iq + s->pld * c] = tv[c];
      *s->pnp = iq + 1;
    }
  }
  return 0;
}

/* PIC.perform!(::MonteCarloCollisions) -- mcc.jl:231-289.
 * E: (nx,ny,3); n_gas: (nx,ny) node density of the target fluid.
 * counts[k] accumulates accepted collisions of process k.  remainder is the
 * carried fractional draw count (mcc.remainder).  Returns 0, -1 on capacity
 * overflow, -2 when max_Pt > 1/N or P_k > 1 (the reference's @assert). */
int orc_mcc_perform(int nx, int ny, double dx, double dy, const double *E,
                    const double *n_gas, int N, const int *types,
                    const double *energies, const int *off, const double *eps,
                    const double *sig, double max_sigma_g, double *remainder,
                    double dt, double *sx, double *sv, int64_t *snp, int64_t sld,
                    double sm, double sq, double sw0, double *px, double *pv,
                    int64_t *pnp, int64_t pld, double pw0, double tm, double tq,
                    double tT, uint64_t seed, int64_t *counts, double *nu) {
  orc_rng r;
  rng_seed(&r, seed);
  orc_species_io s = {sx, sv, snp, sld, sm, sq, sw0, px, pv, pnp, pld, pw0};
  double max_n = n_gas[0];
  for (int64_t k = 1; k < (int64_t)nx * ny; k++) if (n_gas[k] > max_n) max_n = n_gas[k];
  double maxPt = 1.0 - exp(-max_n * max_sigma_g * dt);
  if (maxPt > 1.0 / N) return -2;
  double total = N * maxPt * (double)(*snp) + *remainder;
  double Nc = floor(total); /* modf for non-negative values */
  *remainder = total - Nc;
  double m_ev = orc_mass_ev(sm);
  for (int64_t d = 0; d < (int64_t)Nc; d++) {
    int64_t p = (int64_t)(rng_uniform(&r) * (double)(*snp)); /* rand(1:np) */
    if (p >= *snp) p = *snp - 1;
    int64_t i, j;
    double hx, hy;
    orc_particle_cell(sx[p], sx[p + sld], dx, dy, &i, &j, &hx, &hy);
    double n = n_gas[IDX2(i - 1, j - 1, nx)];
    if (n < 0) continue;
    double U = rng_uniform(&r);
    int k = (int)floor(N * U + 1);
    double g2 = 0.0;
    for (int c = 0; c < 3; c++) {
      double tvc = (tq / tm) * node3(E, nx, ny, i, j, c) * dt;
      double dv = tvc - sv[p + sld * c];
      g2 += dv * dv;
    }
    double g = sqrt(g2);
    double e = 0.5 * m_ev * g * g;
    double sg = orc_sigma(eps + off[k - 1], sig + off[k - 1], off[k] - off[k - 1], e) * g;
    double Pk = 1.0 - exp(-n * sg * dt);
    Pk /= N * maxPt;
    if (Pk > 1.0) return -2;
    if (U > (double)k / N - Pk) {
      if (perform_collision(types[k - 1], energies[k - 1], &s, p, tm, tT, &r) < 0) return -1;
      counts[k - 1]++;
      if (nu) nu[IDX2(i - 1, j - 1, nx) + (int64_t)nx * ny * (k - 1)] += 1;
    }
  }
  return 0;
}

/* Uniform [0,1) and standard-normal draws from the oracle generator, for
 * seeded test inputs (Maxwellian loading, sources.jl:24-34 semantics). */
void orc_fill_uniform(uint64_t seed, int64_t n, double *out) {
  orc_rng r;
  rng_seed(&r, seed);
  for (int64_t k = 0; k < n; k++) out[k] = rng_uniform(&r);
}
void orc_fill_normal(uint64_t seed, int64_t n, double *out) {
  orc_rng r;
  rng_seed(&r, seed);
  for (int64_t k = 0; k < n; k++) out[k] = rng_normal(&r);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
