/*
 * iskra_gpu.h -- C ABI of libiskra_gpu.so, the GB300 (sm_103a) implementation
 * of iskra's electrostatic particle-in-cell step.
 *
 * Each entry point replaces one call of the Julia reference (bchaber/iskra);
 * the cited reference function is the one a ccall-based Julia shim would route
 * to it (paths relative to the reference project root).
 *
 * Conventions
 *   - Every call returns an int status: ISKRA_OK (0) or one of ISKRA_E*.
 *     iskra_last_error(ctx) gives the message of the last failure on ctx.
 *     No call aborts the process or traps the GPU.
 *   - Host arrays use Julia's layout: column-major Float64, node (i,j) of an
 *     (nx,ny) grid at offset (i-1) + nx*(j-1); particle matrices are
 *     (ld x D) with the first np rows live (KineticSpecies.x/.v).  Host
 *     pointers are borrowed for the duration of the call only.
 *   - The library owns all device memory behind iskra_ctx.  One context is
 *     one CUDA stream; calls on a context are not re-entrant.  Asynchronous
 *     calls (marked "async") return once work is queued on the stream; device
 *     error flags raised by that work are reported by the next synchronising
 *     call (iskra_sync, any download, or iskra_status).
 */
#ifndef ISKRA_GPU_H
#define ISKRA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define ISKRA_OK 0
#define ISKRA_EINVAL 1     /* bad argument or unsupported configuration      */
#define ISKRA_ENOMEM 2     /* device or host allocation failed               */
#define ISKRA_ECAPACITY 3  /* species capacity exceeded (particles dropped)  */
#define ISKRA_EDOMAIN 4    /* particle left the grid on an axis without
                              wrap!/discard! (Julia raises BoundsError)       */
#define ISKRA_EPROB 5      /* MCC probability bound violated
                              (Chemistry/src/mcc.jl:244-246,272-279)          */
#define ISKRA_ENAN 6       /* non-finite value in particle or field data     */
#define ISKRA_ETIMEDOUT 7  /* a bounded device wait gave up                  */
#define ISKRA_ECUDA 8      /* CUDA runtime error                             */
#define ISKRA_ENOTCONV 9   /* Poisson iteration did not reach the tolerance  */

/* after_push boundary mode per axis (ParticleInCell/src/pic/surfaces/wrap.jl) */
#define ISKRA_BND_NONE 0
#define ISKRA_BND_WRAP 1    /* wrap!    wrap.jl:20-33 */
#define ISKRA_BND_DISCARD 2 /* discard! wrap.jl:1-18  */

/* Surface kinds of the surface tracker (pic/surfaces/build.jl:8-11,
 * circuit_coupling.jl:4-16) */
#define ISKRA_SURF_ABSORB 1   /* AbsorbingSurface: hit! removes the particle      */
#define ISKRA_SURF_REFLECT 2  /* ReflectiveSurface: mirrors the rest of the step  */
#define ISKRA_SURF_PERIODIC 3 /* PeriodicSurface: hit! does nothing, tracking ends */
#define ISKRA_SURF_FIXED 4    /* FixedPotentialElectrode: absorbs                 */
#define ISKRA_SURF_FLOATING 5 /* FloatingPotentialElectrode: absorbs, σ += q w / area */

/* MCC process types (Chemistry/src/mcc.jl:4-8) */
#define ISKRA_MCC_ELASTIC_ISOTROPIC 0
#define ISKRA_MCC_ELASTIC_BACKWARD 1
#define ISKRA_MCC_INELASTIC_BACKWARD 2
#define ISKRA_MCC_EXCITATION 3
#define ISKRA_MCC_IONIZATION 4

/* Field selectors for iskra_field_download */
#define ISKRA_FIELD_RHO 0 /* ρ (nx,ny)             ParticleInCell.jl:118-122  */
#define ISKRA_FIELD_PHI 1 /* ϕ (nx,ny)             generalized_poisson.jl:377 */
#define ISKRA_FIELD_E 2   /* E (nx,ny,3) FP64      generalized_poisson.jl:398 */

typedef struct iskra_ctx iskra_ctx;

/* Uniform Cartesian grid: RegularGrids.create_uniform_grid(xs, ys; left,
 * right, bottom, top) (RegularGrids/src/RegularGrids.jl:55-69).  bc[k] != 0
 * marks side k (left,right,bottom,top) :periodic; only cell_volume reads it
 * (RegularGrids.jl:26-38).  The origin must be (0,0): particle_cell ignores it
 * (ParticleInCell.jl:28-35) while wrap!/discard! use it, so other origins
 * are inconsistent in the reference itself. */
typedef struct {
  int32_t nx, ny;   /* nodes; 2 <= nx <= 65535, 2 <= ny <= 32768, nx*ny <= 2^30 */
  double dx, dy;    /* node spacing (Δh) */
  double ox, oy;    /* origin, must be 0 */
  int32_t bc[4];
} iskra_grid_t;

/* ---- context ------------------------------------------------------------ */
/* Creates the device context for one grid on the current CUDA device.
 * stream: a cudaStream_t to run on, or 0 for a library-owned stream. */
int iskra_ctx_create(const iskra_grid_t *grid, uint64_t stream, iskra_ctx **out);
int iskra_ctx_destroy(iskra_ctx *ctx);
const char *iskra_last_error(const iskra_ctx *ctx);
/* Waits for queued work, then reports device error flags (clearing them). */
int iskra_sync(iskra_ctx *ctx);
/* The cudaStream_t (as an integer) all work of ctx is queued on. */
int iskra_stream(iskra_ctx *ctx, uint64_t *stream);

/* ---- kinetic species (ParticleInCell/src/pic/kinetic.jl:1-18) ----------- */
/* KineticSpecies{2,3}(name, capacity) with charge q, mass m, default weight
 * w0 (create_kinetic_species, problem/configuration.jl:141-148).  Particles
 * are stored on the device as a cell index plus FP32 in-cell offsets and FP32
 * velocities; every macroparticle carries the weight w0. */
int iskra_species_create(iskra_ctx *ctx, double q, double m, double w0,
                         int64_t capacity, int *sid);
/* Copies np particles in: x (ld x 2) and v (ld x 3) column-major Float64,
 * wg (np, may be NULL; every entry must equal w0), id (np, may be NULL ->
 * 1..np).  Replaces the previous content.  Particles are cell-sorted. */
int iskra_species_upload(iskra_ctx *ctx, int sid, const double *x,
                         const double *v, const double *wg, const uint32_t *id,
                         int64_t np, int64_t ld);
/* Copies the live particles out (compacting first); *np receives the count.
 * Fails with ISKRA_ECAPACITY if ld is too small (nothing written then). */
int iskra_species_download(iskra_ctx *ctx, int sid, double *x, double *v,
                           double *wg, uint32_t *id, int64_t ld, int64_t *np);
/* Live particle count (synchronises). */
int iskra_species_count(iskra_ctx *ctx, int sid, int64_t *np);
/* after_push(part, grid) for this species: per-axis wrap!/discard!/none. */
int iskra_species_set_boundary(iskra_ctx *ctx, int sid, int mode_x, int mode_y);
/* Particles removed by discard! since the last call, per wall
 * {x-low, x-high, y-low, y-high}; the counter is reset. */
int iskra_species_absorbed(iskra_ctx *ctx, int sid, int64_t counts[4]);
/* Counting sort by cell + compaction of discarded particles (async). */
int iskra_species_sort(iskra_ctx *ctx, int sid);

/* ---- surface tracker (pic/surfaces/*.jl, circuit_coupling.jl:45-63) ------
 * With a tracker, every push (iskra_advance, iskra_advance_all, iskra_step)
 * runs track! + check! (track.jl:39-52, check.jl:39-68): a particle whose
 * cell borders a surface edge has its straight path from the old position
 * with the new velocity walked cell by cell; at a surface edge hit!
 * (hit.jl:33-56, circuit_coupling.jl:45-63) absorbs it (ABSORB, FIXED,
 * FLOATING -- the floating electrode's σ dof then gains q w / area before
 * the step's field solve), reflects it (REFLECT: the rest of the step
 * mirrored, the normal velocity component flipped, tracking continues) or
 * ends its tracking (PERIODIC).  after_push (wrap!/discard!) follows.
 * create_surface_tracker(grid, ds) (build.jl:91-97): the domain walls get
 * surface kind default_kind (ISKRA_SURF_ABSORB in the reference). */
int iskra_tracker_create(iskra_ctx *ctx, int default_kind);
/* track_surface!(tracker, bcs, ss) (build.jl:104-106, build_surface_lookup!
 * :41-57) and the tracker half of create_electrode (problem/
 * configuration.jl:22-38): every cell edge whose two end nodes are set in
 * nodes (nx*ny bytes, Julia layout) becomes surface `kind`, replacing what
 * the edge had.  FLOATING: sigma_dof (1-based σ dof of the Poisson solver,
 * add_new_dof) and area (electrode area, configuration.jl:43-51).  *surface
 * receives the surface's index (0-based). */
int iskra_tracker_add_surface(iskra_ctx *ctx, const uint8_t *nodes, int kind,
                              int sigma_dof, double area, int *surface);
/* Particles of species sid absorbed by `surface` since the tracker was
 * created (synchronises). */
int iskra_tracker_hits(iskra_ctx *ctx, int surface, int sid, int64_t *count);

/* ---- particle sources (pic/sources.jl, problem/configuration.jl:89-93) ----
 * MaxwellianSource{2,3}(rate, wx, wv; dx, dv) (sources.jl:8-22) feeding
 * species sid; create_thermalized_beam passes wv = sqrt(2 kB T / m) per
 * component and dv = the beam velocity.  dx, dv may be NULL (zeros).
 * *src receives the source index. */
int iskra_source_create(iskra_ctx *ctx, int sid, double rate, const double wx[2],
                        const double dx[2], const double wv[3], const double dv[3],
                        int *src);
/* sample!(src, species, Δt) (sources.jl:24-34): min(free slots,
 * floor(rate Δt)) particles appended, x = U(0,1) wx + dx, v = N(0,1) wv + dv,
 * identifiers continuing the species' counter; init(src, species, Δt)
 * (ParticleInCell.jl:47-49) is one such call.  Philox keyed by seed and the
 * call number.  A position outside the grid is ISKRA_EDOMAIN. (async) */
int iskra_source_sample(iskra_ctx *ctx, int src, double dt, uint64_t seed);
/* on != 0: iskra_step samples the source at the start of every step, before
 * the MCC sets (the sources loop of ParticleInCell.solve, :104-106), keyed
 * by the step's seed and the device step counter. */
int iskra_source_set_every_step(iskra_ctx *ctx, int src, int on);

/* ---- fields -------------------------------------------------------------- */
/* Replaces the device E field used by the gather with a host (nx,ny,3) array
 * (the E argument of advance!, ParticleInCell.jl:51-57).  E_z is ignored: the
 * 2D xy push never reads a nonzero E_z from the reference's solver. */
int iskra_field_upload_E(iskra_ctx *ctx, const double *E);
/* Copies ρ, ϕ or E (FP64) to the host (synchronises). */
int iskra_field_download(iskra_ctx *ctx, int which, double *out);
/* Same without waiting: the field as the calls queued so far leave it is
 * snapshotted on the device and copied to `out` while later calls (steps)
 * run; `out` holds it after the next synchronising call (iskra_sync, a
 * blocking download or count) and must stay valid until then.  Pinned host
 * memory makes the copy overlap; a later non-blocking download first waits
 * for this one's copy. */
int iskra_field_download_async(iskra_ctx *ctx, int which, double *out);

/* ---- ParticleInCell.advance!(::KineticSpecies, E, B, Δt, config) --------
 * ParticleInCell.jl:51-72: grid_to_particle (cloud_in_cell.jl:20-36), Boris
 * push with B = 0 (pushers.jl:37-50, calculate_magnetic_field
 * generalized_poisson.jl:412-419), after_push (wrap.jl).  The same kernel
 * deposits the pushed particles (cloud_in_cell.jl:1-18) into the species'
 * int64 fixed-point density accumulator, consumed by iskra_density. (async) */
int iskra_advance(iskra_ctx *ctx, int sid, double dt);
/* The same for every species (the loop over species of
 * ParticleInCell.solve, ParticleInCell.jl:113-115); two species with the
 * same boundary rules are pushed by one launch, as inside iskra_step. (async) */
int iskra_advance_all(iskra_ctx *ctx, double dt);

/* ---- density(species, grid) = particle_to_grid(wg) ./ cell_volume -------
 * kinetic.jl:53, cloud_in_cell.jl:1-18, RegularGrids.jl:26-38.  Writes the
 * (nx,ny) density to n_out when non-NULL (synchronises then). */
int iskra_density(iskra_ctx *ctx, int sid, double *n_out);
/* ρ = Σ_s q_s n_s over all kinetic species plus an optional fixed background
 * set by iskra_set_background (ParticleInCell.jl:118-122). (async) */
int iskra_charge_density(iskra_ctx *ctx);
/* Fixed (nx,ny) charge density added to ρ (a neutralising fluid species with
 * constant n, fluid.jl:1-11); NULL clears it. */
int iskra_set_background(iskra_ctx *ctx, const double *rho_bg);

/* ---- Poisson solver (FiniteDifferenceMethod/src/generalized_poisson.jl) -- */
/* create_poisson_solver(grid, ε0) (:27-30,34-68). */
int iskra_poisson_create(iskra_ctx *ctx, double eps0);
/* apply_dirichlet(ps, nodes, ϕ0) (:205-215); nodes: (nx,ny) uint8 mask. */
int iskra_poisson_apply_dirichlet(iskra_ctx *ctx, const uint8_t *nodes,
                                  double phi0);
/* apply_periodic(ps, axis) (:286-324), axis 1 or 2 in the reference's naming. */
int iskra_poisson_apply_periodic(iskra_ctx *ctx, int axis);
/* add_new_dof(ps, :σ) (:217-230); *dof receives the 1-based σ index. */
int iskra_poisson_add_dof(iskra_ctx *ctx, int *dof);
/* apply_neumann(ps, nodes, dof) (:235-269). */
int iskra_poisson_apply_neumann(iskra_ctx *ctx, const uint8_t *nodes, int dof);
/* apply_neumann(ps, nodes, dof) (:235-269) in units consistent with the
 * stencil rows and a σ in C/m^2 (the units advance!(::CircuitRLC) and hit!
 * credit it in, circuit_coupling.jl:35-55): the Gauss law of the electrode
 * node's half cell, -2/Δx^2 ϕ_i + 2/Δx^2 ϕ_i' + 2/(ε0 Δx) σ = -ρ_i/ε0 (the
 * reference's edge row divided by Δx, its σ coefficient 2 replaced by
 * 2/(ε0 Δx)); corner rows divide their σ coefficient by ε0.  The reference's
 * own rows mix a potential gradient with -ρ/ε0 and an undivided σ, which
 * drives a floating electrode to tens of kV within a few steps of a
 * discharge; circuit runs use this form. */
int iskra_poisson_apply_neumann_gauss(iskra_ctx *ctx, const uint8_t *nodes,
                                      int dof);
/* get_rhs(ps, :σ, dof) read / write (:367-370). */
int iskra_poisson_set_sigma(iskra_ctx *ctx, int dof, double value);
int iskra_poisson_get_sigma(iskra_ctx *ctx, int dof, double *value);
/* Time-dependent Dirichlet group for the graph-captured step: nodes get
 * ϕ0(t) = amp*sin(2π f t + phase) + dc at t = (step-1)*Δt, i.e. the
 * `apply_dirichlet(solver, nodes, V(t))` call of a problem's iteration hook
 * (problem/11_rf_discharge.jl:93). */
int iskra_poisson_drive_dirichlet(iskra_ctx *ctx, const uint8_t *nodes,
                                  double amp, double freq, double phase,
                                  double dc);
/* calculate_electric_potential(ps, -ρ) (:372-378) with the device ρ, iterated
 * to relative residual rtol (FP64), followed by calculate_electric_field
 * (:398-410).  iters/relres may be NULL; non-NULL makes the call synchronous. */
int iskra_poisson_solve(iskra_ctx *ctx, double rtol, int maxit, int *iters,
                        double *relres);
/* Same with a host right-hand side f (the argument of
 * calculate_electric_potential) and the potential written to phi_out. */
int iskra_poisson_solve_host(iskra_ctx *ctx, const double *f, double rtol,
                             int maxit, double *phi_out, int *iters,
                             double *relres);
/* Initial guess of the solves inside iskra_step: 0 = the previous step's ϕ,
 * 1 = ϕ extrapolated linearly from the last two steps, 2 ϕ_n - ϕ_(n-1)
 * (default; either way the solve iterates to the same tolerance). */
int iskra_poisson_set_warm_start(iskra_ctx *ctx, int mode);
/* Solver method: 0 = automatic (the exact FFT(y)/tridiagonal(x) solve when
 * the assembled operator is separable, else CG preconditioned by a geometric
 * multigrid V-cycle, or CG with Jacobi scaling when the operator is singular),
 * 1 = CG with Jacobi scaling only, 2 = multigrid-preconditioned CG even for
 * a separable operator.  Every method iterates to the same FP64 relative
 * residual.  Returns the method in effect through *active when non-NULL
 * (0 separable, 1 Jacobi CG, 2 multigrid CG). */
int iskra_poisson_set_method(iskra_ctx *ctx, int method, int *active);

/* ---- Monte Carlo collisions (Chemistry/src/mcc.jl) ----------------------- */
/* mcc(@reactions ...) -> MonteCarloCollisions (:27-51,291-320) for one source
 * species against a fluid target.  Process k has type types[k], energy
 * energies[k] (threshold for excitation/ionisation) and the cross-section
 * table eps[off[k]..off[k+1]), sigma[...] (CrossSection, cross_section.jl).
 * gas_n: (nx,ny) target density (FluidSpecies.n).  product_sid: species that
 * receives ionisation ions (-1 none).  max_sigma_g (may be NULL) receives the
 * constructor's max Σσ_k g. */
int iskra_mcc_create(iskra_ctx *ctx, int source_sid, int nproc,
                     const int *types, const double *energies,
                     const int32_t *off, const double *eps,
                     const double *sigma, double gas_mass, double gas_T,
                     double gas_q, const double *gas_n, int product_sid,
                     double *max_sigma_g, int *mid);
/* PIC.perform!(::MonteCarloCollisions, E, Δt, config) (:231-289): the
 * null-collision step on the current E with a counter-based RNG keyed by
 * (seed, step, particle id). (async) */
int iskra_mcc_perform(iskra_ctx *ctx, int mid, double dt, uint64_t seed,
                      uint64_t step);
/* Accepted collisions per process since the last call (reset after). */
int iskra_mcc_counts(iskra_ctx *ctx, int mid, int64_t *counts);
/* The rate call (process.rate)(ε) of CrossSection (cross_section.jl:8-16:
 * linear interpolation, flat outside the table) as the MCC kernels evaluate
 * it -- FP32 table of set mid, process `process` (0-based) -- at n energies
 * (eV); sigma_out[k] = σ(energies[k]) in m^2.  (synchronises) */
int iskra_mcc_sigma(iskra_ctx *ctx, int mid, int process,
                    const double *energies, int64_t n, double *sigma_out);

/* ---- DSMC (Chemistry/src/dsmc.jl) ----------------------------------------
 * DSMC.ElasticCollision(rate, source, target) of dsmc(@reactions ...)
 * (dsmc.jl:1-13, :140-166) between two kinetic species (source may equal
 * target): rate is the CrossSection with nodes (g[k], sigma[k]), k < n, g
 * increasing (cross_section.jl:8-16: linear, flat outside).  *set receives
 * the set's index. */
int iskra_dsmc_create(iskra_ctx *ctx, int source, int target, const double *g,
                      const double *sigma, int n, int *set);
/* PIC.perform!(dsmc, E, Δt, config) (dsmc.jl:86-138) for one set: per cell
 * Nc = na Nb Δt σgmax / (Pab + (Wb/Wa) Pba) (x2 for two species) plus the
 * carried remainder, floor(Nc) random pairs accepted with probability
 * σ(g) g / σgmax and scattered isotropically in the CM frame
 * (perform!(::ElasticCollision), :31-84).  Philox keyed by (seed, set,
 * step, cell, pair).  iskra_step performs every set each step, after the MCC
 * sets and before the push, keyed by the device step counter. (async) */
int iskra_dsmc_perform(iskra_ctx *ctx, int set, double dt, uint64_t seed,
                       uint64_t step);
/* collisions_remaining (nx*ny FP64) and the accepted collisions of the last
 * perform! per cell (nx*ny, the "nuDSMC" field); either may be NULL.
 * Cells are numbered like nodes: the reference's cell (i, j) is entry
 * (i-1) + nx (j-1). (synchronises) */
int iskra_dsmc_state(iskra_ctx *ctx, int set, double *remaining, uint32_t *nu);

/* ---- RLC circuit (Circuit/src/Circuit.jl, circuit_coupling.jl) ---------- */
/* rlc(@netlist ...) with V(t) = amp*sin(2π f t) + dc, coupled to the σ dof
 * of a floating electrode (positive) and a grounded node set (negative), as a
 * PlasmaDevice (circuit_coupling.jl:18-33).  area: electrode area.
 * sigma_scale multiplies dσ before it enters the σ row (1 = the reference). */
int iskra_circuit_create(iskra_ctx *ctx, double R, double L, double C,
                         double amp, double freq, double dc, int sigma_dof,
                         const uint8_t *pos_nodes, const uint8_t *neg_nodes,
                         double area, double sigma_scale);
/* advance!(circuit, ϕ, Δt, config) (circuit_coupling.jl:35-43 ->
 * Circuit.jl:117-136), FP64, one device thread. (async) */
int iskra_circuit_advance(iskra_ctx *ctx, double dt);
/* {t, i, q, σ, V_ext} */
int iskra_circuit_state(iskra_ctx *ctx, double state[5]);

/* ---- whole step: the loop body of ParticleInCell.solve (:102-135) -------
 * MCC sets (in creation order) -> advance! every species -> circuit ->
 * density/ρ -> Poisson -> E, nsteps times, replayed as one CUDA graph.
 * seed keys the MCC RNG; the step counter continues across calls. (async) */
int iskra_step(iskra_ctx *ctx, double dt, int nsteps, uint64_t seed,
               double rtol);
/* Tile-sort cadence for iskra_step: every > 0 sorts every species each
 * `every` steps, 0 never, < 0 (default) per species from its rms speed.
 * Sorting only reorders particles in memory; the deposit is order-independent. */
int iskra_set_sort_every(iskra_ctx *ctx, int every);
/* Autotunes the sort cadence on the caller's own run: `trial` steps (as
 * iskra_step with dt, seed, rtol) under each factor 0.5, 1, 2, 4 on the
 * speed-based per-species sort periods, each after a sort of every species,
 * timed on the device; keeps the fastest and returns it with its time per
 * step.  Advances the simulation by 4 (trial + 1) steps; results do not
 * depend on the cadence (the sort is a permutation).  Needs the automatic
 * cadence (iskra_set_sort_every(ctx, -1)). */
int iskra_autotune_sort(iskra_ctx *ctx, double dt, int trial, uint64_t seed,
                        double rtol, double *scale, double *ms_per_step);
/* Push tile size (no reference counterpart): tiles of `cells` x `cells`
 * cells, 8, 16 (default) or 32.  Re-sorts every species by the new tiles
 * and rebuilds the step graph; results do not depend on it (the tile decides
 * which block pushes a particle, never how). */
int iskra_set_tile(iskra_ctx *ctx, int cells);
int iskra_get_tile(iskra_ctx *ctx, int *cells);
/* Autotunes the push tile size and the sort cadence together on the
 * caller's own run: `trial` steps (as iskra_step with dt, seed, rtol) per
 * candidate -- tiles of 8, 16, 32 cells x factors 0.5, 1, 2, 4 on the
 * speed-based sort periods -- each after a sort of every species, timed on
 * the device; keeps the fastest pair and returns it (tile, scale) with its
 * time per step; ms_all (12 entries, tile-major, may be NULL) receives every
 * candidate's time.  The choice is cached for the process by (grid,
 * species count, particles per cell rounded to a power of two, tracker): a
 * later call for the same shape applies it without trials (*cached = 1).
 * Advances the simulation by 12 (trial + 1) steps unless cached.  Needs the
 * automatic cadence. */
int iskra_autotune(iskra_ctx *ctx, double dt, int trial, uint64_t seed,
                   double rtol, int *tile, double *scale, double *ms_per_step,
                   double *ms_all, int *cached);
/* Last Poisson solve: iterations and relative residual (synchronises). */
int iskra_solve_info(iskra_ctx *ctx, int *iters, double *relres);
/* Relative residual of a host potential phi (nx,ny) against the assembled
 * system of calculate_electric_potential(ps, f) (generalized_poisson.jl:
 * 372-378: b[ρ] = f/ε0, identity rows their values, σ the current σ), as
 * the solver's tolerance measures it: ||b' - A' ϕ|| / ||b'|| over the
 * non-identity rows, with the identity rows' values and the σ terms moved
 * into b'.  Evaluated in FP64 on the host: the accuracy check of a potential
 * computed elsewhere (another context, an ensemble run).  Singular
 * (all-periodic) operators are measured without the gauge shift. */
int iskra_poisson_residual(iskra_ctx *ctx, const double *f, const double *phi,
                           double *relres);
/* Diagnostic with no reference counterpart: number of kernels iskra_step has
 * launched on this context (graph replays x kernel nodes). */
int iskra_kernel_launches(iskra_ctx *ctx, uint64_t *count);

/* ---- diagnostics: openPMD records as HDF5 (Diagnostics/src/hdf5.jl) ------
 * new_iteration(prefix, i, t, dt) (:47-66) with save_record of every field
 * and particle record (:69-101) and the metadata of Diagnostics/src/openpmd:
 * writes <prefix>/hdf5/data<iteration>.h5 holding, under /data/<iteration>/,
 * fields/{rho, phi, E/{x,y,z}, n<species>, nuMCC-<species>-<k>} (the MCC
 * counts accumulated since the previous record; the reference writes every
 * step's), the circuit's fields/{Q1, I1, V1, Vext} when one is attached and,
 * when particles != 0, particles/<species>/{position/{x,y}, momentum/{x,y,z},
 * weighting, id, charge, mass, positionOffset/{x,y,z}}.  Field arrays in
 * Julia memory order (HDF5 dimensions (ny, nx)).  species_names: one name
 * per species (NULL: "s0", "s1", ...).  The file is laid out from the
 * published HDF5 file format (version 2 superblock and object headers,
 * compact groups, contiguous FP64 datasets); no HDF5 library is linked.
 * (synchronises) */
int iskra_write_openpmd(iskra_ctx *ctx, const char *prefix, int64_t iteration,
                        double time, double dt,
                        const char *const *species_names, int particles);

/* ---- density without device allocation -----------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: a host framework that reserves the GPU's memory up front and
 * forbids later cudaMalloc, or code running while another library holds the
 * stream in capture.  The density of iskra_density (CIC deposit ./
 * cell_volume on int64 fixed-point sums) for the np particles whose
 * positions x (ld x 2, column-major FP64) are in DEVICE memory: bit-identical
 * below 2^15 particles; from 2^15 on each CIC weight is rounded to
 * 2^(s-48) with s = ceil(log2(np+1)) - 15 so that no node sum can overflow,
 * i.e. equal within 2^(s-48) relative per particle.  The grid's origin must
 * be (0,0) as for iskra_ctx_create.  The (nx,ny) density goes to n_out
 * (device memory); *flag (device int) is set to 1 when a position lies
 * outside the grid (that particle is skipped), else 0.
 * Allocates nothing: the accumulator is a library-static device array of
 * 2^20 nodes (8 MiB, held on every GPU that loads the library until exit);
 * larger grids return ISKRA_EINVAL.  The first call on a device looks the
 * array's address up (cudaGetSymbolAddress): make that first call before any
 * stream capture; the address is cached for the device's primary context,
 * which must outlive every call (no cudaDeviceReset in between).  Each call clears the array it shares with every other
 * call; calls that overlap on the GPU race.  Asynchronous on `stream`. */
int iskra_density_noalloc(const iskra_grid_t *grid, const double *x,
                          int64_t np, int64_t ld, double w0, double *n_out,
                          int *flag, uint64_t stream);

/* ---- batched ensembles (config C4: many independent small discharges) ----
 * No single reference counterpart: the reference runs one problem per
 * process; this is the GPUEnsemble drop-in of the batched configuration.  An
 * ensemble copies a configured template context -- species (q, m, w0,
 * boundary rules), MCC sets (mcc.jl:27-51), the assembled Poisson operator
 * with its driven electrodes -- and holds nruns independent runs of it, each
 * with its own particles, fields, MCC seed (default 1000 + run) and drive
 * amplitudes.  One iskra_ens_step advances every run by the reference's loop
 * body (ParticleInCell.jl:102-135: MCC, advance!, ρ, ϕ, E) in one CUDA graph.
 * Runs with the same seed and initial state follow the same algorithm as a
 * single-run context.  Limits: at most 400 cells per run; separable operator
 * with ny <= 16, no x-periodic wrap, no σ dof (electrodes are Dirichlet,
 * possibly driven); no circuit, surface tracker, particle source or DSMC
 * set.  The template context must outlive the
 * ensemble; the ensemble uses the template's stream. */
typedef struct iskra_ens iskra_ens;
int iskra_ens_create(iskra_ctx *tmpl, int nruns, int64_t capacity_per_run,
                     iskra_ens **out);
int iskra_ens_destroy(iskra_ens *ens);
const char *iskra_ens_last_error(const iskra_ens *ens);
/* seeds[nruns] of the MCC random streams (keys as in iskra_step) */
int iskra_ens_set_seeds(iskra_ens *ens, const uint64_t *seeds);
/* amplitude amp[nruns] of driven-electrode group `group` (0-based, creation
 * order of iskra_poisson_drive_dirichlet) */
int iskra_ens_set_drive_amplitude(iskra_ens *ens, int group, const double *amp);
/* particles of one run, layouts as iskra_species_upload / _download */
int iskra_ens_upload(iskra_ens *ens, int run, int sid, const double *x,
                     const double *v, const uint32_t *id, int64_t np,
                     int64_t ld);
int iskra_ens_download(iskra_ens *ens, int run, int sid, double *x, double *v,
                       uint32_t *id, int64_t ld, int64_t *np_out);
int iskra_ens_count(iskra_ens *ens, int run, int sid, int64_t *np);
/* nsteps steps of every run (async) */
int iskra_ens_step(iskra_ens *ens, double dt, int nsteps);
int iskra_ens_sync(iskra_ens *ens);
/* accepted collisions per process of MCC set mid in one run */
int iskra_ens_mcc_counts(iskra_ens *ens, int run, int mid, uint64_t *counts);
/* ρ, ϕ or E of one run (layouts as iskra_field_download) */
int iskra_ens_field(iskra_ens *ens, int run, int which, double *out);
/* steps between compactions of discarded particles (0 = only on count /
 * download) */
int iskra_ens_set_compact_every(iskra_ens *ens, int every);

/* ---- learned warm start of CG solves (config C5) ------------------------
 * A 4-level convolutional encoder-decoder (32 channels, BF16 weights and
 * activations, FP32 accumulation) predicts, from the first residual of a CG
 * Poisson solve, the correction the solve will make; "use" mode adds it to ϕ
 * before CG starts, scaled by an exact line search in CG's energy norm (so
 * the CG error never grows; CG still iterates to the requested tolerance,
 * so only the iteration count changes).  No reference counterpart: this replaces
 * nothing in generalized_poisson.jl, it accelerates the CG fallback of
 * iskra_poisson_solve / iskra_step for non-separable operators (and for
 * iskra_poisson_set_method(ctx, 1, ...)).  nx and ny must be multiples of 8.
 * The network is trained on the GPU on (residual, correction) pairs the
 * simulation's own CG solves record in "harvest" mode. */
/* network with He-initialised weights (seeded) and a ring of `capacity`
 * harvested pairs (0: inference only) */
int iskra_lws_create(iskra_ctx *ctx, int capacity, uint64_t seed);
int iskra_lws_destroy(iskra_ctx *ctx);
/* harvest: record the pair of every CG solve; use: warm-start CG solves;
 * smooth: binomial [1 2 1]^2/16 passes over the prediction before it is
 * applied (its value to CG is in the smooth, slowly converging modes) */
int iskra_lws_set_mode(iskra_ctx *ctx, int harvest, int use, int smooth);
/* harvested pairs, parameter count, CG solves seen, solves warm-started,
 * the mean line-search step of those warm starts (1 = the network's
 * correction taken as predicted) and their mean residual ratio (norm after
 * the warm start / before it) */
int iskra_lws_info(iskra_ctx *ctx, int *pairs, int *nparams, int64_t *solves,
                   int64_t *warm_solves, double *mean_alpha,
                   double *mean_ratio);
/* mean training loss of the network over the harvested pairs (the energy
 * norm e.Se / P of the error e of the predicted correction under the
 * 5-point stencil S, the norm CG minimises), and the same loss of the zero
 * predictor */
int iskra_lws_eval(iskra_ctx *ctx, double *loss, double *zero_loss);
/* FP32 master weights (nparams): read into w_out and/or replace by w_in */
int iskra_lws_weights(iskra_ctx *ctx, float *w_out, const float *w_in);
/* one network pass on a host image in[ny][nx] (x fastest) -> out[ny][nx] */
int iskra_lws_forward(iskra_ctx *ctx, const float *in, float *out);
/* mean squared error against target[ny][nx] and its gradient (nparams) */
int iskra_lws_loss_grad(iskra_ctx *ctx, const float *in, const float *target,
                        double *loss, float *grad);
/* iters Adam steps (learning rate lr) on the harvested pairs, one pair per
 * step drawn with `seed`; *loss = mean loss of the last min(iters, 64) */
int iskra_lws_train(iskra_ctx *ctx, int iters, double lr, uint64_t seed,
                    double *loss);

#ifdef __cplusplus
}
#endif
#endif /* ISKRA_GPU_H */
