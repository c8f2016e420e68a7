/*
 * polyfields_gpu.h — C ABI of libpolyfields_gpu.so, the GB300 SCFT engine that stands in for
 * PolyFields.jl's `scft!(sys, AndersonUpdater; domain = DomainUpdater, opts = SCFTOptions)`.
 *
 * The reference is pure Julia with no C interface; each entry point below replaces the Julia
 * function cited beside it (file:line within the PolyFields.jl project).  A Julia binding
 * calls these through `ccall` (polyfields.jl_gb300/julia/PolyFieldsGPU.jl); the Python package
 * in polyfields.jl_gb300/polyfields calls them through ctypes.
 *
 * Conventions
 *  - Every function returns an int status (PF_OK = 0).  On failure the handle's
 *    pf_last_error() string says why; the Julia shim raises it as the reference's error().
 *  - Grids are float64 arrays of Nx*Ny*Nz values, x fastest (the memory order of the
 *    reference's Array{Float64,3}[x, y, z]); dims must be in descending order, as the
 *    reference's FieldSystem requires (src/system/system.jl:55-58).
 *  - Host arrays are only read or written during the call; device memory is owned by the
 *    handle.  One handle is used by one host thread at a time; it owns one CUDA stream.
 *  - Monomers are addressed by their integer id, species by their 0-based order of addition.
 */
#ifndef POLYFIELDS_GPU_H
#define POLYFIELDS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum pf_status {
  PF_OK = 0,
  PF_EARG = 1,        /* invalid argument (reference: ArgumentError / AssertionError / error) */
  PF_ECUDA = 2,       /* CUDA runtime failure */
  PF_ENAN = 3,        /* "Diverging field updater -- breaking." (src/simulate.jl:109-111) */
  PF_ESINGULAR = 4,   /* "Error inverting Umn matrix" (src/updaters/anderson.jl:184-189) */
  PF_ETIMEOUT = 5,    /* a bounded device wait gave up (a 3D pencil pass's wait for a TMA copy); the
                         results of that solve are invalid, the handle stays usable */
  PF_ESTATE = 6,      /* call out of order (e.g. step before setup) */
  PF_ENOMEM = 7,      /* device allocation failed */
  PF_EUNSUPPORTED = 8, /* grid length outside the supported FFT sizes */
  PF_ETOOLARGE = 9     /* pf_propagate_noalloc: the grid does not fit its fixed scratch array */
};

enum pf_precision {
  PF_FP64 = 0,  /* propagators and FFTs in float64 (the reference's arithmetic) */
  PF_FP32 = 1   /* propagators and FFTs in float32; densities, residuals, Gram, stress sums stay float64 */
};

/* PF_FIELD_COTANGENT: dL/dw written by pf_density_pullback (read only) */
enum pf_grid_kind { PF_FIELD = 0, PF_DENSITY = 1, PF_RESIDUAL = 2, PF_POTENTIAL = 3, PF_FIELD_COTANGENT = 4 };

typedef struct pf_system pf_system;

/* SCFTOptions (src/simulate.jl:12-19) plus the mixed-precision switch.  When
 * mixed_switch_ferr > 0 and the handle runs PF_FP32, scft switches to PF_FP64 once
 * ferr < mixed_switch_ferr, or once the FP32 iterations have not lowered ferr by 1% for 200
 * steps (their rounding floor lies above mixed_switch_ferr), and continues to ftol/stol (FP64
 * polish).  polish selects how: 2 = Newton-Krylov steps (each one float64 residual and a
 * restarted GMRES over float32 finite-difference Jacobian products; runs without a
 * DomainUpdater; falls back to the field updater's float64 steps if a Newton step stalls),
 * 1 = float64 steps of the field updater (the Anderson history restarted at the switch),
 * 0 = automatic: Newton-Krylov on 3D grids, field-updater steps on 1D and 2D grids.
 * Output: with nsout > 0 scft prints the reference's lines (simulate.jl:82-117: the header,
 * "Step (k / n)" every nsout steps, "Updating cell dimensions", "Converged @ step").  With
 * nsout = 0 it prints nothing; the reference still prints its header and the cell and
 * convergence lines there.  A library call stays quiet by default, and batched runs do not
 * interleave their output. */
typedef struct pf_scft_options {
  int nsteps;
  int nsout;
  int nsave;
  int polish;
  double ftol;
  double stol;
  double mixed_switch_ferr;
} pf_scft_options;

/* SCFTResults (src/simulate.jl:26-33) plus the step at which the precision switched (-1 if
 * never) and the density solves of a Newton-Krylov polish (float64 and float32). */
typedef struct pf_scft_results {
  double time;
  int nsteps;
  int converged;
  double ferr;
  double serr;
  double fhelm;
  int switch_step;
  int polish_fp64_solves;
  int polish_fp32_solves;
  int pad0;
} pf_scft_results;

/* ---- library ---- */
int pf_version(void);                       /* 100 * major + minor */
const char* pf_status_string(int status);

/* ---- FieldSystem (src/system/system.jl:51-76) ---- */
int pf_system_create(pf_system** out, int nx, int ny, int nz, int precision);
int pf_system_destroy(pf_system* sys);
const char* pf_last_error(const pf_system* sys);
int pf_set_precision(pf_system* sys, int precision);
int pf_get_precision(const pf_system* sys, int* precision);
/* FieldSystem(...; mde = :RK2 | :RQM4) (src/system/system.jl:53, src/system/mde.jl:7-41):
 * 0 = RK2 operator splitting, 1 = RQM4 Richardson extrapolation of one full and two half RK2
 * steps (mde.jl:83-104; float64 chains only: PF_EUNSUPPORTED with PF_FP32). */
int pf_set_mde(pf_system* sys, int method);
/* SCFTOptions.savepath (src/simulate.jl:12-19): with nsave > 0 in the options, pf_scft writes
 * the fields to this file every nsave steps (simulate.jl:124-128) in savefields' JSON layout
 * (src/fileio.jl:77-97).  NULL or "" disables it. */
int pf_set_savepath(pf_system* sys, const char* path);

/* UnitCell(dim, crystal, params) + add_cell!  (src/system/cell.jl:31-52, system.jl:102-106).
 * crystal is the reference's Symbol name without ':' ("lamellar", "hexagonal", "cubic", ...). */
int pf_set_cell(pf_system* sys, int dim, const char* crystal, const double* params, int nparams);
/* ksq!/dksq! (src/system/cell.jl:268-320) fold the y and z frequencies to |j|
 * (cell.jl:276-277, 306-307), which changes |k|^2 in non-orthogonal cells; the engine does the
 * same by default (on = 0).  on = 1 uses the signed frequencies j - N above N/2 instead (the
 * Nyquist index stays +N/2); the bond operators and stress weights are rebuilt on next use.
 * No counterpart in the reference. */
int pf_set_signed_k(pf_system* sys, int on);
/* cell.params, cell.volume (src/system/cell.jl:14-29) */
int pf_get_cell(const pf_system* sys, double* params, int nparams, double* volume);
/* R and G basis matrices, row-major 3x3 (src/system/cell.jl:113-118) */
int pf_get_basis(const pf_system* sys, double* R, double* G);

/* add_monomer! (src/system/system.jl:113-128) */
int pf_add_monomer(pf_system* sys, int id, double vol, double charge);
/* Multiblock(mon_block, N_block, b_block, Ns) + add_species!(sys, chain, phi)
 * (src/species/multiblock.jl:32-60, src/system/system.jl:137-161). */
int pf_add_multiblock(pf_system* sys, int nblocks, const int* block_mids, const int* N_block,
                      const double* b_block, int Ns, double phi);
/* Point(mon) + add_species! (src/species/point.jl:9-22) */
int pf_add_point(pf_system* sys, int mid, double phi);
/* FloryInteraction set_interaction! + add_interaction! (src/interactions/flory.jl:36-49) */
int pf_set_flory(pf_system* sys, int mid_a, int mid_b, double chi);
/* set_interaction!(::EdwardsInteraction, mid, u) (src/interactions/edwards.jl:26-33): excluded
 * volume (u/2) sum (rho_mid / v)^2, potential u rho_mid / v (edwards.jl:34-87). */
int pf_set_edwards(pf_system* sys, int mid, double u);
/* FieldSystem(...; ensemble = Canonical | Grand) (src/system/system.jl:6-13, 51-76): 0 =
 * Canonical (add_species! values are volume fractions), 1 = Grand (they are chemical
 * potentials mu; phi = Q exp(mu) after each density solve, no mean subtraction).  Must be set
 * before species are added. */
int pf_set_ensemble(pf_system* sys, int ensemble);

/* chain_grid(N_block .* vol, Ns) of a species: Ns after adjustment, Nref, begin_block (nblocks+1,
 * 1-based as in the reference) and ds_block (src/species/base.jl:27-56). */
int pf_species_info(const pf_system* sys, int isp, int* Ns, double* Nref, int* begin_block, double* ds_block,
                    int max_blocks);

/* ---- grids ---- */
/* fieldinit!(sys, fields::Dict) for one monomer without the final residuals! (src/fileio.jl:25-54). */
int pf_set_field(pf_system* sys, int mid, const double* w);
/* sys.fields / density / residuals / potentials[mid] -> host (Ng doubles) */
int pf_get_grid(pf_system* sys, int kind, int mid, double* out);
/* chain.q[s] or chain.qc[s] (0-based s) of a multiblock species -> host */
int pf_get_propagator(pf_system* sys, int isp, int conjugate, int s, double* out);

/* ---- hot path ---- */
int pf_validate(pf_system* sys);                          /* validate(sys)     system.jl:192-237 */
int pf_density(pf_system* sys);                           /* density!(sys)     system.jl:266-289 */
int pf_residuals(pf_system* sys);                         /* residuals!(sys)   system.jl:317-340 */
int pf_free_energy(pf_system* sys, double* out);          /* free_energy(sys)  system.jl:402-433 */
int pf_free_energy_bulk(pf_system* sys, double* out);     /* free_energy_bulk  system.jl:440-458 */
int pf_field_error(pf_system* sys, double* out);          /* field_error(sys)  system.jl:470-486 */
int pf_scfstress(pf_system* sys, double* out, int nparams); /* scfstress(sys)  system.jl:384-395 */
int pf_species_q(pf_system* sys, int isp, double* Q);     /* species.Q after density! */

/* AndersonUpdater(; nhist = 50, iter_euler = 1, lam_euler = 0.01) (src/updaters/anderson.jl:36-47).
 * Replaces the handle's Anderson updater with a fresh one that is not yet set up. */
int pf_anderson_create(pf_system* sys, int nhist, int iter_euler, double lam_euler);
/* setup!(::AndersonUpdater, sys) (src/updaters/anderson.jl:54-92): allocates the history and
 * stores the current fields; keeps the history when already set up. */
int pf_anderson_setup(pf_system* sys);
/* step!(::AndersonUpdater) (src/updaters/anderson.jl:98-228) */
int pf_anderson_step(pf_system* sys);
/* EulerUpdater(; method = :PECE, lam = 0.05) (src/updaters/euler.jl:9-29): method 0 = :PEC,
 * 1 = :PECE.  Adds an updater with its own state to the handle and makes it current. */
int pf_euler_create(pf_system* sys, int method, double lam);
/* MomentumUpdater(; method = :MOM, lam = 0.01, gamma = 0.9, beta1 = 0.9, beta2 = 0.999)
 * (src/updaters/momentum.jl:19-47): method 0 = :MOM, 1 = :RMS, 2 = :ADAM, 3 = :NAG.  Adds an
 * updater with its own state to the handle and makes it current. */
int pf_momentum_create(pf_system* sys, int method, double lam, double gamma, double beta1, double beta2);
/* Several updaters on one system, as the reference's updater objects allow
 * (test/test_updaters.jl:16-30 sets up an Euler, a NAG and an Anderson updater on one system,
 * then steps each in turn).  pf_updater_current writes the id of the current updater (-1: the
 * Anderson updater; 0, 1, ...: the Euler/Momentum updaters in creation order);
 * pf_updater_select makes one current again (PF_EARG for an unknown id, PF_ESTATE for -1
 * without an Anderson updater).  Their device state lives until pf_system_destroy. */
int pf_updater_current(pf_system* sys, int* id);
int pf_updater_select(pf_system* sys, int id);
/* setup!(updater, sys) / step!(updater) for the current field updater (Anderson, Euler or
 * Momentum): src/updaters/base.jl:7-9 dispatch. */
int pf_updater_setup(pf_system* sys);
int pf_updater_step(pf_system* sys);
/* DomainUpdater(; nper = 10, nskip = 200, lam = 0.1, pmax = 1.0, rlxn = 0.5) (src/updaters/domain.jl:20-24) */
int pf_domain_create(pf_system* sys, int nper, int nskip, double lam, double pmax, double rlxn);
/* setup!(::DomainUpdater, sys) (src/updaters/domain.jl:32-42): computes the stress. */
int pf_domain_setup(pf_system* sys);
/* step!(::DomainUpdater; nsteps) (src/updaters/domain.jl:50-92) */
int pf_domain_step(pf_system* sys, int nsteps);
/* stress_error(domain) (src/updaters/domain.jl:30) */
int pf_domain_stress_error(pf_system* sys, double* out);

/* scft!(sys, updater; domain, opts) (src/simulate.jl:60-148) with the current field updater
 * (pf_anderson_create, pf_euler_create, pf_momentum_create or pf_updater_select; required) and the
 * DomainUpdater of pf_domain_create (used when use_domain != 0). */
int pf_scft(pf_system* sys, const pf_scft_options* opts, int use_domain, pf_scft_results* out);

/* ---- pullback of density! (no counterpart in the reference: PolyFields.jl has no derivatives) ----
 * For a scalar loss L of the pooled densities, set dL/drho_mid with pf_set_density_cotangent
 * (NULL: zero; kept until changed), then pf_density_pullback recomputes density!(sys) at the
 * current fields and cell and walks the adjoint of every chain backward through the same
 * propagator kernels.  Outputs: dL/dw_mid for every monomer (pf_get_grid(...,
 * PF_FIELD_COTANGENT, mid, out)), cell_bar[ncell] = dL/dtheta for the cell parameters
 * (cell.jl parameter order), and nref_bar[nnref] = dL/dNref_b for the blocks of the
 * Multiblock species in the order they were added (block lengths varied with the contour
 * step counts fixed, ds_b = Nref_b / Ns_b: the derivative with respect to a composition f).
 * dL/dchi is zero (chi does not enter density! at fixed fields).  Works in the handle's
 * precision; float32 chains keep the forward solve's per-step rescaling. */
int pf_set_density_cotangent(pf_system* sys, int mid, const double* rho_bar);
/* every > 0: the pullback reads each chain's propagators only at the checkpoints s = 0,
 * every, 2 every, ... and recomputes the contour steps in between (one segment at a time,
 * into a buffer of every + 1 grids) instead of reading every stored step; 0 (the default):
 * read the stored histories. */
int pf_set_adjoint_checkpoints(pf_system* sys, int every);
int pf_density_pullback(pf_system* sys, double* cell_bar, int ncell, double* nref_bar, int nnref);
/* Gradient of free_energy(sys) (src/system/system.jl:402-433, with the translational term as the
 * reference computes it, mu = phi) at the current fields and cell, with respect to the fields
 * (read as pf_get_grid(..., PF_FIELD_COTANGENT, mid, out)), the cell parameters (cell_bar), the
 * block lengths Nref_b (nref_bar, as for pf_density_pullback), the Flory chi of every pair in
 * ascending (id_a, id_b) order, id_a < id_b (chi_bar), and the Edwards u of every monomer that has
 * one, in ascending id order (u_bar); *fhelm receives free_energy.  Solves density! first and
 * replaces the density cotangent of pf_set_density_cotangent.  Canonical ensemble, RK2. */
int pf_free_energy_pullback(pf_system* sys, double* cell_bar, int ncell, double* nref_bar, int nnref, double* chi_bar,
                            int nchi, double* u_bar, int nu, double* fhelm);

/* Many independent scft! runs (a phase-diagram sweep: src/simulate.jl:60-148 once per
 * FieldSystem) driven together: nthreads host threads (0: min(n, 32)) take the systems in
 * decreasing order of cost (grid points x contour steps) and run pf_scft on each, every
 * system on its own CUDA stream (density solves replayed from captured CUDA graphs as in
 * single runs), so the GPU runs up to nthreads solves at once.  results[i] and status[i] receive
 * system i's outcome (pf_last_error(systems[i]) its message); returns PF_OK when every run
 * returned PF_OK, else the first nonzero status in index order.  A handle must not be used
 * elsewhere meanwhile.  Streams beyond the runtime's hardware work queues share queues and wait
 * on one another: the library sets CUDA_DEVICE_MAX_CONNECTIONS=32 when it is loaded (unless the
 * variable is already set), which only takes effect if the process creates its CUDA context
 * afterwards; a caller that initialises CUDA first should set it itself. */
int pf_scft_batch(pf_system* const* systems, int n, const pf_scft_options* opts, int use_domain,
                  pf_scft_results* results, int* status, int nthreads);

/* ---- low level: PseudoSpectralSolver update! + propagate! (src/system/mde.jl:43-81) ----
 * Propagates nsteps RK2 steps from qin with the operators of (omega, vol, b, ds) on the
 * handle's current cell; qout receives the last step.  Host arrays. */
int pf_propagate(pf_system* sys, const double* omega, double vol, double b, double ds,
                 const double* qin, double* qout, int nsteps);

/* ---- allocation-free propagation (no counterpart in the reference) ----
 * For callers that cannot allocate device memory (code inside another framework's memory
 * pool, allocation-free real-time paths, bindings that own every device buffer): runs nsteps
 * RK2 contour steps of one chain entirely on caller-provided device buffers and calls no
 * cudaMalloc/cudaFree.  hist holds (nsteps+1) grids of Nx*Ny*Nz values of the precision's
 * type (float64 for PF_FP64, float32 for PF_FP32): grid 0 is the input q, grids 1..nsteps
 * receive the steps.  lw is the Nx*Ny*Nz real-space factor exp(-ds*vol*w/2); ld is the half
 * spectrum factor exp(-ds*b^2*|k|^2/6)/(Nx*Ny*Nz), (Nx/2+1)*Ny*Nz values, layout [kz][kx][ky]
 * (ky fastest).
 * Work is queued on `stream` (a cudaStream_t; NULL = default stream) and is complete when
 * that stream is.  Internal state lives in one 16 MiB __device__ array per GPU (held until
 * the process exits): the 3D half spectrum must fit 16 MiB - 96 KiB (float32 up to 128^3,
 * float64 up to 96^3), otherwise PF_ETOOLARGE; nsteps <= 3840.  Calls whose GPU work
 * overlaps race on that array.  The first call on each device looks up the array's device
 * address, so make it before any stream capture.  A 3D call whose pencil pass gave up waiting
 * for a TMA copy leaves a status word set in the array: pf_propagate_noalloc_status reports it. */
int pf_propagate_noalloc(int nx, int ny, int nz, int precision, void* hist, const void* lw, const void* ld,
                         int nsteps, void* stream);
/* Status of the pf_propagate_noalloc calls made since the last query on this device: waits for
 * `stream` (queue it after the calls' work), then returns PF_ETIMEOUT when a pencil pass of one
 * of them gave up waiting for a TMA copy (their output is invalid) and PF_OK otherwise, and
 * clears the word.  Allocates nothing. */
int pf_propagate_noalloc_status(void* stream);

/* Time limit of the bounded waits of this handle's 3D pencil passes for their TMA copies
 * (default 1 s of GPU time; [0, 10]).  A wait that runs out marks the solve invalid: the next
 * call that reads results returns PF_ETIMEOUT and the handle stays usable.  0 makes every such
 * wait give up at once, which exercises that path in tests without a fault; copies already in
 * flight are still drained with the default limit before a pencil pass exits. */
int pf_set_wait_limit(pf_system* sys, double seconds);

/* Schedule of the 3D pencil pass for this handle's grid in its current precision: pipeline
 * stages (2 or 3 tile buffers per CTA) and rounds (tiles per CTA).  The engine's autotuner
 * picks them by timing real contour steps of each candidate the first time a handle of this
 * process solves a density on that grid (*tuned = 1 from then on; PF_NO_AUTOTUNE=1 in the
 * environment keeps the default 3 stages x 2 rounds).  No counterpart in the reference. */
int pf_get_pencil_schedule(pf_system* sys, int* stages, int* rounds, int* tuned);

/* ---- measurement ---- */
/* Device time (ms) of the last density solve's propagator launches, measured with CUDA
 * events on the handle's stream; 0 if not recorded.  Enable with pf_set_timing(sys, 1). */
int pf_set_timing(pf_system* sys, int enable);
int pf_last_timing(const pf_system* sys, double* propagate_ms, double* density_ms, int* mde_steps);
/* Record CUDA event slot (0..7) on the handle's stream; elapsed device time between two
 * recorded slots (waits for slot b). */
int pf_record_event(pf_system* sys, int slot);
int pf_elapsed_ms(pf_system* sys, int a, int b, double* ms);
/* Kernels launched by this library so far (all handles). */
long pf_launch_count(void);
/* Synchronise the handle's stream. */
int pf_synchronize(pf_system* sys);

#ifdef __cplusplus
}
#endif
#endif /* POLYFIELDS_GPU_H */
