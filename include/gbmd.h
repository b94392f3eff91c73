/*
 * gbmd.h -- C ABI of the GB300 (sm_103a) MD hot path: cell-grid neighbour
 * list, Lennard-Jones and eam_alloy force operators, velocity-Verlet push and
 * the thermodynamic reduction of exaStamp.
 *
 * Conventions
 *   - Every call returns an int status: GBMD_OK (0) or a positive GBMD_ERR_*;
 *     gbmd_last_error() gives a one-line message.  Nothing aborts or traps.
 *   - Host arrays are SoA FP64 in the caller's atom order (the order of the
 *     last gbmd_upload_atoms); the library keeps atoms cell-sorted internally
 *     and reorders on the way in and out.
 *   - Units are the caller's: the reference's internal system is angstrom,
 *     dalton, picosecond (energy Da*A^2/ps^2); Lennard-Jones runs may use
 *     reduced units.  eam_alloy tables are in eV and are scaled by the
 *     conversion factors given to gbmd_set_eam_alloy.
 *   - One context = one device + one CUDA stream, driven by one host thread
 *     at a time.  All work is stream-ordered; calls that return host data
 *     synchronise the stream.
 *
 * The reference entry points each call replaces are cited per function
 * (paths inside the exaStamp / exaNBody trees).
 */
#ifndef GBMD_H
#define GBMD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBMD_ABI_VERSION 1

typedef struct gbmd_context gbmd_context;

enum gbmd_status {
  GBMD_OK = 0,
  GBMD_ERR_INVALID = 1,          /* bad argument or call order */
  GBMD_ERR_CUDA = 2,             /* CUDA runtime error */
  GBMD_ERR_NO_DEVICE = 3,
  GBMD_ERR_NEIGHBOR_OVERFLOW = 4,/* a list build exceeded its per-atom capacity */
  GBMD_ERR_LOST_ATOM = 5,        /* an atom left the periodic box by more than one image */
  GBMD_ERR_NONFINITE = 6,        /* NaN/Inf force */
  GBMD_ERR_IO = 7,               /* setfl file unreadable */
  GBMD_ERR_UNSUPPORTED = 8,
  GBMD_ERR_TOO_LARGE = 9
};

enum gbmd_precision {
  GBMD_PRECISION_FP64 = 0,  /* plain FP64 pair arithmetic */
  GBMD_PRECISION_MIXED = 1  /* FP32 pair arithmetic on cell-relative coordinates, compensated
                               FP32 sums; FP64 state, push, wrap and reductions */
};

enum gbmd_potential {
  GBMD_POT_NONE = 0,
  GBMD_POT_LJ = 1,          /* lj_compute_force */
  GBMD_POT_LJ_MULTI = 2,    /* lj_multi_force */
  GBMD_POT_EAM_ALLOY = 3,   /* eam_alloy_force (rho, rho2emb, force passes) */
  GBMD_POT_EAM_JOHNSON = 4, /* johnson_force: analytic single-element EAM, 2 passes */
  GBMD_POT_EAM_SUTTON_CHEN = 5 /* sutton_chen_force: analytic single-element EAM, 2 passes */
};

enum gbmd_force_flags {
  GBMD_FORCE_ENERGY = 1,    /* per-atom ep (trigger_thermo_state) */
  GBMD_FORCE_VIRIAL = 2,    /* per-atom virial tensor (compute_virial) */
  /* Split EAM passes (eam_alloy_force with eam_rho / eam_rho2emb / eam_force,
   * src/potential/eam_potential_template/eam_potential_multimat.cu L101-104,
   * L186-232).  Neither or both bits: every pass.  DENSITY alone: density +
   * embedding (F'(rho) kept in the context; the embedding energy too with
   * GBMD_FORCE_ENERGY).  FORCE alone: the final pair pass from the kept
   * F'(rho); for EAM it needs a DENSITY call on the same positions and list
   * (GBMD_ERR_INVALID otherwise), and energies need that call to have had
   * GBMD_FORCE_ENERGY.  Pair potentials have no density pass: DENSITY
   * alone does nothing and FORCE alone is the whole evaluation. */
  GBMD_FORCE_PASS_DENSITY = 4,
  GBMD_FORCE_PASS_FORCE = 8
};

/* ---- context --------------------------------------------------------------
 * Replaces the onika execution context + grid ownership that every operator
 * receives (src/tutorial/my_gpu_test.cxx L80-92: parallel_execution_context()
 * ->gpu_stream()).  stream may be NULL (the context creates its own) or a
 * cudaStream_t cast to void*. */
int gbmd_create(gbmd_context** ctx, int device, void* stream);
int gbmd_destroy(gbmd_context* ctx);
const char* gbmd_last_error(const gbmd_context* ctx);
int gbmd_abi_version(void);

/* Orthorhombic periodic domain [lo, hi) (exaNBody Domain bounds/periodic,
 * set by the reference's `domain` setup operator; xform identity).  Only
 * fully periodic boxes are supported. */
int gbmd_set_box(gbmd_context* ctx, const double lo[3], const double hi[3], const int periodic[3]);

/* Per-type masses (ParticleSpecies m_mass: include/exaStamp/particle_species/
 * particle_specie.h L52-70); used by force_to_accel and the push. */
int gbmd_set_species(gbmd_context* ctx, int ntypes, const double* masses);

/* Copy atoms in (grid cell arrays rx,ry,rz,vx,vy,vz,type,id:
 * include/exaStamp/fields.h L64-79).  vx/vy/vz/type/id may be NULL
 * (zero velocity, type 0, id = index). Invalidates the neighbour list. */
int gbmd_upload_atoms(gbmd_context* ctx, int64_t n, const double* rx, const double* ry,
                      const double* rz, const double* vx, const double* vy, const double* vz,
                      const uint8_t* type, const uint64_t* id);
/* Positions (and optionally velocities) only, same atoms and order as the
 * last upload; keeps the neighbour list (the adapter's per-step copy-in). */
int gbmd_upload_positions(gbmd_context* ctx, const double* rx, const double* ry, const double* rz,
                          const double* vx, const double* vy, const double* vz);
/* The whole per-step grid state in upload order: positions, velocities and
 * accelerations (the r, v and f fields the exaNBody grid keeps between
 * operators).  The given accelerations are taken as the forces of these
 * positions, so a following gbmd_run_nve continues without a force call.
 * The list is kept unless an atom moved more than skin/2 since the last
 * rebuild (particle_displ_over, config_move_particles.msp L19-22). */
int gbmd_upload_state(gbmd_context* ctx, const double* rx, const double* ry, const double* rz,
                      const double* vx, const double* vy, const double* vz, const double* ax,
                      const double* ay, const double* az);
/* Copy state out in upload order; any pointer may be NULL.  a* is the
 * acceleration (force_to_accel writes f/m into the force fields,
 * src/compute/force_to_accel.cu L42-48); vir is n x 9 row-major. */
int gbmd_download(gbmd_context* ctx, double* rx, double* ry, double* rz, double* vx, double* vy,
                  double* vz, double* ax, double* ay, double* az, double* ep, double* vir);
int gbmd_num_atoms(const gbmd_context* ctx, int64_t* n);

/* ---- potentials ----------------------------------------------------------- */
/* lj_compute_force: slots parameters{epsilon,sigma}, rcut
 * (src/potential/pair_potential_template/pair_potential_impl.hxx L104-121,
 * pair function lennard_jones.h L41-50, ecut = e(rcut) L489-498). */
int gbmd_set_lj(gbmd_context* ctx, double epsilon, double sigma, double rcut);
/* lj_multi_force: per type-pair (epsilon, sigma, rcut) tables, ntypes x ntypes
 * symmetric, plus the operator's common rcut (rcut_max = max of all)
 * (pair_potential_force_op_multiparam.h L57-118, YAML L249-284). */
int gbmd_set_lj_multi(gbmd_context* ctx, int ntypes, const double* epsilon, const double* sigma,
                      const double* rcut, double rcut_common);
/* eam_alloy parameters from raw setfl tables (eam_alloy.cpp): F(rho)
 * nel x nrho, rho(r) nel x nr, z2r (nel*(nel+1)/2) x nr in file order; the
 * library builds the 7-coefficient splines (eam_alloy.cpp L29-58).  rcut is
 * the operator's rcut slot (eam_potential_multimat.cu L91); conv_z2r and
 * conv_frho convert eV*A and eV to internal energy (eam_alloy.h L156-157). */
int gbmd_set_eam_alloy(gbmd_context* ctx, int nelements, int nrho, double drho, int nr, double dr,
                       const double* frho, const double* rhor, const double* z2r, double rcut,
                       double conv_z2r, double conv_frho);
/* eam_alloy_init: read a setfl (.eam.alloy) file (eam_alloy.cpp L66-201). */
/* johnson_force (src/potential/eam_potentials/johnson/johnson.h L28-176 with
 * the mono-material 2-pass template src/potential/eam_potential_template/
 * eam_potential.cu L69-193, eam_force_op_singlemat.h L39-171): analytic
 * phi(r), rho(r), F(rho) of one element.  params[19] in the order of
 * EamJohnsonParameters: re, fe, rhoe, alpha, beta, A, B, kappa, lambda, Fn0,
 * Fn1, Fn2, Fn3, F0, F1, F2, F3, Fo, eta, already in the caller's units
 * (energies in the energy unit, re in the length unit; alpha, beta, kappa,
 * lambda and eta dimensionless).  Every atom must be of type 0. */
int gbmd_set_eam_johnson(gbmd_context* ctx, const double params[19], double rcut);
/* sutton_chen_force (src/potential/eam_potentials/sutton_chen/sutton_chen.h
 * L30-67 with the same mono-material 2-pass template): phi(r) = epsilon
 * (a0/r)^n, rho(r) = (a0/r)^m, F(rho) = -c epsilon sqrt(rho).  params[5] in
 * the order of EamSuttonChenParameters: c, epsilon, a0, n, m, in the
 * caller's units (epsilon an energy, a0 a length; c, n, m dimensionless).
 * Every atom must be of type 0. */
int gbmd_set_eam_sutton_chen(gbmd_context* ctx, const double params[5], double rcut);
int gbmd_load_setfl(gbmd_context* ctx, const char* path, double rcut, double conv_z2r,
                    double conv_frho);

int gbmd_set_precision(gbmd_context* ctx, int precision);
/* Lanes per atom (1,2,4,8,16) and threads per block for the pair kernels;
 * the autotuner's knobs.  Invalidates the neighbour list layout.
 * gbmd_set_launch keeps one list entry per lane per load. */
int gbmd_set_launch(gbmd_context* ctx, int lanes_per_atom, int block);
int gbmd_get_launch(const gbmd_context* ctx, int* lanes_per_atom, int* block);
/* As gbmd_set_launch, plus the list entries each lane reads per load in the
 * mixed-precision kernels: 1, or 4 (one 16-byte load; at most 4 lanes per
 * atom).  The list rows are laid out lanes_per_atom * entries wide. */
int gbmd_set_launch_ex(gbmd_context* ctx, int lanes_per_atom, int entries_per_load, int block);
int gbmd_get_launch_ex(const gbmd_context* ctx, int* lanes_per_atom, int* entries_per_load, int* block);
/* Threads per block of the EAM density kernels (0 = the pair kernels'
 * block).  On GB300 the density pass prefers smaller blocks than the force
 * pass (4 M-atom Cu: 128 vs 256); the autotuner sets both. */
int gbmd_set_density_block(gbmd_context* ctx, int block);
int gbmd_get_density_block(const gbmd_context* ctx, int* block);
/* With one lane per atom and 4 entries per load, the mixed-precision pair
 * kernels can run one block per run of home cells along x and read
 * neighbour positions from a shared-memory copy of the surrounding cells
 * instead of gathering them (enable = 1; default 0, the gathers are faster
 * on GB300); results are the same bit for bit. */
int gbmd_set_neighbor_staging(gbmd_context* ctx, int enable);
int gbmd_get_neighbor_staging(const gbmd_context* ctx, int* enabled);
/* Newton-3 mode (lj_compute_force_symetric,
 * src/potential/pair_potential_template/pair_potential_singlemat_symetric.cpp
 * L44, L230-320; eam_alloy's eam_symmetry,
 * src/potential/eam_potential_template/eam_force_op_multimat.h L162-169,
 * L305-338): the list keeps each unordered pair once (j after i in cell
 * order).  The kernels add to j, with 64-bit fixed-point integer atomics,
 * what the pair gives it: the reaction force, half the pair energy and half
 * the pair virial, and for eam_alloy its density rho_ti(r).  The sums do not
 * depend on the order of the additions, so runs are bit-reproducible.  A
 * contribution beyond 2^16 times its kind's bound (an LJ pair force beyond
 * 2^16 x 24 eps/sigma, i.e. pairs closer than ~0.49 sigma) is outside the
 * fixed-point range; gbmd_check_errors / gbmd_run_nve then return
 * GBMD_ERR_TOO_LARGE.  LJ potentials and eam_alloy in mixed precision with
 * the 1 lane x 4 entries launch only; other set-ups return
 * GBMD_ERR_UNSUPPORTED at the force call.  Default 0. */
int gbmd_set_newton3(gbmd_context* ctx, int enable);
int gbmd_get_newton3(const gbmd_context* ctx, int* enabled);

/* ---- neighbour list --------------------------------------------------------
 * chunk_neighbors (exaNBody; config data/config/config_move_particles.msp
 * L54-68, decode contract src/debug/atom_neighbors_stats.cpp L169-228) with
 * chunk_size 1, preceded by the periodic wrap and rebinning of
 * move_particles.  Radius = rcut_max + skin (global.rcut_inc,
 * data/config/config_globals.msp L8).  The pair set is {(i, j, image n) :
 * d2 <= (rcut_max+skin)^2} with d2 from ((x_j + n L) - x_i) in FP64 without
 * contraction. */
int gbmd_set_skin(gbmd_context* ctx, double skin);
/* Always a full build: wrap, rebin into cells, list (with a list buffer set,
 * the outer list too, on cells of the outer radius, and the list filtered
 * from it: the same pairs, rows in the order of those cells). */
int gbmd_build_neighbors(gbmd_context* ctx);
/* Two-level list (no reference counterpart; the pair set is unchanged).
 * With buffer d > 0 a full build also makes an outer list of radius
 * rcut_max + skin + d, and every later rebuild filters the list from it
 * (the entries within rcut_max + skin now, band entries re-tested in FP64
 * as above, in the outer rows' order) without the wrap and rebin.  The outer
 * list, with the wrap and rebin, is built again only when some atom moved
 * more than d/2 since it was built: then every pair within rcut_max + skin
 * is in it.  Between outer builds the atoms keep their cells and their
 * coordinates run on past the box faces.  Cells are at least
 * rcut_max + skin + d wide, so each box edge must be that long.  0 (the
 * default) turns it off.  Invalidates the list. */
int gbmd_set_list_buffer(gbmd_context* ctx, double buffer);
/* buffer and the number of outer builds so far (either may be NULL). */
int gbmd_get_list_buffer(const gbmd_context* ctx, double* buffer, int64_t* outer_builds);
/* check_and_update_particles (data/config/config_move_particles.msp L116-152:
 * trigger_move_particles = particle_displ_over, L19-22, then the full update
 * when it fires): the skin/2 displacement test of the current positions
 * against those of the last rebuild, on the device, and a rebuild (wrap,
 * rebin, list, regrown on overflow) when some atom moved farther; builds the
 * list when there is none.  rebuilt (may be NULL) receives 1 when it did.
 * Synchronises the stream (the test's outcome is read back). */
int gbmd_update_neighbors(gbmd_context* ctx, int* rebuilt);
/* Export the list as (id_i, id_j, n_x, n_y, n_z) rows, rows of one atom in
 * list order, atoms in cell-sorted order. count receives the number of rows
 * (call with cap 0 to size). */
int gbmd_export_pairs(gbmd_context* ctx, int64_t cap, uint64_t* id_i, uint64_t* id_j, int8_t* img,
                      int64_t* count);
int gbmd_neighbor_stats(gbmd_context* ctx, int64_t* npairs, int* maxnb, int* nc3);

/* ---- force operators -------------------------------------------------------
 * compute_all_forces_energy = zero_force_energy + compute_force +
 * force_to_accel (data/config/config_numerical_schemes.msp L8-15): after this
 * call a* holds f/m, ep the per-atom energy (GBMD_FORCE_ENERGY) and vir the
 * per-atom virial (GBMD_FORCE_VIRIAL). Builds the list first if needed. */
int gbmd_compute_forces(gbmd_context* ctx, int flags);
/* Waits for the context's stream and reports the device error word, then
 * clears it: GBMD_ERR_NONFINITE (a non-finite force), GBMD_ERR_TOO_LARGE (a
 * Newton-3 contribution beyond the fixed-point range),
 * GBMD_ERR_NEIGHBOR_OVERFLOW, GBMD_ERR_LOST_ATOM.  The force call returns
 * before its kernels finish; gbmd_run_nve and gbmd_run_minimize check on
 * their own. */
int gbmd_check_errors(gbmd_context* ctx);

/* ---- integration -----------------------------------------------------------
 * push_f_v_r: r += v*dt' + a*dt'^2/2, dt' = dt*dt_scale; push_f_v: v += a*dt*
 * dt_scale (exaNBody; schedule config_numerical_schemes.msp L23-28, formula
 * src/numerical_schemes/push_vec3_2nd_order_xform_minimization.cpp L33-38). */
int gbmd_push_f_v_r(gbmd_context* ctx, double dt, double dt_scale);
int gbmd_push_f_v(gbmd_context* ctx, double dt, double dt_scale);
/* push_f_v_r_xform_minimization, identity xform (same file L116-149):
 * r += a*dt'^2/2; tolF > 0 clips each acceleration component first. */
int gbmd_push_min(gbmd_context* ctx, double dt, double dt_scale, double tolF);

/* rebuild_every value: rebuild when some atom moved more than skin/2 since
 * the last rebuild (particle_displ_over, data/config/config_move_particles.msp
 * L19-22, L116-118), tested every step on the device. */
#define GBMD_REBUILD_ON_DISPLACEMENT (-1)

/* verlet_nve for nsteps (config_numerical_schemes.msp L44-52): first half,
 * rebuild every `rebuild_every` steps (0 = never, GBMD_REBUILD_ON_DISPLACEMENT
 * = on the displacement trigger), forces, second half.
 * thermo_every > 0 writes the 27-double reduction every thermo_every steps
 * into thermo_out (rows of 27, step 0 first); thermo_out may be NULL.
 * use_graph != 0 replays chunks of steps from a CUDA graph: 2*rebuild_every
 * steps, or with the trigger thermo_every steps when even (20 without
 * thermo); the remaining steps are launched one by one. */
int gbmd_run_nve(gbmd_context* ctx, int nsteps, double dt, int rebuild_every, int thermo_every,
                 double* thermo_out, int use_graph);
/* verlet_nve on a state held in host arrays (the caller's grid, in upload
 * order): the state goes in (the given accelerations are the forces of the
 * given positions), nsteps of verlet_nve run (no thermo, no graph), then r,
 * v, a are written back.  Page-locked arrays with a list in place are read
 * by one kernel over the host link that also applies step 1's first half,
 * after which the skin/2 displacement test of the pushed positions decides
 * a rebuild (check_and_update_particles after verlet_first_half); other
 * arrays go through gbmd_upload_state.  The positions of the last step are
 * final after its first half and go back to the host while its force pass
 * runs; v and a follow.  Returns once every array is written.
 * One step (nsteps == 1) on page-locked arrays is pipelined when
 * gbmd_set_host_pipeline allows it: the arrays are read in chunks of the
 * caller order, the pair passes run slab by slab (whole z layers of the
 * cell grid) as soon as the chunks holding their neighbourhood are in, and
 * v, a of each chunk go back as soon as its slabs are done, so that the host
 * link and the passes overlap; the results are those of the unpipelined
 * step, bit for bit.  The overlap needs a caller order that follows the
 * cell order along z (atoms stored cell by cell, z slowest, as exaNBody's
 * grids hold them); another order gives a more serial schedule.  A step
 * whose first half moves an atom more than skin/2 from its position at the
 * last rebuild is finished without the pipeline after the rebuild; the
 * pipelined step also applies the next step's first half to the state it
 * returns, and when that moves an atom past skin/2 the next step (given
 * that state back) is run without the pipeline from the start. */
int gbmd_run_nve_host(gbmd_context* ctx, int nsteps, double dt, int rebuild_every, double* rx, double* ry,
                      double* rz, double* vx, double* vy, double* vz, double* ax, double* ay, double* az);
/* slabs: -1 automatic (16 slabs from 262,144 atoms up, else off; the
 * default), 0 off, 4..64 that many slabs (at most one per z layer of the
 * cell grid).  The pipeline is not used with Newton-3 half lists or staged
 * neighbour positions. */
int gbmd_set_host_pipeline(gbmd_context* ctx, int slabs);
/* How the pipeline moves the chunks over the host link.  mode 1 (the
 * default): grid-stride kernels of `blocks` blocks of `threads` threads
 * (40 x 512 by default) that read and write the page-locked arrays
 * directly, few enough to leave the SMs to the pair passes.  mode 0: the
 * copy engines, through staging arrays in HBM (9 doubles per atom; measured
 * slower at 4 M atoms); blocks and threads are ignored. */
int gbmd_set_host_pipeline_link(gbmd_context* ctx, int mode, int blocks, int threads);
/* Timeline of the last pipelined host step, the analogue of onika's
 * per-operator timers for it: with tracing on, each step records CUDA
 * events on its streams; gbmd_get_host_pipeline_trace returns up to `cap`
 * marks of the last step as t_ms (milliseconds since the step's start),
 * kind (GBMD_PIPE_MARK_*) and index (the chunk or slab), and their number
 * in *count.  Tracing adds one event record per mark. */
enum {
  GBMD_PIPE_MARK_START = 0,
  GBMD_PIPE_MARK_CHUNK_IN = 1,    /* caller chunk read, first half applied */
  GBMD_PIPE_MARK_DENSITY = 2,     /* slab's density (embedding) pass done */
  GBMD_PIPE_MARK_FORCE = 3,       /* slab's force pass done */
  GBMD_PIPE_MARK_CHUNK_OUT = 4,   /* caller chunk's v, a written back */
  GBMD_PIPE_MARK_END = 5
};
int gbmd_set_host_pipeline_trace(gbmd_context* ctx, int on);
int gbmd_get_host_pipeline_trace(gbmd_context* ctx, int cap, double* t_ms, int* kind, int* index, int* count);
/* slabs the next host step would use (0: unpipelined), the number of
 * steps that stood as pipelined so far, and the number of pipelined steps
 * discarded because they needed a rebuild that was not predicted (those are
 * finished unpipelined).  Any pointer may be NULL. */
int gbmd_get_host_pipeline(const gbmd_context* ctx, int* slabs, int64_t* steps, int64_t* redone);
/* Minimiser: nsteps of compute forces + push_min (r += a dt^2/2, clipped);
 * rebuild_every as gbmd_run_nve. */
int gbmd_run_minimize(gbmd_context* ctx, int nsteps, double dt, double tolF, int rebuild_every);
/* Parameter adjoint of lj_compute_force (no reference counterpart: the
 * reference has no gradients).  Computes forces and per-atom energies of the
 * current state (precision as set), the force-matching + energy loss
 *   L = w_force sum_i |F_i - F*_i|^2 + w_energy sum_i (E_i - E*_i)^2
 * against host targets in upload order (F = m a, E = per-atom energy), and
 * dL/d(epsilon, sigma) with every pair term recomputed in FP64.  grad[2]. */
int gbmd_lj_loss_grad(gbmd_context* ctx, const double* fx_target, const double* fy_target, const double* fz_target,
                      const double* e_target, double w_force, double w_energy, double* loss, double grad[2]);
/* The same loss for lj_multi_force: gradients with respect to each species
 * pair's (epsilon, sigma), the (a,b) and (b,a) table entries being one
 * parameter.  grad_eps and grad_sigma receive ntypes x ntypes row-major
 * (symmetric) arrays. */
int gbmd_lj_multi_loss_grad(gbmd_context* ctx, const double* fx_target, const double* fy_target,
                            const double* fz_target, const double* e_target, double w_force, double w_energy,
                            double* loss, double* grad_eps, double* grad_sigma);

/* Number of neighbour-list builds since the context was created, including
 * the displacement-triggered ones (counted on the device, folded in when
 * gbmd_run_nve / gbmd_run_minimize return) and, with a list buffer, the
 * lists filtered from the outer list. */
int gbmd_list_builds(const gbmd_context* ctx, int64_t* count);

/* ---- thermodynamic state ---------------------------------------------------
 * simulation_thermodynamic_state (src/thermo_state/
 * simulation_thermodynamic_state.cpp L101-163): out[27] = virial(9),
 * ke_tensor(9), momentum(3), kinetic energy(3), potential energy, mass,
 * particle count, reduced in FP64 on the device. */
int gbmd_thermo(gbmd_context* ctx, double out[27]);

/* The 27-double thermodynamic reduction of gbmd_thermo on the caller's own
 * device arrays, without allocating anything.  No counterpart in the
 * reference: it exists for callers that may not call cudaMalloc -- a plugin
 * whose device memory must all come from its host framework's pool, code
 * running while its stream is being captured into a CUDA graph, or a
 * latency-critical loop that cannot afford the device-wide synchronisation
 * an allocation can cause.
 *   vx, vy, vz, ep (may be NULL), vir (n x 9, may be NULL), type: device
 *   arrays of n atoms; type values must be < ntypes (an atom of another
 *   type is checked on the device and turns the mass-weighted sums --
 *   out[9..23] and out[25] -- into NaN).  masses: HOST array of
 *   ntypes doubles (ntypes <= 8).  out: DEVICE array of 27 doubles, same
 *   layout as gbmd_thermo.  stream: cudaStream_t (NULL = default stream).
 *   The work is enqueued on `stream`; nothing is synchronised.
 * Scratch: a fixed array of 1184 x 26 doubles (246,272 bytes) inside the
 * library's device image, present on every GPU that loads the library until
 * the process exits; every partial it uses is overwritten before it is read,
 * so no clearing is needed.  All calls on a device share that array: calls
 * whose kernels overlap on the GPU (different streams, no ordering between
 * them) race and give wrong sums.  Every call looks the array's address up
 * (cudaGetSymbolAddress, no allocation) with the caller's device current,
 * so the address stays valid across a cudaDeviceReset; the first call on a
 * device also loads the library's device code there, so make that first
 * call before any stream capture.  n > 67,108,864 atoms returns
 * GBMD_ERR_TOO_LARGE; bad pointers or ntypes return GBMD_ERR_INVALID. */
int gbmd_thermo_reduce_noalloc(int64_t n, const double* vx, const double* vy, const double* vz,
                               const double* ep, const double* vir, const uint8_t* type,
                               const double* masses, int ntypes, double* out, void* stream);

/* ---- batched replicas ------------------------------------------------------
 * Many independent periodic single-element eam_alloy systems (<= 2048 atoms
 * each, every box edge >= rcut) evaluated in one persistent launch: forward
 * (per-atom forces and energies, per-replica energy and virial) and,
 * optionally, the gradient of L = wF sum |F - F*|^2 + wE sum (E - E*)^2 with
 * respect to up to 9 potential parameters.  Forces are in table units x
 * conv (eV/A with conv = 1), not accelerations.  No reference counterpart
 * for the batching itself: each replica is the eam_alloy_force operator
 * (eam_potential_multimat.cu L113-257) on its own periodic domain. */
typedef struct gbmd_batch gbmd_batch;
int gbmd_batch_create(gbmd_batch** b, int device, void* stream);
int gbmd_batch_destroy(gbmd_batch* b);
const char* gbmd_batch_last_error(const gbmd_batch* b);
/* single-element setfl tables (F nrho, rho nr, z2r nr knots), as gbmd_set_eam_alloy */
int gbmd_batch_set_eam_alloy(gbmd_batch* b, int nrho, double drho, int nr, double dr, const double* frho,
                             const double* rhor, const double* z2r, double rcut, double conv_z2r,
                             double conv_frho);
/* d(knot values)/d(parameter): nparam x nrho, nparam x nr, nparam x nr; the
 * library splines them (the spline map is linear in the knot values). */
int gbmd_batch_set_param_derivatives(gbmd_batch* b, int nparam, const double* dfrho, const double* drhor,
                                     const double* dz2r, double conv_z2r, double conv_frho);
/* offsets: nrep+1 atom offsets; lo, hi: nrep x 3 boxes; x, y, z: all atoms */
int gbmd_batch_upload(gbmd_batch* b, int nrep, const int64_t* offsets, const double* lo, const double* hi,
                      const double* x, const double* y, const double* z);
int gbmd_batch_set_targets(gbmd_batch* b, const double* fx, const double* fy, const double* fz, const double* e,
                           double wF, double wE);
/* launch shape (the autotuner's knobs): threads per block (64-512) and the
 * cell stencil radius (1: cells >= rcut, 2: cells >= rcut/2) */
int gbmd_batch_set_launch(gbmd_batch* b, int block, int stencil);
/* Replicas of at most 512 atoms run in a second kernel with smaller blocks
 * (several per SM): its threads per block, 64-256 (default 128). */
int gbmd_batch_set_small_block(gbmd_batch* b, int block);
/* per_replica != 0: one launch per replica (the comparison mode);
 * use_graph != 0: the persistent launch is captured once and replayed */
int gbmd_batch_run(gbmd_batch* b, int adjoint, int per_replica, int use_graph);
int gbmd_batch_synchronize(gbmd_batch* b);
/* any pointer may be NULL; rep_virial is nrep x 9; loss / grad[9] summed
 * over replicas in replica order */
int gbmd_batch_download(gbmd_batch* b, double* fx, double* fy, double* fz, double* ep, double* rep_energy,
                        double* rep_virial, double* loss, double* grad);

/* Per-kernel timing of one step's kernels with CUDA events on the context
 * stream, averaged over `reps` launches of each (the analogue of onika's
 * per-operator profiling timers, data/config/config_defaults.msp L21-23):
 * ms[0] neighbour rebuild (wrap, sort, list), ms[1] EAM density+embedding
 * pass (0 for LJ), ms[2] final pair kernel with the fused Verlet halves,
 * ms[3] standalone first-half push, ms[4] thermo reduction.  Positions are
 * pushed with dt = 0, so the state is unchanged. */
int gbmd_profile_step(gbmd_context* ctx, int reps, double ms[5]);

/* Device pointers of the cell-sorted FP64 state (for zero-copy adapters):
 * order is internal; user_index[i] gives the upload index of sorted atom i. */
int gbmd_device_state(gbmd_context* ctx, double** rx, double** ry, double** rz, double** vx,
                      double** vy, double** vz, double** ax, double** ay, double** az, double** ep,
                      int32_t** user_index);

int gbmd_synchronize(gbmd_context* ctx);

#ifdef __cplusplus
}
#endif
#endif /* GBMD_H */
