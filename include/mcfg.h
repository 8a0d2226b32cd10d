/*
 * mcfg.h -- C-ABI of the GB300-native SDPD right-hand side and time step.
 *
 * This library replaces the per-step particle routines of MCF (Fortran 90 on
 * the PPM library) with CUDA kernels for sm_103a.  MCF's driver keeps its
 * configuration files, its Physics/Control objects and its particle arrays;
 * a thin iso_c_binding module fills `mcfg_params` from MCF's getters and
 * calls the entry points below.  Every entry point:
 *   - returns an int status: MCFG_OK (0) or a negative MCFG_E* code.  It never
 *     aborts the process (MCF's convention is `stat_info = 0 / -1`,
 *     e.g. mcf/src/particles_compute_interaction.F90:896-953);
 *   - takes caller-owned host buffers that it never frees; device memory is
 *     owned by the handle and released by mcfg_destroy;
 *   - uses MCF's array layout on the host side: x(d,N) column-major REAL(8),
 *     i.e. interleaved [x0 y0 (z0) x1 y1 (z1) ...], id(2,N) INTEGER(4) with
 *     id(1)=pid, id(2)=sid (sid 0 fluid, <0 wall, >0 colloid number),
 *     mcf/src/Class_Particles.F90:132-141, mcf/src/mcf_header.F90:118-120.
 * A handle is used by one host thread at a time and drives one GPU.
 */
#ifndef MCFG_H
#define MCFG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MCFG_OK 0
#define MCFG_EINVAL -1     /* bad argument or parameter combination          */
#define MCFG_ECUDA -2      /* CUDA runtime error (message in mcfg_last_error) */
#define MCFG_ENOMEM -3     /* device allocation failed                        */
#define MCFG_ESTATE -4     /* call out of order (e.g. force before density)   */
#define MCFG_EOVERFLOW -5  /* a fixed-capacity list overflowed (neighbours)   */
#define MCFG_EPHYS -6      /* physics check failed (zero mass/density, NaN)   */
#define MCFG_ENODEV -7     /* no CUDA device / kernels not loadable           */
#define MCFG_ETIMEOUT -8   /* a bounded device wait gave up                   */
#define MCFG_ENOTSUP -9    /* option not supported by the library            */

/* ---- enumerations (values are MCF's own) -------------------------------- */
/* boundary types, PPM ppm_param.h: periodic 1, freespace 2, symmetry 3,
 * wall_sym 7, wall_solid 9, Lees-Edwards 10.  A freespace face has no
 * periodic images and no wall particles: the faces of one subdomain of a
 * decomposed box, whose halo particles the caller supplies. */
#define MCFG_BC_PERIODIC 1
#define MCFG_BC_FREESPACE 2
#define MCFG_BC_WALL_SOLID 9
#define MCFG_BC_LE 10

#define MCFG_PRECISION_FP64 0       /* pair arithmetic in FP64              */
#define MCFG_PRECISION_FP32_MIXED 1 /* FP32 pair arithmetic, FP64 state     */

/* Flat parameter block, filled from MCF's Control/Physics/Boundary/Colloid
 * getters.  Field names follow the keys of mcf_config/ctrl.mcf and
 * mcf_config/physics_config.mcf. */
typedef struct mcfg_params {
  int32_t num_dim;            /* 2 or 3                                      */
  int32_t bcdef[6];           /* per face x-,x+,y-,y+,z-,z+: 1 periodic, 2
                                 freespace, 9 solid wall, 10 Lees-Edwards (y
                                 faces only: planes sliding along x; x, z
                                 periodic with min_phys_t 0; no walls or
                                 colloids)                                   */
  double min_phys[3];         /* fluid domain                                */
  double max_phys[3];
  double min_phys_t[3];       /* total domain incl. wall layers              */
  double max_phys_t[3];
  double cut_off;             /* kernel support rc                           */
  double cell_factor;         /* cell side = cell_factor*rc (MCF: 1.0001)    */
  int32_t kernel_type;        /* 1 quintic spline (h=rc/3), 2 Lucy (h=rc)    */
  int32_t rhs_density_type;   /* 1 mass density, 2 number density            */
  int32_t rhs_force_type;     /* 1 Morris, 2 Espanol-Revenga, 3 Hu-Adams,
                                 4 Hu-Adams angular                          */
  int32_t stateEquation_type; /* 1 Morris p=c^2(rho^gamma-rho_ref),
                                 2 Batchelor p=p0((rho/rho_ref)^gamma-1)     */
  double c;                   /* sound speed                                 */
  double rho;                 /* initial density (Batchelor p0)              */
  double rho_ref;
  double gamma;
  double eta;                 /* shear viscosity (solvent eta_s if not
                                 Newtonian)                                  */
  double eta_coef;            /* angular Hu-Adams viscosity coefficient      */
  double kt;                  /* thermal energy kT                           */
  double dt;                  /* time step used by the random force when the
                                 interaction is called outside a VV step     */
  int32_t Brownian;           /* 1: Wiener-increment random force            */
  int32_t symmetry;           /* MCF symmetry flag (pair evaluation mode of
                                 the CPU path; the GPU result is the same)   */
  int32_t body_force_type;    /* 0 none, 1 constant, 2 reverse Poiseuille,
                                 3 g_x*sin(2 pi y / L_y)                     */
  int32_t wall_rho_type;      /* 0 constant, 1 dynamic                       */
  double body_force[3];
  int32_t wall_noslip_type;   /* 1 frozen, 2 Morris extrapolation            */
  int32_t stress_tensor;      /* 1: accumulate per-particle stress s(d^2,N) */
  double wall_v[6][3];        /* velocity of each solid-wall or Lees-Edwards
                                 face (MCF's shear_v0; a Lees-Edwards pair
                                 may differ only along x)                    */
  double init_density;        /* constant density of boundary particles      */
  int32_t Newtonian;          /* 1 Newtonian; 0 Oldroyd-B conformation model */
  int32_t precision;          /* MCFG_PRECISION_*                            */
  double tau;                 /* Oldroyd-B relaxation time                   */
  double n_p;                 /* polymer number density                      */
  double kt_p;                /* polymer kT (G = n_p*kt_p)                   */
  uint64_t seed;              /* Philox key for the Wiener increments        */
  int32_t device;             /* CUDA device ordinal                         */
  /* reserved[0]: neighbour-list capacity per particle (0: from the first
   *   upload's mean number density, 1.3 x the particles within the cut-off
   *   + 16, at least 256 in 3D and 96 in 2D).
   * reserved[1]: non-zero enables neighbour-list reuse in mcfg_step_vv /
   *   mcfg_run_vv: the candidates within rc + skin are listed at a rebuild
   *   (skin = 0.99 x (smallest cell side - cut_off), so the cell stencil of
   *   the rebuild holds every pair) and re-tested exactly every step; the
   *   rebuild -- wrap, MCF's cell list, candidate list -- happens on the
   *   device when a particle has moved more than skin/2 since the last one
   *   (with Lees-Edwards faces: displacements measured from the shear the
   *   faces impose, against skin/2 less the shear's change over rc + skin,
   *   and at every re-entry through a y face).
   *   The pair set of every step is the same as without reuse; positions
   *   may sit up to skin/2 past a periodic face between rebuilds (mcfg_download
   *   returns them wrapped).  Widen the skin with cell_factor.
   * reserved[2..6]: must be 0. */
  int32_t reserved[7];
} mcfg_params;

typedef struct mcfg_handle mcfg_handle;

/* sizeof(mcfg_params) as compiled into the library, so that bindings
 * (iso_c_binding, ctypes) can verify their copy of the layout. */
int64_t mcfg_sizeof_params(void);

/* Rigid colloids made of boundary particles (sid = colloid number 1..nc),
 * the Colloid object's parameters (mcf/src/Class_Colloid.F90); spheres in
 * 3D, disks in 2D. */
typedef struct mcfg_colloid_params {
  int32_t num_colloid;
  int32_t noslip_type;      /* 1 frozen (rigid velocity), 2 Morris extrapolation */
  int32_t rho_type;         /* 0 constant density, 1 dynamic                 */
  int32_t translate;        /* colloid translates (V used)                    */
  int32_t rotate;           /* colloid rotates (Omega used)                   */
  int32_t pp_interact_cc;   /* boundary particles of different colloids
                               interact (pp_interaction_cc.inc)              */
  int32_t cc_repul_type;    /* 0 none, 1 Hookean, 2 DLVO                      */
  int32_t reserved0;
  double dout;              /* outer layer, mcf_colloid_out_layer_coeff*dx   */
  double cc_repul_F0;
  double cc_repul_cut_off;  /* hn */
  double cc_repul_cut_on;   /* hm */
} mcfg_colloid_params;

/* Per-handle counters, readable at any time. */
typedef struct mcfg_info {
  int64_t num_part;       /* particles uploaded                              */
  int32_t num_cell_dim[3];/* real cells per dimension of the cell list       */
  int32_t num_cell;       /* product of num_cell_dim                         */
  int64_t num_outside;    /* particles outside the cell mesh at the last
                             list build (PPM gives them no box; they do not
                             interact)                                       */
  int64_t num_pairs;      /* directed pairs inside the cut-off, last build   */
  int32_t max_neigh;      /* largest per-particle neighbour count           */
  int32_t neigh_capacity; /* per-particle neighbour list capacity           */
  int64_t kernel_launches;/* kernels launched by this handle so far          */
  int64_t device_bytes;   /* device memory held by the handle               */
  int64_t list_rebuilds;  /* candidate-list rebuilds so far (list reuse)    */
  double skin;            /* list-reuse skin (0: reuse off)                  */
  double time_current;    /* MCF's time_current (advanced by dt per step)    */
  double shear_length;    /* Lees-Edwards offset along x of the images above
                             the y+ face at the last boundary update        */
} mcfg_info;

/* Create a handle on params->device.  Replaces the construction of MCF's
 * Technique/Kernel/Rhs/StateEquation objects, mcf/src/mcf.F90:335-659
 * (kernel_new.F90:41-93, stateEquation_new.F90:65-110). */
int mcfg_create(const mcfg_params* params, mcfg_handle** out);

/* Release all device memory of the handle. */
int mcfg_destroy(mcfg_handle* h);

/* Message of the last failing call on this handle (never NULL). */
const char* mcfg_last_error(const mcfg_handle* h);

/* Message of the last mcfg_create failure (no handle exists yet). */
const char* mcfg_create_error(void);

int mcfg_get_info(const mcfg_handle* h, mcfg_info* info);

/* Copy the real particles to the device (host order is kept as the
 * particle index of every output).  x, v: [n*d]; m: [n]; id: [n*2];
 * ct: [n*d*d] conformation tensor or NULL (Newtonian).  Replaces the
 * particle arrays of Class_Particles (mcf/src/Class_Particles.F90:132-141)
 * as produced by particles_init_* / io_read_particles. */
int mcfg_upload(mcfg_handle* h, int64_t n, const double* x, const double* v,
                const double* m, const int32_t* id, const double* ct);

/* Load accelerations f(d,N) in host order (e.g. MCF's this%f of the last
 * step) so that mcfg_step_vv can follow mcfg_upload directly, as when MCF
 * keeps its particle arrays on the host between steps. */
int mcfg_upload_force(mcfg_handle* h, const double* f);

/* Periodic wrap of the real particles, particles_adjust_particles.F90:137-389
 * (periodic faces only; solid-wall faces clamp wall particles). */
int mcfg_adjust_particles(mcfg_handle* h);

/* Build the cell list of the current positions.  Replaces
 * technique_build_list (mcf/src/technique_build_list.F90:94-109) ->
 * ppm_neighlist_clist -> ppm_util_rank3d/2d.  Cells are the real cells of
 * PPM's mesh, numbered i + j*Nx + k*Nx*Ny (0-based).  Optional outputs:
 * num_cell_dim[3]; cell_start[num_cell+1] (0-based CSR, like PPM lhbx minus
 * one and restricted to real cells); lpdx[n] (0-based host particle indices
 * sorted by cell, stable in host index order, like PPM lpdx). */
int mcfg_build_list(mcfg_handle* h, int32_t* num_cell_dim,
                    int32_t* cell_start, int32_t* lpdx);

/* Density summation, particles_compute_density.F90:369-867 with
 * rhs_density.F90:95-96 (includes the self term W(0) and the half-shell
 * pair fold-back of particles_map_ghost_put).  Needs mcfg_build_list. */
int mcfg_compute_density(mcfg_handle* h);

/* Overwrite the densities rho[n] (host order) after mcfg_compute_density,
 * before mcfg_compute_pressure: the second ghost get of MCF's step
 * (particles_map_ghost_get.F90 at marching_integrate_VV.F90:1128), for a
 * subdomain whose halo particles' densities come from their owners. */
int mcfg_update_density(mcfg_handle* h, const double* rho);

/* Equation of state for all particles, particles_compute_pressure.F90:66-95
 * -> stateEquation_compute_pressure.F90:147-180. */
int mcfg_compute_pressure(mcfg_handle* h);

/* Pair accelerations f(d,N) (and stress s(d^2,N) if params.stress_tensor),
 * particles_compute_interaction.F90:609-900 with pp_interaction.inc:37-223,
 * rhs_force_ff_Newtonian*.F90; the random term is keyed by
 * (seed, step, min pid, max pid) so dW_ij = dW_ji. */
int mcfg_compute_interaction(mcfg_handle* h, int64_t step);

/* f += body force, particles_apply_body_force.F90:96-353 (types 1-3). */
int mcfg_apply_body_force(mcfg_handle* h);

/* v += lambda*f*dt for fluid particles, particles_integrate_velocity.F90:84-94 */
int mcfg_integrate_velocity(mcfg_handle* h, double dt, double lambda);

/* x += v*dt for fluid particles, particles_integrate_position.F90:82-111
 * (accuracy order 1). */
int mcfg_integrate_position(mcfg_handle* h, double dt);

/* Right-hand side before the first step: list, density, pressure, force,
 * body force, as marching_marching.F90:528-911. */
int mcfg_init_force(mcfg_handle* h, int64_t step);

/* One velocity-Verlet step, marching_integrate_VV.F90:303-1620: half kick,
 * drift, wrap, list, density, pressure, force, body force, half kick. */
int mcfg_step_vv(mcfg_handle* h, int64_t step, double dt);

/* nsteps consecutive VV steps starting at step0 (step numbers step0+1 ...),
 * the loop of marching_marching.F90:1329-1531 without I/O. */
int mcfg_run_vv(mcfg_handle* h, int64_t step0, int32_t nsteps, double dt);

/* One VV step with the state in the caller's host arrays, MCF's per-step
 * drop-in in one call: x, v [n*d] (pinned memory for full speed) go over,
 * the step runs (as mcfg_step_vv), and x, v of the new state come back into
 * the same arrays.  Equivalent to mcfg_update_state(h, x, v, NULL) +
 * mcfg_step_vv + mcfg_download(h, x, v, ...), but the positions' copy back
 * runs on a second stream, overlapping the density and force sweeps (the
 * positions are final once the step's list phase is done).  The forces stay
 * on the device between steps (MCF does not change them between steps;
 * mcfg_download returns them on output steps).  With neighbour-list reuse
 * and page-locked x, v (pinned, or mcfg_host_register), the call replays a
 * CUDA graph captured for these arrays (the copies, the step, the copies
 * back): the same bits as per-step launches, fewer launch gaps.  The arrays
 * must stay registered while the handle steps with them. */
int mcfg_step_vv_host(mcfg_handle* h, int64_t step, double dt, double* x, double* v);

/* Page-lock a caller's host array (cudaHostRegister) so that the copies of
 * mcfg_step_vv_host, mcfg_update_state and mcfg_download run at full DMA
 * speed: MCF's x and v are ordinary Fortran arrays; registering them once
 * after allocation gives the speed of pinned buffers.  Unregister before
 * the array is freed (or reallocated by MCF).  ptr must not already be
 * registered; bytes > 0. */
int mcfg_host_register(mcfg_handle* h, void* ptr, int64_t bytes);
int mcfg_host_unregister(mcfg_handle* h, void* ptr);

/* Overwrite the positions, velocities and/or accelerations (any pointer may
 * be NULL) of the particles of the last mcfg_upload, in host order, keeping
 * the device's particle order and neighbour-list state: MCF's per-step
 * drop-in hands back the arrays it received from mcfg_download (after its
 * own changes, if any), and the next step rebuilds lists only if a particle
 * has moved past the reuse skin.  Positions are taken in the periodic image
 * the device holds.  The particle set (count, ids, masses) must be that of
 * the last mcfg_upload; call mcfg_upload when it changes. */
int mcfg_update_state(mcfg_handle* h, const double* x, const double* v, const double* f);

/* Copy state back in host particle order; any pointer may be NULL.
 * x,v,f: [n*d]; rho,p: [n]; ct: [n*d*d]; s: [n*d*d] (stress_tensor). */
int mcfg_download(mcfg_handle* h, double* x, double* v, double* rho,
                  double* p, double* f, double* ct, double* s);

/* MCF's particle files, formatted on the device in host order and written
 * to path in one host write.  kind 0: the particle output of
 * io_write_particles.F90:225-403 (name it as MCF does,
 * TRIM(output_particles_file)//I8.8 step//'.out'); kind 1: the restart file
 * of io_write_restart_particles.F90:100-215 (the particle count first,
 * list-directed).  One record per particle, format (<ncol>E16.8): x(d) v(d)
 * rho m pid sid, and with flags & 1 (kind 0, stress_tensor on) the stress
 * components s(2) s(3) of MCF's __IO_PARTICLES_STRESS_TOTAL build.  E16.8
 * digits are the correctly rounded decimal values (ties to even), exact for
 * magnitudes in [1e-18, 1e30). */
int mcfg_write_particles(mcfg_handle* h, const char* path, int32_t kind, int32_t flags);

/* One line of MCF's statistic file, io_write_statistic.F90:131-257,
 * appended to path (created when absent; io_open.F90:188-211 appends to an
 * existing file on a restarted run): format (I9,<1+num_data>E16.8) of step,
 * time, kinetic energy, momentum(1:d) and, with stress_tensor on, the
 * stress sums s(2) s(3) -- the global sums mcfg_statistics returns.  The
 * optional columns of runs with flow_v_fixed, dynamic_density_ref or
 * p_energy are not written (those features are not on this path).  A step
 * outside I9's range prints nine asterisks, as Fortran does. */
int mcfg_write_statistic(mcfg_handle* h, const char* path, int64_t step, double time);

/* Moving boundaries, MCF's Boundary object (Class_Boundary.F90: shear_type,
 * shear_v0 = mcfg_params.wall_v, shear_freq) and its time: shear_type[f] 2
 * makes solid-wall face f oscillate, shear_v = wall_v[f] cos(shear_freq[f] t)
 * (boundary_update_boundary.F90:78-98); any other value keeps
 * shear_v = wall_v[f].  time is MCF's time_current before the next step
 * (marching_marching.F90:330); mcfg_step_vv and mcfg_run_vv advance it by dt
 * first, as marching_marching.F90:1393 does.  With solid walls or
 * Lees-Edwards faces a VV step then follows marching_integrate_VV.F90:
 * 783-806 and 1650-1675: boundary update at (time + dt, time + dt/2), wall
 * particles drift with their velocity (particles_integrate_boundary_
 * position.F90), and take the face's shear_v at time + dt at the end of the
 * step (particles_set_boundary_velocity.F90).  Lees-Edwards images above the
 * y+ face sit at x + (wall_v[3][0] - wall_v[2][0]) (time + dt) modulo L_x
 * (ppm_bcdef_le_y.inc) with velocity + (wall_v[3][0] - wall_v[2][0])
 * (particles_set_boundary_ghost_velocity.F90).  Without this call every
 * shear_type is 0 and time_current starts at 0. */
int mcfg_set_boundary_motion(mcfg_handle* h, const int32_t* shear_type /* [6] */,
                             const double* shear_freq /* [6] */, double time);

/* Colloid state for the pair terms: centres x[nc*d], velocities v[nc*d],
 * angular velocities omega[nc*3], radii radius[nc].  The colloid pair
 * terms are pp_interaction_fc.inc / pp_interaction_cf.inc with the Morris
 * no-slip velocity of colloid_noslip_Morris_sphere.F90:129-300 (disk in
 * 2D) or the frozen one (colloid_noslip_frozen.F90); boundary-particle
 * velocities follow particles_set_colloid_velocity.F90:73-95.  Call after
 * mcfg_upload (the boundary particles are the uploaded sid > 0 ones) and
 * again whenever the colloids move. */
int mcfg_set_colloids(mcfg_handle* h, const mcfg_colloid_params* cp,
                      const double* x, const double* v, const double* omega,
                      const double* radius);

/* Move every colloid's boundary particles with it after MCF's Colloid
 * object has integrated the rigid bodies (the O(N_c) Adams-Bashforth
 * translation/rotation stays on the host): each particle is taken relative
 * to the nearest image of its colloid's current centre, turned by the
 * colloid's rotation matrix of the step (rot[9c + i + 3j] = R(i,j), MCF's
 * coll_rot_matrix(:,:,c); NULL or rotate off: no turn), and put at the new
 * centre x_new[c*d..] -- particles_compute_colloid_relative_position.F90 and
 * particles_compute_colloid_absolute_position.F90 around the colloid update
 * of marching_integrate_VV.F90:455-765.  The colloids' state becomes
 * (x_new, v, omega).  Nothing moves unless translate or rotate is on. */
int mcfg_move_colloids(mcfg_handle* h, const double* x_new, const double* rot,
                       const double* v, const double* omega);

/* Rigid-body dynamics of the colloids on the device: the Colloid object's
 * explicit Adams-Bashforth update (integrate_colloid_type 1-2) of
 * marching_integrate_VV.F90:455-765, run inside every mcfg_step_vv /
 * mcfg_run_vv / mcfg_step_vv_host step once this call has been made, so a
 * step needs no host round trip for the colloids.  Per step: the fluid's
 * drag and torque on each colloid from its boundary particles
 * (particles_collect_colloid_interaction.F90:93-136), then per sub-step
 * (dt / sub_time_step): rotation vector from the angular-velocity history
 * (colloid_compute_rotation_vector.F90), rotation matrix
 * (tool_rotation_matrix.F90), accumulated orientation
 * (colloid_compute_accumulation_matrix.F90), angular velocity
 * (colloid_integrate_rotate_velocity.F90), centre and velocity
 * (colloid_integrate_translate_position/_velocity.F90, AB orders 1-5 ramping
 * up from the first step after step_start), colloid-colloid repulsion at
 * the new centres (colloid_compute_interaction.F90 with
 * colloid_compute_repulsion_cc.F90, nearest image, partners in index
 * order), body force (colloid_apply_body_force.F90), accelerations
 * (colloid_compute_translate/rotate_acceleration.F90; spheres and disks),
 * periodic wrap or wall clamp of the centres (colloid_adjust_colloid.F90),
 * and the boundary particles moved with their colloid (relative position
 * turned by the rotation, put at the new centre).  mcfg_init_force then also
 * computes the initial accelerations, as marching_marching.F90:995-1110.
 * Histories use MCF's layouts: v_hist(d, nc, AB), omega_hist(3, nc, AB),
 * f_hist(d, nc, AB), alpha_hist(3, nc, AB) (level 1 first, column-major),
 * acc_matrix(3, 3, nc), theta(3, nc); NULL gives MCF's start: level 1 of
 * v / omega from mcfg_set_colloids and zeros elsewhere, zero accelerations,
 * the identity orientation, zero angles.  mass[nc], mmi[nc*3] (moments of
 * inertia, particles_compute_mass.F90: spheres 0.4 m a^2, disks
 * 0.5 m a^2 in mmi(3)).  Call after mcfg_set_colloids; colloid-wall
 * repulsion and lubrication are not supported (MCFG_ENOTSUP). */
typedef struct mcfg_colloid_dynamics {
  int32_t integrate_AB;    /* Adams-Bashforth order 1..5 (Colloid%integrate_AB) */
  int32_t sub_time_step;   /* colloid sub-steps per fluid step, >= 1          */
  int64_t step_start;      /* MCF's step_start                                 */
  int32_t body_force_type; /* 0 none, 1 constant body_force per unit mass     */
  int32_t reserved0;       /* must be 0                                        */
  double body_force[3];
} mcfg_colloid_dynamics;

int mcfg_set_colloid_dynamics(mcfg_handle* h, const mcfg_colloid_dynamics* cd,
                              const double* mass, const double* mmi, const double* v_hist,
                              const double* omega_hist, const double* f_hist,
                              const double* alpha_hist, const double* acc_matrix,
                              const double* theta);

/* The colloid part of one VV step alone (what mcfg_step_vv runs for the
 * colloids after the fluid's half kick and drift, marching_integrate_VV.F90:
 * 455-765), for stage-by-stage use and comparison; step is the step number
 * of the VV step it belongs to. */
int mcfg_colloid_integrate(mcfg_handle* h, int64_t step, double dt);

/* Colloid state after the last step (any pointer may be NULL), layouts as
 * mcfg_set_colloid_dynamics: x[nc*d], histories, drag[nc*d] (fluid +
 * repulsion + body force, what the last translate acceleration divided by
 * the mass), torque[nc*3], rot_matrix[nc*9] of the last sub-step,
 * acc_matrix[nc*9], acc_vector[nc*4] (axis, angle from acc_matrix as
 * tool_rotation_vector.F90 computes them, for MCF's colloid output),
 * theta[nc*3]. */
int mcfg_get_colloid_state(mcfg_handle* h, double* x, double* v_hist, double* omega_hist,
                           double* f_hist, double* alpha_hist, double* drag, double* torque,
                           double* rot_matrix, double* acc_matrix, double* acc_vector,
                           double* theta);

/* Drag and torque of every colloid from its boundary particles' last
 * accelerations, particles_collect_colloid_interaction.F90:93-136:
 * drag[nc*d] = sum m f, torque[nc*3] = sum r x (m f). */
int mcfg_colloid_drag(mcfg_handle* h, double* drag, double* torque);

/* Colloid-colloid repulsion force[nc*d] (Hookean or DLVO),
 * colloid_compute_repulsion_cc.F90:95-164 over the nearest periodic image
 * of each colloid pair (colloid_compute_interaction.F90:532-576). */
int mcfg_colloid_repulsion(mcfg_handle* h, double* force);

/* Global FP64 sums of statistic_compute_statistic.F90:230-303: kinetic
 * energy and momentum over fluid particles, stress sum over sid >= 0.
 * mom: [3], stress: [9] (column-major d x d); either may be NULL. */
int mcfg_statistics(mcfg_handle* h, double* k_energy, double* momentum,
                    double* stress);

/* The same sums over the first n_owned particles of the last upload (host
 * order): a subdomain's own particles, its ghost copies left out -- the
 * per-rank sums MCF all-reduces at statistic_compute_statistic.F90:348-403. */
int mcfg_statistics_owned(mcfg_handle* h, int64_t n_owned, double* k_energy,
                          double* momentum, double* stress);

/* Wait for all work of the handle to finish (error check point). */
int mcfg_synchronize(mcfg_handle* h);

/* The CUDA stream (cudaStream_t) all kernels of the handle run on, for
 * callers that time or order work around them; NULL on error. */
void* mcfg_get_stream(mcfg_handle* h);

/* Adjoint of the time-averaged stress (differentiation form; MCF has no
 * counterpart, it differentiates the VV step of marching_integrate_VV.F90:
 * 303-1620 as this library computes it).  From the state the handle holds
 * (x0, v0, ct0 as uploaded) the call runs the initial right-hand side at
 * step0 (as mcfg_init_force) and nsteps VV steps step0+1 ... (as
 * mcfg_run_vv) and evaluates
 *     J = (1/nsteps) sum_{t=1..nsteps} sum_q w[q] S_t[q],
 * S_t being the stress mcfg_statistics reports after step t (d*d entries,
 * the same layout; stress_tensor must be on).  The reverse sweep replays
 * the Philox noise of every pair from the same keys, keeps a checkpoint of
 * the state every checkpoint_every steps (<= 0: 20) and recomputes each
 * segment forward before walking it backwards; the pair and density sums
 * have hand-written adjoint kernels.  Outputs (any may be NULL): J;
 * dJ_dparams[3] = dJ/d(eta, tau, c) (c the sound speed of the equation of
 * state, tau at fixed G = n_p kt_p; tau's entry is 0 for a Newtonian run);
 * dJ_dx0, dJ_dv0 [n*d] and dJ_dct0 [n*d*d] (Oldroyd-B only) in host particle
 * order.  Afterwards the handle holds the state after the last step, as
 * mcfg_run_vv would leave it.  Supported: FP64 precision, all-fluid
 * periodic boxes (no walls or colloids), number density (rhs_density_type
 * 2), Hu-Adams force (rhs_force_type 3) with or without the random term,
 * either kernel, either equation of state, body force types 0-3, Newtonian
 * or Oldroyd-B; anything else returns MCFG_ENOTSUP. */
int mcfg_adjoint_run(mcfg_handle* h, int64_t step0, int32_t nsteps, double dt,
                     int32_t checkpoint_every, const double* w, double* J,
                     double* dJ_dparams, double* dJ_dx0, double* dJ_dv0,
                     double* dJ_dct0);

/* Per-phase device timers (CUDA events on the handle's stream), the
 * GPU counterpart of MCF's __DEBUG_INTEGRATE_VV phase times
 * (marching_integrate_VV.F90:131-143,1679-1709).  Phases: 0 cell list,
 * 1 density (+ neighbour list, pressure), 2 pair force (+ body force, kick),
 * 3 kick-drift-wrap, 4 other.  ms[5] total milliseconds, counts[5] launches
 * timed; mcfg_set_profiling(h, 0) stops recording, (h, 1) starts, (h, 2)
 * clears the totals. */
int mcfg_set_profiling(mcfg_handle* h, int mode);
int mcfg_get_phase_times(mcfg_handle* h, double* ms, int64_t* counts);

/* Number density of n particles for callers that cannot allocate device
 * memory (a caching allocator holding its lock, a host that hands over only
 * buffers it registered itself, a fixed device-memory budget).  This entry
 * point has no counterpart in the reference: it is an allocation-free
 * variant of mcfg_compute_density.  x [n*d], m [n], id [n*2] and the output
 * rho [n] are DEVICE pointers owned by the caller, laid out like the host
 * arrays of mcfg_upload; stream is a cudaStream_t (NULL = default stream)
 * and the call is asynchronous on it.  Species rules as mcfg_compute_density:
 * fluid sums over its pairs, walls when params->wall_rho_type is 1, colloid
 * boundary particles (sid > 0) when coll_rho_type is 1 (the rho_type of
 * mcfg_colloid_params; 0 = constant init_density); the others get the
 * constant density.  Sums run in a fixed order (host index order inside
 * each cell): repeated calls give identical bits.  Nothing is allocated: the
 * cell list lives in a fixed array inside the library (about 1.3 MB, held on
 * every GPU that loads the library until the process exits), so
 * n <= 65,536 and the mesh may have at most 65,536 real cells; larger inputs
 * return MCFG_EINVAL.  The first call on a device looks up that array's
 * device address (with the device current); make that first call before
 * any stream capture.  The caller's current device is the same after the
 * call.  All calls share the array: calls whose GPU work overlaps race, so
 * serialise them.  Errors: mcfg_noalloc_error(). */
int mcfg_density_noalloc(const mcfg_params* params, int32_t coll_rho_type, int32_t n,
                         const double* x, const double* m, const int32_t* id, double* rho,
                         void* stream);
/* Status of the last mcfg_density_noalloc on device: waits for stream and
 * sets *flags to 0, or to 1 when a density came out <= 0 or NaN (the handle
 * path's MCFG_EPHYS condition).  Allocates nothing. */
int mcfg_noalloc_status(int32_t device, void* stream, int32_t* flags);
const char* mcfg_noalloc_error(void);

#ifdef __cplusplus
}
#endif

#endif /* MCFG_H */
