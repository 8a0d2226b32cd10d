/*
 * mcf_oracle.h -- CPU FP64 restatement of MCF's SDPD step (test
 * infrastructure only: the parity checker and the timed CPU baseline).
 *
 * Parity status: parity unpinned against reference outputs.  MCF is
 * Fortran 90 + MPI + PPM and cannot be compiled in this image (no gfortran,
 * no MPI); the reference ships no golden vectors.  The restatement is pinned
 * instead by (a) line-by-line correspondence with the cited Fortran, (b) the
 * analytic self-checks in the tests (kernel normalisation, lattice density,
 * momentum conservation, the transient-Poiseuille series solution of
 * mcf/scripts/poiseuille_theoretical_2d.perl, PPM's ghost-count test
 * ppm:test/ppm_module_map_part_ghost_test.F90:89-100) and (c) committed
 * regression fixtures generated from it.
 *
 * The state mirrors MCF's Particles object: reals first, PPM-style periodic
 * ghost copies after them, PPM cell lists over reals+ghosts, the half-shell
 * (symmetry=T) or full (symmetry=F) cell-pair loops and the additive
 * ghost put.  The random term uses the counter-based stream shared with the
 * CUDA path (the reference's sequential RANDOM_NUMBER stream cannot be
 * matched draw for draw).
 */
#ifndef MCF_ORACLE_H
#define MCF_ORACLE_H

#include <stdint.h>
#include "../include/mcfg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_state orc_state;

orc_state* orc_create(const mcfg_params* p, char* err, int errlen);
void orc_destroy(orc_state* s);
const char* orc_last_error(const orc_state* s);

/* threads used by the pair loops.  symmetry = T (MCF's half-shell loops):
 * 1 thread runs them in MCF's sequential order, more threads run x-slabs of
 * cells in two colours (race-free, deterministic).  symmetry = F (full
 * stencil): OpenMP over centre cells. */
int orc_set_threads(orc_state* s, int nthreads);

int orc_upload(orc_state* s, int64_t n, const double* x, const double* v,
               const double* m, const int32_t* id, const double* ct);
int orc_adjust_particles(orc_state* s);
int orc_build_list(orc_state* s);
int orc_export_lists(orc_state* s, int32_t* num_cell_dim, int32_t* cell_start,
                     int32_t* lpdx);
int orc_compute_density(orc_state* s);
int orc_update_density(orc_state* s, const double* rho);
int orc_compute_pressure(orc_state* s);
int orc_compute_interaction(orc_state* s, int64_t step);
int orc_apply_body_force(orc_state* s);
int orc_integrate_velocity(orc_state* s, double dt, double lambda);
int orc_integrate_position(orc_state* s, double dt);
int orc_init_force(orc_state* s, int64_t step);
int orc_step_vv(orc_state* s, int64_t step, double dt);
int orc_run_vv(orc_state* s, int64_t step0, int32_t nsteps, double dt);
/* moving boundaries: shear_type[6] (2 = oscillating solid wall),
 * shear_freq[6], MCF's time_current (advanced by dt at every step) */
int orc_set_boundary_motion(orc_state* s, const int32_t* shear_type, const double* shear_freq,
                            double time);
double orc_time(const orc_state* s);
int orc_download(orc_state* s, double* x, double* v, double* rho, double* p,
                 double* f, double* ct, double* s_out);
int orc_statistics(orc_state* s, double* k_energy, double* momentum,
                   double* stress);
/* the same sums over the first n_owned particles (host order) */
int orc_statistics_owned(orc_state* s, int64_t n_owned, double* k_energy, double* momentum,
                         double* stress);

/* per real particle: sum over its pairs of |pair acceleration| (the scale
 * of the force parity tolerance); valid after orc_compute_interaction */
int orc_force_scale(const orc_state* s, double* out);
int orc_set_colloids(orc_state* s, const mcfg_colloid_params* cp, const double* x,
                     const double* v, const double* omega, const double* radius);
int orc_move_colloids(orc_state* s, const double* x_new, const double* rot, const double* v,
                      const double* omega);
int orc_colloid_drag(orc_state* s, double* drag, double* torque);
int orc_colloid_repulsion(orc_state* s, double* force);
/* rigid-body dynamics of the colloids (marching_integrate_VV.F90:455-765),
 * arguments as mcfg_set_colloid_dynamics; orc_step_vv then runs the colloid
 * part of every step and orc_init_force the initial accelerations */
int orc_set_colloid_dynamics(orc_state* s, const mcfg_colloid_dynamics* cd, const double* mass,
                             const double* mmi, const double* v_hist, const double* omega_hist,
                             const double* f_hist, const double* alpha_hist,
                             const double* acc_matrix, const double* theta);
int orc_colloid_integrate(orc_state* s, int64_t step, double dt);
int orc_get_colloid_state(const orc_state* s, double* x, double* v_hist, double* omega_hist,
                          double* f_hist, double* alpha_hist, double* drag, double* torque,
                          double* rot, double* acc, double* theta);
/* counts: [0] reals, [1] ghosts, [2] pairs inside cut-off (last force) */
int orc_counts(const orc_state* s, int64_t* counts);
/* per-phase wall seconds accumulated since create:
 * [0] wrap+ghost+list, [1] density, [2] pressure+force, [3] update */
int orc_timers(const orc_state* s, double* t);

/* Lattice initialisation of particles_init_global_inter_cubic/_square
 * (sx += dx repeated addition) restricted to fluid, with the mass of
 * particles_compute_mass.F90:363-450; writes n*d positions. */
int64_t orc_lattice(int dim, const double* min_t, const double* max_t,
                    const double* dx, double* x_out, int64_t cap);

/* Philox4x32-10 block, exported for the stream tests. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
/* the six (3D) / three (2D) pair normals of one (seed, step, pid pair) */
void orc_pair_normals(uint64_t seed, int64_t step, int32_t pid_a,
                      int32_t pid_b, int dim, float* z);
void orc_pair_normals_batch(uint64_t seed, int64_t step, int64_t npairs, const int32_t* pa,
                            const int32_t* pb, int dim, float* z);
/* the Hu-Adams random vector We of pair (pidi, pidj) with unit vector e */
int orc_pair_we(const orc_state* s, int64_t step, int32_t pidi, int32_t pidj, const double* e,
                double* We);

/* kernel value and derivative (kernel_kernel_*), for unit tests */
int orc_kernel(const orc_state* s, double r, double* w, double* gradw);

#ifdef __cplusplus
}
#endif
#endif
