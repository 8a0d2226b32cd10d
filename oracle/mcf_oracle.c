/*
 * mcf_oracle.c -- CPU FP64 restatement of MCF's SDPD right-hand side and
 * velocity-Verlet step.  TEST INFRASTRUCTURE ONLY: it is the parity checker
 * of the CUDA path and the timed CPU baseline; the product never links it.
 *
 * Parity unpinned (see mcf_oracle.h): MCF cannot be built here and ships no
 * golden vectors.  Each routine cites the Fortran it restates
 * (paths relative to the MCF project; "ppm:" = libppm-1.1.1/src inside
 * ppm/distfiles/libppm-1.1.1.tar.gz).
 *
 * Build with -ffp-contract=off so that every FP64 expression is rounded as
 * the gfortran -O2 x86-64 build of MCF rounds it (no fused multiply-add).
 */
#include "mcf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MK_PI 3.141592653589793238 /* mcf_header.F90:50 */
#define MAX_NNP 27

struct orc_state {
  mcfg_params p;
  int d;
  /* kernel (kernel_new.F90:41-93) */
  double h, coef, coef_grad, cut_off2;
  /* Batchelor p0 (stateEquation_new.F90:102-103) */
  double p0;
  double gs;           /* ghost size = cut_off * 1.0001 (mcf.F90:617) */
  double len[3];       /* max_phys_t - min_phys_t                      */
  double machine_zero; /* technique_new.F90:361-363 -> 1e-14           */
  int periodic[3];
  /* particles: reals [0,nreal), ghosts [nreal,nall) */
  int64_t nreal, nall, cap;
  double *x, *v, *f, *rho, *pr, *m, *s, *ct;
  double* fabs_sum; /* per particle sum of |pair acceleration| (test scale) */
  double *vgt, *act; /* Oldroyd-B: velocity gradient, d(ct)/dt (d*d per particle) */
  int32_t *pid, *sid;
  int64_t* owner;
  /* cell list (ppm_util_rank3d.F90 / rank2d) */
  int Nm[3], Ngl[6], Nmtot[3];
  int64_t nbox;
  int32_t* lhbx; /* nbox+1, 0-based CSR                                  */
  int32_t* lpdx; /* particle indices (0-based) sorted by box             */
  int64_t nlpdx;
  int32_t* pbox; /* box per particle, -1 = no box                        */
  int inp[MAX_NNP][3], jnp[MAX_NNP][3], nnp;
  int have_list, have_density, have_pressure;
  int64_t npairs;
  int nthreads;
  /* colloids (Class_Colloid): centre, velocity, angular velocity, radius */
  mcfg_colloid_params cp;
  double *cx, *cv, *com, *crad;
  /* rigid-body dynamics of the colloids (Class_Colloid.F90), on when cdyn:
   * mass, moments of inertia mmi(3,num), the Adams-Bashforth histories
   * v(d,num,AB), omega(3,num,AB), f(d,num,AB), alpha(3,num,AB) (level 1
   * first), rot_matrix and acc_matrix (3,3,num), theta(3,num), and the last
   * drag(d,num) / torque(3,num) of colloid_compute_interaction */
  int cdyn;
  mcfg_colloid_dynamics cd;
  double *cm, *cmmi, *cvh, *comh, *cfh, *calh, *crot, *cacc, *ctheta, *cdrag, *ctorque;
  /* moving boundaries (Class_Boundary.F90): shear_type, shear_freq, the
   * current shear_v per face, Lees-Edwards shear_length along x of the y+
   * face (the y- face's is its negative), time_current */
  int walls, le;
  int32_t shear_type[6];
  double shear_freq[6];
  double shear_v[6][3];
  double le_S;
  double time_current;
  double timers[4];
  char err[256];
};

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int fail(orc_state* s, const char* msg) {
  snprintf(s->err, sizeof s->err, "%s", msg);
  return MCFG_EINVAL;
}

const char* orc_last_error(const orc_state* s) { return s ? s->err : "null"; }

/* ------------------------------------------------------------------------
 * Kernel: kernel_new.F90:41-93, kernel_kernel_quintic_spline.F90:69-99,
 * 177-215, kernel_kernel_Lucy.F90:68-78,155-168.
 * ---------------------------------------------------------------------- */
static void kernel_init(orc_state* s) {
  const double rc = s->p.cut_off;
  const int d = s->d;
  if (s->p.kernel_type == 1) {
    s->h = rc / 3.0;
    if (d == 2)
      s->coef = 7.0 / (478.0 * MK_PI * (s->h * s->h));
    else
      s->coef = 3.0 / (359.0 * MK_PI * (s->h * s->h * s->h));
  } else {
    s->h = rc;
    if (d == 2)
      s->coef = 5.0 / (MK_PI * (s->h * s->h));
    else
      s->coef = 105.0 / (16.0 * MK_PI * (s->h * s->h * s->h));
  }
  s->coef_grad = -s->coef / s->h;
}

static inline double pow4(double a) {
  double a2 = a * a;
  return a2 * a2;
}

/* returns W; *gw (if non-NULL) = dW/dr */
static inline double kernel_eval(const orc_state* s, double rij, double* gw) {
  const double sv = rij / s->h;
  if (s->p.kernel_type == 1) {
    const double s1 = 1.0 - sv, s2 = 2.0 - sv, s3 = 3.0 - sv;
    double s1_4 = pow4(s1), s2_4 = pow4(s2), s3_4 = pow4(s3);
    const double s1_5 = 15.0 * s1_4 * s1;
    const double s2_5 = -6.0 * s2_4 * s2;
    const double s3_5 = s3_4 * s3;
    s1_4 = 75.0 * s1_4;
    s2_4 = -30.0 * s2_4;
    s3_4 = 5.0 * s3_4;
    double w, g;
    if (sv < 1.0) {
      w = s->coef * (s3_5 + s2_5 + s1_5);
      g = s->coef_grad * (s3_4 + s2_4 + s1_4);
    } else if (sv < 2.0) {
      w = s->coef * (s3_5 + s2_5);
      g = s->coef_grad * (s3_4 + s2_4);
    } else if (sv < 3.0) {
      w = s->coef * s3_5;
      g = s->coef_grad * s3_4;
    } else {
      w = 0.0;
      g = 0.0;
    }
    if (gw) *gw = g;
    return w;
  } else {
    double w = 0.0, g = 0.0;
    if (sv <= 1.0) {
      const double om = 1.0 - sv;
      w = s->coef * (1.0 + 3.0 * sv) * (om * om * om);
      g = s->coef_grad * 12.0 * sv * (om * om);
    }
    if (gw) *gw = g;
    return w;
  }
}

int orc_kernel(const orc_state* s, double r, double* w, double* gradw) {
  double g;
  double wv = kernel_eval(s, r, &g);
  if (w) *w = wv;
  if (gradw) *gradw = g;
  return 0;
}

/* ------------------------------------------------------------------------
 * Counter-based stream (replaces random_random.F90:48-73 /
 * random_random_Gaussian.F90:79-175): Philox4x32-10 of Salmon, Moraes,
 * Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11),
 * Box-Muller normals.  Key = seed, counter = (min pid, max pid, step, call).
 * ---------------------------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* odd multiple of 2^-24 in (0,1): exact in FP32 */
static inline float u01(uint32_t r) {
  return (float)((r >> 9) * 2u + 1u) * (1.0f / 16777216.0f);
}

/* Box-Muller pair; the device code calls CUDA's logf / sincospif, here the
 * same quantities are formed in double and rounded to float. */
static inline void box_muller(uint32_t a, uint32_t b, float* z0, float* z1) {
  const float u1 = u01(a), u2 = u01(b);
  const float lg = (float)log((double)u1);
  const float rad = sqrtf(-2.0f * lg);
  /* angle 2 pi u2 - pi, on [-pi, pi] */
  const double th = 2.0 * MK_PI * (double)u2 - MK_PI;
  const float cs = (float)cos(th), sn = (float)sin(th);
  *z0 = rad * cs;
  *z1 = rad * sn;
}

/* Normals for one pair: 3D -> z[0..5] (diag 0..2, off-diagonal 3..5),
 * 2D -> z[0..2] (diag 0..1, off-diagonal 2).  Independent of pair order. */
void orc_pair_normals(uint64_t seed, int64_t step, int32_t pid_a, int32_t pid_b,
                      int dim, float* z) {
  const uint32_t a = (uint32_t)(pid_a < pid_b ? pid_a : pid_b);
  const uint32_t b = (uint32_t)(pid_a < pid_b ? pid_b : pid_a);
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {a, b, (uint32_t)step, 0u};
  uint32_t r[4];
  orc_philox4x32_10(ctr, key, r);
  box_muller(r[0], r[1], &z[0], &z[1]);
  float t0, t1;
  box_muller(r[2], r[3], &t0, &t1);
  z[2] = t0;
  if (dim == 3) {
    z[3] = t1;
    ctr[3] = 1u;
    orc_philox4x32_10(ctr, key, r);
    box_muller(r[0], r[1], &z[4], &z[5]);
  }
}

/* the normals of many pairs (z[k*6 ...]) for checkers that evaluate pairs
 * in their own order */
void orc_pair_normals_batch(uint64_t seed, int64_t step, int64_t npairs, const int32_t* pa,
                            const int32_t* pb, int dim, float* z) {
  for (int64_t k = 0; k < npairs; ++k) orc_pair_normals(seed, step, pa[k], pb[k], dim, z + 6 * k);
}

/* ------------------------------------------------------------------------
 * Create / destroy
 * ---------------------------------------------------------------------- */
orc_state* orc_create(const mcfg_params* p, char* err, int errlen) {
  const char* msg = NULL;
  if (!p)
    msg = "params NULL";
  else if (p->num_dim != 2 && p->num_dim != 3)
    msg = "num_dim must be 2 or 3";
  else if (!(p->cut_off > 0.0))
    msg = "cut_off must be positive";
  else if (p->kernel_type != 1 && p->kernel_type != 2)
    msg = "kernel_type must be 1 or 2";
  else if (p->rhs_density_type != 1 && p->rhs_density_type != 2)
    msg = "rhs_density_type must be 1 or 2";
  else if (p->rhs_force_type < 1 || p->rhs_force_type > 4)
    msg = "rhs_force_type must be 1..4";
  else if (p->stateEquation_type != 1 && p->stateEquation_type != 2)
    msg = "stateEquation_type must be 1 or 2";
  else if (!p->Newtonian && p->rhs_force_type != 3)
    msg = "the Oldroyd-B model needs rhs_force_type 3 (Hu-Adams)";
  else if (!p->Newtonian && !(fabs(p->tau) > 1e-14))
    msg = "tau should not be zero";
  else if ((p->bcdef[2] == MCFG_BC_LE) != (p->bcdef[3] == MCFG_BC_LE))
    msg = "Lees-Edwards faces come in pairs";
  if (msg) {
    if (err) snprintf(err, (size_t)errlen, "%s", msg);
    return NULL;
  }
  orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
  s->p = *p;
  s->d = p->num_dim;
  if (!(s->p.cell_factor > 0.0)) s->p.cell_factor = 1.0001;
  kernel_init(s);
  s->cut_off2 = p->cut_off * p->cut_off;
  s->gs = p->cut_off * s->p.cell_factor;
  /* stateEquation_new.F90:102-103 */
  if (p->stateEquation_type == 2)
    s->p0 = p->c * p->c * p->rho * pow(p->rho_ref / p->rho, p->gamma) / p->gamma;
  s->machine_zero = 1e-14; /* 10**(INT(LOG10(EPSILON(1d0)))+1) */
  for (int i = 0; i < s->d; ++i) {
    s->len[i] = p->max_phys_t[i] - p->min_phys_t[i];
    s->periodic[i] = (p->bcdef[2 * i] == MCFG_BC_PERIODIC);
  }
  /* boundary_set_bcdef (boundary_set.F90): num_shear counts wall and
   * Lees-Edwards faces; shear_v starts at shear_v0 (boundary_set_shear_v0) */
  for (int f = 0; f < 2 * s->d; ++f) {
    if (p->bcdef[f] == MCFG_BC_WALL_SOLID) s->walls = 1;
    if (p->bcdef[f] == MCFG_BC_LE) s->le = 1;
  }
  memcpy(s->shear_v, p->wall_v, sizeof s->shear_v);
  s->nthreads = 1;
  return s;
}

/* boundary_update_boundary.F90:78-122: oscillating solid walls
 * shear_v = shear_v0 cos(shear_freq time_v) (with walls), Lees-Edwards
 * shear_length = (shear_v0(y+) - shear_v0(y-)) time_r along x */
static void boundary_update(orc_state* s, double time_r, double time_v) {
  for (int f = 0; f < 6; ++f)
    if (s->walls && s->shear_type[f] == 2)
      for (int a = 0; a < 3; ++a)
        s->shear_v[f][a] = s->p.wall_v[f][a] * cos(s->shear_freq[f] * time_v);
  if (s->le) s->le_S = (s->p.wall_v[3][0] - s->p.wall_v[2][0]) * time_r;
}

int orc_set_boundary_motion(orc_state* s, const int32_t* shear_type, const double* shear_freq,
                            double time) {
  for (int f = 0; f < 6; ++f) {
    s->shear_type[f] = shear_type[f];
    s->shear_freq[f] = shear_freq[f];
  }
  s->time_current = time;
  boundary_update(s, time, time);
  return 0;
}

double orc_time(const orc_state* s) { return s->time_current; }

/* gfortran's MODULO for reals (p > 0): fmod, plus p for a negative
 * remainder */
static double f_modulo(double a, double p) {
  double r = fmod(a, p);
  if (r < 0.0) r = r + p;
  return r;
}

static void free_arrays(orc_state* s) {
  free(s->x); free(s->v); free(s->f); free(s->rho); free(s->pr); free(s->m);
  free(s->s); free(s->ct); free(s->pid); free(s->sid); free(s->owner); free(s->fabs_sum);
  free(s->vgt); free(s->act);
  s->x = s->v = s->f = s->rho = s->pr = s->m = s->s = s->ct = s->fabs_sum = NULL;
  s->vgt = s->act = NULL;
  s->pid = s->sid = NULL;
  s->owner = NULL;
}

void orc_destroy(orc_state* s) {
  if (!s) return;
  free_arrays(s);
  free(s->cx); free(s->cv); free(s->com); free(s->crad);
  free(s->cm); free(s->cmmi); free(s->cvh); free(s->comh); free(s->cfh); free(s->calh);
  free(s->crot); free(s->cacc); free(s->ctheta); free(s->cdrag); free(s->ctorque);
  free(s->lhbx); free(s->lpdx); free(s->pbox);
  free(s);
}

int orc_set_threads(orc_state* s, int nthreads) {
  s->nthreads = nthreads < 1 ? 1 : nthreads;
  return 0;
}

static void ensure_cap(orc_state* s, int64_t need) {
  if (need <= s->cap) return;
  int64_t cap = need + need / 2 + 16;
  const int d = s->d, d2 = s->d * s->d;
  s->x = (double*)realloc(s->x, sizeof(double) * (size_t)(cap * d));
  s->v = (double*)realloc(s->v, sizeof(double) * (size_t)(cap * d));
  s->f = (double*)realloc(s->f, sizeof(double) * (size_t)(cap * d));
  s->rho = (double*)realloc(s->rho, sizeof(double) * (size_t)cap);
  s->pr = (double*)realloc(s->pr, sizeof(double) * (size_t)cap);
  s->m = (double*)realloc(s->m, sizeof(double) * (size_t)cap);
  s->s = (double*)realloc(s->s, sizeof(double) * (size_t)(cap * d2));
  s->ct = (double*)realloc(s->ct, sizeof(double) * (size_t)(cap * d2));
  s->pid = (int32_t*)realloc(s->pid, sizeof(int32_t) * (size_t)cap);
  s->sid = (int32_t*)realloc(s->sid, sizeof(int32_t) * (size_t)cap);
  s->owner = (int64_t*)realloc(s->owner, sizeof(int64_t) * (size_t)cap);
  s->fabs_sum = (double*)realloc(s->fabs_sum, sizeof(double) * (size_t)cap);
  s->vgt = (double*)realloc(s->vgt, sizeof(double) * (size_t)(cap * d2));
  s->act = (double*)realloc(s->act, sizeof(double) * (size_t)(cap * d2));
  s->cap = cap;
}

int orc_upload(orc_state* s, int64_t n, const double* x, const double* v,
               const double* m, const int32_t* id, const double* ct) {
  if (n < 0 || (n > 0 && (!x || !v || !m || !id))) return fail(s, "orc_upload: bad arguments");
  const int d = s->d, d2 = d * d;
  ensure_cap(s, n + 1);
  memcpy(s->x, x, sizeof(double) * (size_t)(n * d));
  memcpy(s->v, v, sizeof(double) * (size_t)(n * d));
  memcpy(s->m, m, sizeof(double) * (size_t)n);
  for (int64_t j = 0; j < n; ++j) {
    s->pid[j] = id[2 * j];
    s->sid[j] = id[2 * j + 1];
    s->owner[j] = j;
  }
  if (ct)
    memcpy(s->ct, ct, sizeof(double) * (size_t)(n * d2));
  else
    for (int64_t j = 0; j < n; ++j)
      for (int a = 0; a < d2; ++a) s->ct[j * d2 + a] = (a % (d + 1) == 0) ? 1.0 : 0.0;
  memset(s->f, 0, sizeof(double) * (size_t)(n * d));
  memset(s->rho, 0, sizeof(double) * (size_t)n);
  memset(s->pr, 0, sizeof(double) * (size_t)n);
  memset(s->s, 0, sizeof(double) * (size_t)(n * d2));
  memset(s->vgt, 0, sizeof(double) * (size_t)(n * d2));
  memset(s->act, 0, sizeof(double) * (size_t)(n * d2));
  s->nreal = s->nall = n;
  s->have_list = s->have_density = s->have_pressure = 0;
  return 0;
}

/* ------------------------------------------------------------------------
 * Periodic wrap, particles_adjust_particles.F90:137-389 (periodic faces;
 * solid walls clamp wall particles to the total domain).
 * ---------------------------------------------------------------------- */
int orc_adjust_particles(orc_state* s) {
  const int d = s->d;
  const double* mn = s->p.min_phys;
  const double* mx = s->p.max_phys;
  for (int64_t j = 0; j < s->nreal; ++j) {
    for (int i = 0; i < d; ++i) {
      double* xi = &s->x[j * d + i];
      if (s->p.bcdef[2 * i] == MCFG_BC_LE) {
        /* particles_adjust_particles.F90:228-257, 352-381: through the
         * lower face x(i) + length, the others MODULO(x(k) -
         * shear_length(k, 2i-1), length(k)), v(k) + shear_v(k, 2i) -
         * shear_v(k, 2i-1); the upper face alike; then no further axis
         * (EXIT).  shear_length(x, y-) = -S, (x, y+) = S, 0 along z. */
        if (s->sid[j] < 0) continue;
        int face = 0;
        if (*xi < mn[i])
          face = 1;
        else if (*xi >= mx[i])
          face = 2;
        if (face == 0) continue;
        const double lk = mx[i] - mn[i];
        *xi = (face == 1) ? *xi + lk : *xi - lk;
        for (int k = 0; k < d; ++k) {
          if (k == i) continue;
          const double sl = (k == 0) ? (face == 1 ? -s->le_S : s->le_S) : 0.0;
          const double lenk = mx[k] - mn[k];
          s->x[j * d + k] = f_modulo(s->x[j * d + k] - sl, lenk);
          const double jump = (face == 1) ? s->shear_v[2 * i + 1][k] - s->shear_v[2 * i][k]
                                          : s->shear_v[2 * i][k] - s->shear_v[2 * i + 1][k];
          s->v[j * d + k] = s->v[j * d + k] + jump;
        }
        break;
      }
      if (*xi < mn[i]) {
        if (s->p.bcdef[2 * i] == MCFG_BC_PERIODIC) {
          *xi = *xi + s->len[i];
        } else if (s->p.bcdef[2 * i] == MCFG_BC_WALL_SOLID) {
          if (s->sid[j] < 0 && *xi < s->p.min_phys_t[i]) {
            *xi = s->p.min_phys_t[i];
            s->v[j * d + i] = 0.0;
          }
        }
      }
      if (*xi >= mx[i]) {
        if (s->p.bcdef[2 * i + 1] == MCFG_BC_PERIODIC) {
          *xi = *xi - s->len[i];
        } else if (s->p.bcdef[2 * i + 1] == MCFG_BC_WALL_SOLID) {
          if (s->sid[j] < 0 && *xi > s->p.max_phys_t[i]) {
            *xi = s->p.max_phys_t[i] - s->machine_zero;
            s->v[j * d + i] = 0.0;
          }
        }
      }
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------
 * Periodic ghosts, ppm:src/ppm_map_part_ghost_get.F90:441-525 with
 * ppm_bcdef_periodic_{x,y,z}.inc: images x + len for x < min + ghostsize
 * (and, without symmetry, x - len for x > max - ghostsize), x first, then y
 * over reals and x-images, then z.  Ghost fields are copies of the owner.
 * ---------------------------------------------------------------------- */
static void copy_particle(orc_state* s, int64_t to, int64_t from) {
  const int d = s->d, d2 = d * d;
  memcpy(&s->x[to * d], &s->x[from * d], sizeof(double) * (size_t)d);
  memcpy(&s->v[to * d], &s->v[from * d], sizeof(double) * (size_t)d);
  memcpy(&s->ct[to * d2], &s->ct[from * d2], sizeof(double) * (size_t)d2);
  s->m[to] = s->m[from];
  s->rho[to] = s->rho[from];
  s->pr[to] = s->pr[from];
  s->pid[to] = s->pid[from];
  s->sid[to] = s->sid[from];
  s->owner[to] = s->owner[from];
}

static void ghost_get(orc_state* s) {
  const int d = s->d;
  s->nall = s->nreal;
  if (s->le) {
    /* ppm_bcdef_le_y.inc (before the periodic images,
     * ppm_map_part_ghost_get.F90:776-800): a particle with y in
     * [min, min + ghostsize) gets an image at y + len, other coordinates
     * MODULO(x + shear_length(x, y+), len); without symmetry also
     * (max - ghostsize, max] at y - len with shear_length(x, y-) */
    const double ymin = s->p.min_phys[1], ymax = s->p.max_phys[1];
    const double ly = ymax - ymin;
    const int64_t nnow = s->nall;
    for (int64_t i = 0; i < nnow; ++i) {
      const double yv = s->x[i * d + 1];
      if (yv >= ymin && yv < ymin + s->gs) {
        ensure_cap(s, s->nall + 1);
        copy_particle(s, s->nall, i);
        double* xg = &s->x[s->nall * d];
        xg[1] = yv + ly;
        xg[0] = f_modulo(xg[0] + s->le_S, s->p.max_phys[0] - s->p.min_phys[0]);
        if (d == 3) xg[2] = f_modulo(xg[2] + 0.0, s->p.max_phys[2] - s->p.min_phys[2]);
        s->nall++;
      }
    }
    if (!s->p.symmetry) {
      for (int64_t i = 0; i < nnow; ++i) {
        const double yv = s->x[i * d + 1];
        if (yv > ymax - s->gs && yv <= ymax) {
          ensure_cap(s, s->nall + 1);
          copy_particle(s, s->nall, i);
          double* xg = &s->x[s->nall * d];
          xg[1] = yv - ly;
          xg[0] = f_modulo(xg[0] - s->le_S, s->p.max_phys[0] - s->p.min_phys[0]);
          if (d == 3) xg[2] = f_modulo(xg[2] + 0.0, s->p.max_phys[2] - s->p.min_phys[2]);
          s->nall++;
        }
      }
    }
  }
  for (int dim = 0; dim < d; ++dim) {
    if (!s->periodic[dim]) continue;
    const double xminf = s->p.min_phys_t[dim], xmini = xminf + s->gs;
    const double xmaxf = s->p.max_phys_t[dim], xmaxi = xmaxf - s->gs;
    const int64_t nnow = s->nall;
    for (int64_t i = 0; i < nnow; ++i) {
      const double xv = s->x[i * d + dim];
      if (xv >= xminf && xv < xmini) {
        ensure_cap(s, s->nall + 1);
        copy_particle(s, s->nall, i);
        s->x[s->nall * d + dim] = xv + s->len[dim];
        s->nall++;
      }
    }
    if (!s->p.symmetry) {
      for (int64_t i = 0; i < nnow; ++i) {
        const double xv = s->x[i * d + dim];
        if (xv > xmaxi && xv <= xmaxf) {
          ensure_cap(s, s->nall + 1);
          copy_particle(s, s->nall, i);
          s->x[s->nall * d + dim] = xv - s->len[dim];
          s->nall++;
        }
      }
    }
  }
}

/* refresh ghost copies of rho, v, p (second ghost get,
 * marching_integrate_VV.F90:1128) */
static void ghost_refresh(orc_state* s) {
  const int d = s->d, d2 = d * d;
  for (int64_t g = s->nreal; g < s->nall; ++g) {
    const int64_t o = s->owner[g];
    s->rho[g] = s->rho[o];
    s->pr[g] = s->pr[o];
    memcpy(&s->v[g * d], &s->v[o * d], sizeof(double) * (size_t)d);
    memcpy(&s->ct[g * d2], &s->ct[o * d2], sizeof(double) * (size_t)d2);
    if (s->le) {
      /* particles_set_boundary_ghost_velocity.F90: a ghost beyond a
       * Lees-Edwards face moves with the face velocity difference */
      const double yg = s->x[g * d + 1];
      for (int k = 0; k < d; ++k) {
        if (k == 1) continue;
        if (yg < s->p.min_phys[1])
          s->v[g * d + k] = s->v[g * d + k] + (s->shear_v[2][k] - s->shear_v[3][k]);
        else if (yg >= s->p.max_phys[1])
          s->v[g * d + k] = s->v[g * d + k] + (s->shear_v[3][k] - s->shear_v[2][k]);
      }
    }
  }
}

/* ------------------------------------------------------------------------
 * Cell list: ppm:src/ppm_neighlist_clist.F90:318-438 ->
 * ppm:src/ppm_util_rank3d.F90:308-531 (rank2d alike) and
 * ppm:src/ppm_neighlist_MkNeighIdx.F90:146-269.
 * ---------------------------------------------------------------------- */
static void make_neigh_idx(orc_state* s) {
  memset(s->inp, 0, sizeof s->inp);
  memset(s->jnp, 0, sizeof s->jnp);
  if (s->p.symmetry) {
    if (s->d == 2) {
      s->nnp = 5;
      s->jnp[1][0] = 1;                    /* 0 -- 1 */
      s->inp[2][1] = 1;                    /* 0 -- 3 */
      s->jnp[3][0] = 1; s->jnp[3][1] = 1;  /* 0 -- 4 */
      s->inp[4][0] = 1; s->jnp[4][1] = 1;  /* 1 -- 3 */
    } else {
      s->nnp = 14;
      s->jnp[1][0] = 1;
      s->inp[2][1] = 1;
      s->jnp[3][0] = 1; s->jnp[3][1] = 1;
      s->jnp[4][2] = 1;
      s->jnp[5][0] = 1; s->jnp[5][2] = 1;
      s->jnp[6][1] = 1; s->jnp[6][2] = 1;
      s->jnp[7][0] = 1; s->jnp[7][1] = 1; s->jnp[7][2] = 1;
      s->inp[8][0] = 1; s->jnp[8][1] = 1;
      s->inp[9][0] = 1; s->jnp[9][2] = 1;
      s->inp[10][0] = 1; s->jnp[10][1] = 1; s->jnp[10][2] = 1;
      s->inp[11][1] = 1; s->jnp[11][2] = 1;
      s->inp[12][1] = 1; s->jnp[12][0] = 1; s->jnp[12][2] = 1;
      s->inp[13][0] = 1; s->inp[13][1] = 1; s->jnp[13][2] = 1;
    }
  } else {
    const int nz = (s->d == 3) ? 1 : 0;
    int l = 0;
    for (int k = -nz; k <= nz; ++k)
      for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) {
          s->jnp[l][0] = i;
          s->jnp[l][1] = j;
          s->jnp[l][2] = k;
          ++l;
        }
    s->nnp = l;
  }
}

static int rank_particles(orc_state* s) {
  const int d = s->d;
  double xmin[3], xmax[3], rdx[3];
  for (int i = 0; i < d; ++i) {
    xmin[i] = s->p.min_phys_t[i];
    xmax[i] = s->p.max_phys_t[i];
    int nm = (int)((xmax[i] - xmin[i]) / s->gs); /* clist.F90:370-376 */
    if (nm < 1) nm = 1;
    s->Nm[i] = nm;
  }
  for (int i = 0; i < 6; ++i) s->Ngl[i] = 0;
  for (int i = 0; i < d; ++i) {
    if (s->p.symmetry) {
      s->Ngl[d + i] = 1;
    } else {
      s->Ngl[i] = 1;
      s->Ngl[d + i] = 1;
    }
  }
  s->nbox = 1;
  for (int i = 0; i < 3; ++i) s->Nmtot[i] = 1;
  for (int i = 0; i < d; ++i) {
    s->Nmtot[i] = s->Nm[i] + s->Ngl[i] + s->Ngl[d + i];
    s->nbox *= s->Nmtot[i];
    rdx[i] = (double)s->Nm[i] / (xmax[i] - xmin[i]); /* rank3d.F90:352-354 */
  }
  free(s->lhbx);
  free(s->pbox);
  free(s->lpdx);
  s->lhbx = (int32_t*)calloc((size_t)s->nbox + 1, sizeof(int32_t));
  s->pbox = (int32_t*)malloc(sizeof(int32_t) * (size_t)(s->nall + 1));
  int32_t* npbx = (int32_t*)calloc((size_t)s->nbox + 1, sizeof(int32_t));
  const int64_t n2 = (int64_t)s->Nmtot[0] * s->Nmtot[1];
  int64_t icount = 0;
  for (int64_t ip = 0; ip < s->nall; ++ip) {
    int c[3] = {0, 0, 0};
    for (int a = 0; a < d; ++a) {
      const double xa = s->x[ip * d + a];
      /* rank3d.F90:422-424: subtraction before multiplication */
      int ia = (int)floor((xa - xmin[a]) * rdx[a]) + s->Ngl[a];
      const int top = s->Nm[a] + s->Ngl[a];
      if (xa >= xmax[a] && ia < top) ia = top;      /* :433-445 */
      if (xa < xmax[a] && ia >= top) ia = top - 1;  /* :447-459 */
      c[a] = ia;
    }
    int inside = 1;
    for (int a = 0; a < d; ++a)
      if (c[a] < 0 || c[a] >= s->Nmtot[a]) inside = 0;
    if (inside) {
      const int64_t ibox = c[0] + (int64_t)c[1] * s->Nmtot[0] + (int64_t)c[2] * n2;
      s->pbox[ip] = (int32_t)ibox;
      npbx[ibox]++;
      icount++;
    } else {
      s->pbox[ip] = -1;
    }
  }
  /* stable counting sort, rank3d.F90:504-531 */
  s->lhbx[0] = 0;
  for (int64_t b = 0; b < s->nbox; ++b) s->lhbx[b + 1] = s->lhbx[b] + npbx[b];
  s->lpdx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(icount + 1));
  s->nlpdx = icount;
  for (int64_t b = 0; b < s->nbox; ++b) npbx[b] = s->lhbx[b];
  for (int64_t ip = 0; ip < s->nall; ++ip) {
    const int32_t b = s->pbox[ip];
    if (b >= 0) s->lpdx[npbx[b]++] = (int32_t)ip;
  }
  free(npbx);
  make_neigh_idx(s);
  return 0;
}

int orc_build_list(orc_state* s) {
  const double t0 = now_s();
  ghost_get(s);
  rank_particles(s);
  s->have_list = 1;
  s->have_density = s->have_pressure = 0;
  s->timers[0] += now_s() - t0;
  return 0;
}

/* Real-cell lists in the layout of mcfg_build_list: cells i+j*Nx+k*Nx*Ny
 * over the real cells only; entries are real particle indices. */
int orc_export_lists(orc_state* s, int32_t* num_cell_dim, int32_t* cell_start,
                     int32_t* lpdx) {
  if (!s->have_list) return fail(s, "orc_export_lists: no list");
  const int d = s->d;
  int nm[3] = {1, 1, 1};
  for (int a = 0; a < d; ++a) nm[a] = s->Nm[a];
  if (num_cell_dim)
    for (int a = 0; a < 3; ++a) num_cell_dim[a] = nm[a];
  const int64_t n2 = (int64_t)s->Nmtot[0] * s->Nmtot[1];
  int64_t pos = 0, cell = 0;
  for (int k = 0; k < nm[2]; ++k)
    for (int j = 0; j < nm[1]; ++j)
      for (int i = 0; i < nm[0]; ++i) {
        const int64_t ibox = (i + s->Ngl[0]) + (int64_t)(j + s->Ngl[1]) * s->Nmtot[0] +
                             (d == 3 ? (int64_t)(k + s->Ngl[2]) * n2 : 0);
        if (cell_start) cell_start[cell] = (int32_t)pos;
        for (int32_t q = s->lhbx[ibox]; q < s->lhbx[ibox + 1]; ++q) {
          const int32_t ip = s->lpdx[q];
          if (ip < s->nreal) {
            if (lpdx) lpdx[pos] = ip;
            pos++;
          }
        }
        cell++;
      }
  if (cell_start) cell_start[cell] = (int32_t)pos;
  return 0;
}

/* ------------------------------------------------------------------------
 * Cell-pair iteration shared by density and force:
 * particles_compute_density.F90:578-867, particles_compute_interaction.F90:
 * 609-900.  Symmetric: real cells 0..Nm-1, 14/5 cell pairs, j>i inside one
 * cell; full: real cells with 27/9 neighbours, self excluded.
 * ---------------------------------------------------------------------- */
typedef void (*pair_fn)(orc_state* s, int64_t ip, int64_t jp, void* ctx);

static void cell_range(const orc_state* s, int* st, int* en) {
  const int d = s->d;
  for (int a = 0; a < 3; ++a) {
    st[a] = 0;
    en[a] = 0;
  }
  for (int a = 0; a < d; ++a) {
    if (s->p.symmetry) {
      st[a] = 0;
      en[a] = s->Nmtot[a] - 2;
    } else {
      st[a] = 1;
      en[a] = s->Nmtot[a] - 2;
    }
  }
}

/* one centre cell: all its (icell,jcell) interactions */
static void loop_centre_cell(orc_state* s, int ci, int cj, int ck, pair_fn fn,
                             void* ctx, int64_t* npairs_out) {
  const int d = s->d;
  const int64_t n1 = s->Nmtot[0];
  const int64_t n2 = (d == 2) ? 0 : (int64_t)s->Nmtot[0] * s->Nmtot[1];
  const int64_t ccell = ci + n1 * cj + n2 * ck;
  int64_t np = 0;
  for (int it = 0; it < s->nnp; ++it) {
    const int64_t icell = ccell + s->inp[it][0] + n1 * s->inp[it][1] + n2 * s->inp[it][2];
    const int64_t jcell = ccell + s->jnp[it][0] + n1 * s->jnp[it][1] + n2 * s->jnp[it][2];
    if (icell < 0 || jcell < 0 || icell >= s->nbox || jcell >= s->nbox) continue;
    const int32_t istart = s->lhbx[icell], iend = s->lhbx[icell + 1];
    int32_t jstart = s->lhbx[jcell];
    const int32_t jend = s->lhbx[jcell + 1];
    for (int32_t ipart = istart; ipart < iend; ++ipart) {
      const int64_t ip = s->lpdx[ipart];
      if (jcell == icell && s->p.symmetry) jstart = ipart + 1;
      for (int32_t jpart = jstart; jpart < jend; ++jpart) {
        if (jcell == icell && jpart == ipart) continue;
        const int64_t jp = s->lpdx[jpart];
        fn(s, ip, jp, ctx);
        ++np;
      }
    }
  }
  *npairs_out += np;
}

static void for_all_pairs(orc_state* s, pair_fn fn, void* ctx) {
  int st[3], en[3];
  cell_range(s, st, en);
  const int d = s->d;
  const int kst = (d == 2) ? 0 : st[2], ken = (d == 2) ? 0 : en[2];
  int64_t npairs = 0;
  if (s->nthreads > 1 && !s->p.symmetry) {
    /* full stencil writes only to particles of the centre cell: cells are
     * independent and the loop parallelises without races */
    const int nx = en[0] - st[0] + 1, ny = en[1] - st[1] + 1, nz = ken - kst + 1;
    const int64_t ncell = (int64_t)nx * ny * nz;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(s->nthreads) reduction(+ : npairs)
#endif
    for (int64_t c = 0; c < ncell; ++c) {
      const int i = st[0] + (int)(c % nx);
      const int j = st[1] + (int)((c / nx) % ny);
      const int k = kst + (int)(c / ((int64_t)nx * ny));
      loop_centre_cell(s, i, j, k, fn, ctx, &npairs);
    }
  } else if (s->nthreads > 1) {
    /* MCF's symmetric half-shell loops (symmetry = T) on all threads: each
     * centre cell writes to particles of cells at x offsets 0 and +1 only
     * (ppm_neighlist_MkNeighIdx's 2x2x2 block; periodic images are ghost
     * copies, folded back after the loop), so x-slabs of at least one cell
     * column, run in two colours (even slabs, then odd), never write the
     * same particle at the same time.  Each particle's sums keep a fixed
     * order: deterministic, and equal to the sequential loops to rounding. */
    const int nx = en[0] - st[0] + 1;
    int nslab = 2 * s->nthreads;
    if (nslab > nx) nslab = nx;
    for (int colour = 0; colour < 2; ++colour) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(s->nthreads) reduction(+ : npairs)
#endif
      for (int q = colour; q < nslab; q += 2) {
        const int i0 = st[0] + (int)((int64_t)q * nx / nslab);
        const int i1 = st[0] + (int)((int64_t)(q + 1) * nx / nslab);
        for (int k = kst; k <= ken; ++k)
          for (int j = st[1]; j <= en[1]; ++j)
            for (int i = i0; i < i1; ++i) loop_centre_cell(s, i, j, k, fn, ctx, &npairs);
      }
    }
  } else {
    for (int k = kst; k <= ken; ++k)
      for (int j = st[1]; j <= en[1]; ++j)
        for (int i = st[0]; i <= en[0]; ++i) loop_centre_cell(s, i, j, k, fn, ctx, &npairs);
  }
  s->npairs = npairs;
}

/* ------------------------------------------------------------------------
 * Density: particles_compute_density.F90:369-558 (self terms) and
 * :700-855 (pairs), rhs_density.F90:95-96; ghost put particles_map_ghost_put.
 * ---------------------------------------------------------------------- */
static int dyn_rho(const orc_state* s, int32_t sid) {
  if (sid == 0) return 1;
  if (sid < 0) return s->p.wall_rho_type == 1;
  return s->cp.rho_type == 1;
}

/* colloid_in_nearest_image.F90 (periodic part): image of colloid c's centre
 * nearest to x (within radius + dout per axis), its velocity, and
 * rx = x - image */
static void colloid_nearest_image(const orc_state* s, const double* x, int c, double* ximg,
                                  double* rx, double* vimg) {
  const int d = s->d;
  const double dmax = s->crad[c] + s->cp.dout;
  for (int a = 0; a < d; ++a) {
    ximg[a] = s->cx[c * d + a];
    vimg[a] = s->cv[c * d + a];
    const double r = x[a] - ximg[a];
    if (r > dmax && s->periodic[a]) ximg[a] = ximg[a] + s->len[a];
    else if (-r > dmax && s->periodic[a]) ximg[a] = ximg[a] - s->len[a];
    rx[a] = x[a] - ximg[a];
  }
}

static void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

/* colloid_particle_velocity.F90: V + Omega x rx of a boundary particle */
static void colloid_particle_velocity(const orc_state* s, const double* x, int c, double* vout) {
  const int d = s->d;
  for (int a = 0; a < d; ++a) vout[a] = 0.0;
  if (!(s->cp.translate || s->cp.rotate)) return;
  double ximg[3], rx[3] = {0, 0, 0}, vimg[3];
  colloid_nearest_image(s, x, c, ximg, rx, vimg);
  for (int a = 0; a < d; ++a) vout[a] = vimg[a];
  if (s->cp.rotate) {
    double r3[3] = {rx[0], rx[1], d == 3 ? rx[2] : 0.0}, w[3];
    cross3(&s->com[c * 3], r3, w);
    for (int a = 0; a < d; ++a) vout[a] = vout[a] + w[a];
  }
}

/* colloid_noslip_Morris_sphere.F90:129-300 (disk in 2D) and
 * colloid_noslip_frozen.F90: velocity given to boundary particle xc of
 * colloid c seen from fluid particle xf with velocity vf */
static void colloid_noslip(const orc_state* s, const double* xf, const double* xc,
                           const double* vf, int c, double* vc) {
  const int d = s->d;
  double xcoll[3], r_xc[3] = {0, 0, 0}, vcoll[3];
  colloid_nearest_image(s, xc, c, xcoll, r_xc, vcoll);
  const double* om = &s->com[c * 3];
  if (s->cp.noslip_type <= 1) {
    for (int a = 0; a < d; ++a) vc[a] = vcoll[a];
    if (s->cp.rotate) {
      double r3[3] = {r_xc[0], r_xc[1], d == 3 ? r_xc[2] : 0.0}, w[3];
      cross3(om, r3, w);
      for (int a = 0; a < d; ++a) vc[a] = vc[a] + w[a];
    }
    return;
  }
  const double R = s->crad[c];
  double r_xf[3] = {0, 0, 0};
  for (int a = 0; a < d; ++a) r_xf[a] = xf[a] - xcoll[a];
  double dd = 0.0;
  for (int a = 0; a < d; ++a) dd = dd + r_xf[a] * r_xf[a];
  const double d_fcoll = sqrt(dd);
  if (d_fcoll <= R) {
    for (int a = 0; a < d; ++a) vc[a] = vcoll[a];
    if (s->cp.rotate) {
      double r3[3] = {r_xc[0], r_xc[1], d == 3 ? r_xc[2] : 0.0}, w[3];
      cross3(om, r3, w);
      for (int a = 0; a < d; ++a) vc[a] = vc[a] + w[a];
    }
    return;
  }
  double nvec[3] = {0, 0, 0}, d_cn = 0.0;
  for (int a = 0; a < d; ++a) nvec[a] = r_xf[a] / d_fcoll;
  for (int a = 0; a < d; ++a) d_cn = d_cn + r_xc[a] * nvec[a];
  const double d_cs = R - d_cn;
  double d_fs = d_fcoll - R;
  double r_xs[3] = {0, 0, 0};
  for (int a = 0; a < d; ++a) r_xs[a] = R / d_fcoll * r_xf[a];
  double corr;
  if (fabs(d_fs) < s->machine_zero) {
    d_fs = s->machine_zero;
    corr = 0.5; /* mcf_colloid_dist_ratio_max */
  } else {
    corr = d_cs / d_fs;
    if (corr > 0.5) corr = 0.5;
    else if (corr < -0.5) corr = -0.5;
  }
  double r_vs[3] = {0, 0, 0};
  if (s->cp.rotate) cross3(om, r_xs, r_vs);
  for (int a = 0; a < d; ++a) vc[a] = -corr * (vf[a] - vcoll[a] - r_vs[a]) + vcoll[a] + r_vs[a];
}

int orc_set_colloids(orc_state* s, const mcfg_colloid_params* cp, const double* x,
                     const double* v, const double* omega, const double* radius) {
  const int nc = cp->num_colloid, d = s->d;
  s->cp = *cp;
  free(s->cx); free(s->cv); free(s->com); free(s->crad);
  s->cx = (double*)malloc(sizeof(double) * (size_t)(nc * d + 1));
  s->cv = (double*)malloc(sizeof(double) * (size_t)(nc * d + 1));
  s->com = (double*)malloc(sizeof(double) * (size_t)(nc * 3 + 1));
  s->crad = (double*)malloc(sizeof(double) * (size_t)(nc + 1));
  memcpy(s->cx, x, sizeof(double) * (size_t)(nc * d));
  memcpy(s->cv, v, sizeof(double) * (size_t)(nc * d));
  memcpy(s->com, omega, sizeof(double) * (size_t)(nc * 3));
  memcpy(s->crad, radius, sizeof(double) * (size_t)nc);
  return 0;
}

/* The boundary-particle kinematics around MCF's colloid integration
 * (marching_integrate_VV.F90:455-765): particles_compute_colloid_relative_
 * position.F90 takes each boundary particle relative to its colloid's
 * nearest centre image and turns it by the colloid's rotation matrix of the
 * step (MATMUL(R, rx), R(i,j) = rot[9c + i + 3j]); after the colloids have
 * moved, particles_compute_colloid_absolute_position.F90 adds the new
 * centre.  Then the colloid state is (x_new, v, omega).  Nothing moves
 * unless the colloids translate or rotate. */
int orc_move_colloids(orc_state* s, const double* x_new, const double* rot, const double* v,
                      const double* omega) {
  const int d = s->d, nc = s->cp.num_colloid;
  if (s->cp.translate || s->cp.rotate) {
    for (int64_t j = 0; j < s->nreal; ++j) {
      const int c = s->sid[j] - 1;
      if (s->sid[j] <= 0 || c >= nc) continue;
      double ximg[3], rx[3] = {0, 0, 0}, vimg[3], rb[3] = {0, 0, 0};
      colloid_nearest_image(s, &s->x[j * d], c, ximg, rx, vimg);
      if (s->cp.rotate && rot) {
        for (int a = 0; a < d; ++a) {
          double t = 0.0;
          for (int q = 0; q < d; ++q) t = t + rot[c * 9 + a + 3 * q] * rx[q];
          rb[a] = t;
        }
      } else {
        for (int a = 0; a < d; ++a) rb[a] = rx[a];
      }
      for (int a = 0; a < d; ++a) s->x[j * d + a] = rb[a] + x_new[c * d + a];
    }
  }
  memcpy(s->cx, x_new, sizeof(double) * (size_t)(nc * d));
  memcpy(s->cv, v, sizeof(double) * (size_t)(nc * d));
  memcpy(s->com, omega, sizeof(double) * (size_t)(nc * 3));
  s->have_list = s->have_density = s->have_pressure = 0;
  return 0;
}

/* particles_collect_colloid_interaction.F90:93-136 */
int orc_colloid_drag(orc_state* s, double* drag, double* torque) {
  const int d = s->d, nc = s->cp.num_colloid;
  for (int k = 0; k < nc * d; ++k) drag[k] = 0.0;
  for (int k = 0; k < nc * 3; ++k) torque[k] = 0.0;
  for (int64_t j = 0; j < s->nreal; ++j) {
    const int c = s->sid[j] - 1;
    if (s->sid[j] <= 0 || c >= nc) continue;
    double F[3] = {0, 0, 0};
    for (int a = 0; a < d; ++a) F[a] = s->f[j * d + a] * s->m[j];
    for (int a = 0; a < d; ++a) drag[c * d + a] = drag[c * d + a] + F[a];
    double ximg[3], rx[3] = {0, 0, 0}, vimg[3], T[3];
    colloid_nearest_image(s, &s->x[j * d], c, ximg, rx, vimg);
    cross3(rx, F, T);
    for (int a = 0; a < 3; ++a) torque[c * 3 + a] = torque[c * 3 + a] + T[a];
  }
  return 0;
}

/* colloid_compute_repulsion_cc.F90:95-164, nearest periodic image */
int orc_colloid_repulsion(orc_state* s, double* force) {
  const int d = s->d, nc = s->cp.num_colloid;
  for (int k = 0; k < nc * d; ++k) force[k] = 0.0;
  if (s->cp.cc_repul_type < 1) return 0;
  const double hn = s->cp.cc_repul_cut_off, hm = s->cp.cc_repul_cut_on, F0 = s->cp.cc_repul_F0;
  for (int i = 0; i < nc; ++i)
    for (int j = i + 1; j < nc; ++j) {
      double R12[3] = {0, 0, 0}, rr = 0.0;
      for (int a = 0; a < d; ++a) {
        double r = s->cx[i * d + a] - s->cx[j * d + a];
        if (s->periodic[a]) {
          if (r > 0.5 * s->len[a]) r -= s->len[a];
          else if (r < -0.5 * s->len[a]) r += s->len[a];
        }
        R12[a] = r;
        rr += r * r;
      }
      const double r = sqrt(rr);
      double h = r - (s->crad[i] + s->crad[j]);
      if (!(h < 5.0 * hn)) continue;
      double F = 0.0;
      if (s->cp.cc_repul_type == 1) {
        if (h < hn) {
          if (h < hm) h = hm;
          F = F0 - F0 * h / hn;
        }
      } else {
        if (h < hm) h = hm;
        F = F0 / hn * exp(-h / hn) / (1.0 - exp(-h / hn)) -
            F0 / hn * exp(-5.0) / (1.0 - exp(-5.0));
      }
      /* R12 / r first, then F times it (colloid_compute_repulsion_cc.F90:
       * 155-156); F_p(i) += F_ij, F_p(j) -= F_ij
       * (colloid_compute_interaction.F90), so each colloid's sum runs over
       * its partners in index order */
      for (int a = 0; a < d; ++a) {
        const double fij = F * (R12[a] / r);
        force[i * d + a] = force[i * d + a] + fij;
        force[j * d + a] = force[j * d + a] - fij;
      }
    }
  return 0;
}

/* ------------------------------------------------------------------------
 * Rigid-body dynamics of the colloids, marching_integrate_VV.F90:455-765
 * (explicit integrate_colloid_type 1-2) and the initial accelerations of
 * marching_marching.F90:995-1110.
 * ---------------------------------------------------------------------- */

/* Adams-Bashforth order of a step (the Colloid routines' "IF (step < itype)
 * order = step ELSE order = itype") */
static int ab_order(int64_t step, int itype) { return step < itype ? (int)step : itype; }

/* Adams-Bashforth increment over the history h (level k at h[k * stride]),
 * in the operation order of colloid_integrate_translate_position.F90,
 * colloid_integrate_translate_velocity.F90, colloid_integrate_rotate_
 * velocity.F90 and colloid_compute_rotation_vector.F90 (coefficients
 * times levels, left to right, times dt, over the divisor) */
static double ab_incr(int order, const double* h, size_t st, double dt) {
  switch (order) {
    case 1:
      return h[0] * dt;
    case 2:
      return (3.0 * h[0] - h[st]) * dt / 2.0;
    case 3:
      return (23.0 * h[0] - 16.0 * h[st] + 5.0 * h[2 * st]) * dt / 12.0;
    case 4:
      return (55.0 * h[0] - 59.0 * h[st] + 37.0 * h[2 * st] - 9.0 * h[3 * st]) * dt / 24.0;
    default:
      return (1901.0 * h[0] - 2774.0 * h[st] + 2616.0 * h[2 * st] - 1274.0 * h[3 * st] +
              251.0 * h[4 * st]) *
             dt / 720.0;
  }
}

/* "i = itype; DO WHILE (i >= 2): h(:,:,i) = h(:,:,i-1)" of the history of
 * n values per level */
static void ab_shift(double* h, size_t n, int itype) {
  for (int k = itype - 1; k >= 1; --k) memcpy(h + (size_t)k * n, h + (size_t)(k - 1) * n,
                                               sizeof(double) * n);
}

/* tool_rotation_matrix.F90: rotation by phi about the unit axis ax,
 * rm(i,j) at rm[i + 3j] */
static void rotation_matrix(const double* ax, double phi, double* rm) {
  const double cp = cos(phi), cp1 = 1.0 - cp, sp = sin(phi);
  rm[0 + 3 * 0] = ax[0] * ax[0] * cp1 + cp;
  rm[0 + 3 * 1] = ax[0] * ax[1] * cp1 - ax[2] * sp;
  rm[0 + 3 * 2] = ax[0] * ax[2] * cp1 + ax[1] * sp;
  rm[1 + 3 * 0] = ax[1] * ax[0] * cp1 + ax[2] * sp;
  rm[1 + 3 * 1] = ax[1] * ax[1] * cp1 + cp;
  rm[1 + 3 * 2] = ax[1] * ax[2] * cp1 - ax[0] * sp;
  rm[2 + 3 * 0] = ax[2] * ax[0] * cp1 - ax[1] * sp;
  rm[2 + 3 * 1] = ax[2] * ax[1] * cp1 + ax[0] * sp;
  rm[2 + 3 * 2] = ax[2] * ax[2] * cp1 + cp;
}

int orc_set_colloid_dynamics(orc_state* s, const mcfg_colloid_dynamics* cd, const double* mass,
                             const double* mmi, const double* v_hist, const double* omega_hist,
                             const double* f_hist, const double* alpha_hist,
                             const double* acc_matrix, const double* theta) {
  const int d = s->d, nc = s->cp.num_colloid;
  if (!cd || cd->integrate_AB < 1 || cd->integrate_AB > 5 || cd->sub_time_step < 1 || !mass ||
      !mmi || (cd->body_force_type != 0 && cd->body_force_type != 1))
    return fail(s, "bad colloid dynamics");
  const int AB = cd->integrate_AB;
  s->cd = *cd;
  double** arrs[] = {&s->cm, &s->cmmi, &s->cvh, &s->comh, &s->cfh, &s->calh,
                     &s->crot, &s->cacc, &s->ctheta, &s->cdrag, &s->ctorque};
  const size_t sizes[] = {(size_t)nc, (size_t)nc * 3, (size_t)nc * d * AB, (size_t)nc * 3 * AB,
                          (size_t)nc * d * AB, (size_t)nc * 3 * AB, (size_t)nc * 9,
                          (size_t)nc * 9, (size_t)nc * 3, (size_t)nc * d, (size_t)nc * 3};
  for (int q = 0; q < 11; ++q) {
    free(*arrs[q]);
    *arrs[q] = (double*)calloc(sizes[q] + 1, sizeof(double));
  }
  memcpy(s->cm, mass, sizeof(double) * (size_t)nc);
  memcpy(s->cmmi, mmi, sizeof(double) * (size_t)nc * 3);
  if (v_hist) memcpy(s->cvh, v_hist, sizeof(double) * sizes[2]);
  else memcpy(s->cvh, s->cv, sizeof(double) * (size_t)nc * d);
  if (omega_hist) memcpy(s->comh, omega_hist, sizeof(double) * sizes[3]);
  else memcpy(s->comh, s->com, sizeof(double) * (size_t)nc * 3);
  if (f_hist) memcpy(s->cfh, f_hist, sizeof(double) * sizes[4]);
  if (alpha_hist) memcpy(s->calh, alpha_hist, sizeof(double) * sizes[5]);
  for (int c = 0; c < nc; ++c)
    for (int q = 0; q < 9; ++q) s->crot[c * 9 + q] = (q % 4 == 0) ? 1.0 : 0.0;
  if (acc_matrix) memcpy(s->cacc, acc_matrix, sizeof(double) * (size_t)nc * 9);
  else memcpy(s->cacc, s->crot, sizeof(double) * (size_t)nc * 9);
  if (theta) memcpy(s->ctheta, theta, sizeof(double) * (size_t)nc * 3);
  /* level 1 of the histories is the colloids' current velocity */
  memcpy(s->cv, s->cvh, sizeof(double) * (size_t)nc * d);
  memcpy(s->com, s->comh, sizeof(double) * (size_t)nc * 3);
  s->cdyn = 1;
  return 0;
}

/* colloid_compute_interaction.F90 (repulsion only; no lubrication, no
 * walls) + colloid_apply_body_force.F90 + colloid_compute_translate_
 * acceleration.F90, from the fluid's drag and torque */
static void colloid_translate_accel(orc_state* s, const double* fdrag, const double* ftorque) {
  const int d = s->d, nc = s->cp.num_colloid, AB = s->cd.integrate_AB;
  double* rep = (double*)calloc((size_t)nc * d + 1, sizeof(double));
  orc_colloid_repulsion(s, rep);
  for (int q = 0; q < nc * d; ++q) s->cdrag[q] = fdrag[q] + rep[q];
  for (int q = 0; q < nc * 3; ++q) s->ctorque[q] = ftorque[q];
  free(rep);
  if (s->cd.body_force_type == 1)
    for (int a = 0; a < d; ++a)
      for (int c = 0; c < nc; ++c)
        s->cdrag[c * d + a] = s->cdrag[c * d + a] + s->cd.body_force[a] * s->cm[c];
  ab_shift(s->cfh, (size_t)nc * d, AB);
  for (int a = 0; a < d; ++a)
    for (int c = 0; c < nc; ++c)
      s->cfh[c * d + a] = s->cp.translate ? s->cdrag[c * d + a] / s->cm[c] : 0.0;
}

/* colloid_compute_rotate_acceleration.F90 (spheres in 3D, disks in 2D) */
static void colloid_rotate_accel(orc_state* s) {
  const int nc = s->cp.num_colloid, AB = s->cd.integrate_AB;
  ab_shift(s->calh, (size_t)nc * 3, AB);
  if (s->cp.rotate) {
    for (int c = 0; c < nc; ++c) {
      if (s->d == 2) {
        s->calh[c * 3 + 2] = s->ctorque[c * 3 + 2] / s->cmmi[c * 3 + 2];
      } else {
        for (int a = 0; a < 3; ++a) s->calh[c * 3 + a] = s->ctorque[c * 3 + a] / s->cmmi[c * 3 + a];
      }
    }
  } else {
    for (int q = 0; q < nc * 3; ++q) s->calh[q] = 0.0;
  }
}

/* colloid_adjust_colloid.F90: periodic faces wrap the centre back by whole
 * box lengths; a solid wall face puts it one radius inside (and stops that
 * velocity component) */
static void colloid_adjust(orc_state* s) {
  const int d = s->d, nc = s->cp.num_colloid;
  for (int c = 0; c < nc; ++c)
    for (int a = 0; a < d; ++a) {
      double* x = &s->cx[c * d + a];
      const double lo = s->p.min_phys[a], hi = s->p.max_phys[a], L = hi - lo;
      if (*x < lo) {
        if (s->p.bcdef[2 * a] == MCFG_BC_PERIODIC) {
          const int nover = (int)((hi - *x) / L);
          *x = *x + L * (double)nover;
        } else if (s->p.bcdef[2 * a] == MCFG_BC_WALL_SOLID) {
          *x = lo + s->crad[c];
          s->cvh[c * d + a] = 0.0;
        }
      }
      if (*x >= hi) {
        if (s->p.bcdef[2 * a + 1] == MCFG_BC_PERIODIC) {
          const int nover = (int)((*x - lo) / L);
          *x = *x - L * (double)nover;
        } else if (s->p.bcdef[2 * a + 1] == MCFG_BC_WALL_SOLID) {
          *x = hi - s->crad[c] - s->machine_zero;
          s->cvh[c * d + a] = 0.0;
        }
      }
    }
}

/* marching_marching.F90:995-1110: after the first right-hand side, the
 * fluid's drag and torque, repulsion, body force and both accelerations */
static int colloid_initial_accel(orc_state* s) {
  const int d = s->d, nc = s->cp.num_colloid;
  double* dr = (double*)calloc((size_t)nc * d + 1, sizeof(double));
  double* tq = (double*)calloc((size_t)nc * 3 + 1, sizeof(double));
  orc_colloid_drag(s, dr, tq);
  colloid_translate_accel(s, dr, tq);
  colloid_rotate_accel(s);
  free(dr);
  free(tq);
  return 0;
}

/* The colloid part of a VV step, marching_integrate_VV.F90:455-765 */
int orc_colloid_integrate(orc_state* s, int64_t step, double dt) {
  if (!s->cdyn) return fail(s, "orc_set_colloid_dynamics must come first");
  const int d = s->d, nc = s->cp.num_colloid, AB = s->cd.integrate_AB;
  if (nc == 0) return 0;
  double* dr = (double*)calloc((size_t)nc * d + 1, sizeof(double));
  double* tq = (double*)calloc((size_t)nc * 3 + 1, sizeof(double));
  orc_colloid_drag(s, dr, tq); /* particles_collect_colloid_interaction */
  if (s->cp.translate || s->cp.rotate) {
    const int nsub = s->cd.sub_time_step;
    const double dts = dt / (double)nsub;
    for (int i = 1; i <= nsub; ++i) {
      const int oa = ab_order(step - 1 + i - s->cd.step_start, AB);
      /* colloid_integrate_rotate_velocity is called with step-1+i+step_start */
      const int orr = ab_order(step - 1 + i + s->cd.step_start, AB);
      if (oa < 1 || orr < 1) {
        free(dr);
        free(tq);
        return fail(s, "colloid integration before the first step");
      }
      if (s->cp.rotate) {
        for (int c = 0; c < nc; ++c) {
          double ax[3], phi;
          for (int a = 0; a < 3; ++a) ax[a] = ab_incr(oa, &s->comh[c * 3 + a], (size_t)nc * 3, dts);
          phi = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
          if (phi < s->machine_zero) {
            phi = 0.0;
            ax[0] = 1.0;
            ax[1] = ax[2] = 0.0;
          } else {
            for (int a = 0; a < 3; ++a) ax[a] = ax[a] / phi;
          }
          s->ctheta[c * 3 + 2] = s->ctheta[c * 3 + 2] + phi;
          rotation_matrix(ax, phi, &s->crot[c * 9]);
          double acc[9];
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
              double t = 0.0;
              for (int q = 0; q < 3; ++q) t = t + s->crot[c * 9 + a + 3 * q] * s->cacc[c * 9 + q + 3 * b];
              acc[a + 3 * b] = t;
            }
          memcpy(&s->cacc[c * 9], acc, sizeof acc);
        }
      }
      /* particles_compute_colloid_relative_position: boundary particles
       * relative to the nearest centre image, turned by the rotation */
      for (int64_t j = 0; j < s->nreal; ++j) {
        const int c = s->sid[j] - 1;
        if (s->sid[j] <= 0 || c >= nc) continue;
        double ximg[3], rx[3] = {0, 0, 0}, vimg[3];
        colloid_nearest_image(s, &s->x[j * d], c, ximg, rx, vimg);
        if (s->cp.rotate) {
          for (int a = 0; a < d; ++a) {
            double t = 0.0;
            for (int q = 0; q < d; ++q) t = t + s->crot[c * 9 + a + 3 * q] * rx[q];
            s->x[j * d + a] = t;
          }
        } else {
          for (int a = 0; a < d; ++a) s->x[j * d + a] = rx[a];
        }
      }
      if (s->cp.rotate) {
        ab_shift(s->comh, (size_t)nc * 3, AB);
        for (int q = 0; q < nc * 3; ++q)
          s->comh[q] = s->comh[q] + ab_incr(orr, &s->calh[q], (size_t)nc * 3, dts);
      }
      if (s->cp.translate) {
        for (int q = 0; q < nc * d; ++q)
          s->cx[q] = s->cx[q] + ab_incr(oa, &s->cvh[q], (size_t)nc * d, dts);
        ab_shift(s->cvh, (size_t)nc * d, AB);
        for (int q = 0; q < nc * d; ++q)
          s->cvh[q] = s->cvh[q] + ab_incr(oa, &s->cfh[q], (size_t)nc * d, dts);
      }
      colloid_translate_accel(s, dr, tq);
      colloid_adjust(s);
      colloid_rotate_accel(s);
      /* particles_compute_colloid_absolute_position */
      for (int64_t j = 0; j < s->nreal; ++j) {
        const int c = s->sid[j] - 1;
        if (s->sid[j] <= 0 || c >= nc) continue;
        for (int a = 0; a < d; ++a) s->x[j * d + a] = s->x[j * d + a] + s->cx[c * d + a];
      }
      memcpy(s->cv, s->cvh, sizeof(double) * (size_t)nc * d);
      memcpy(s->com, s->comh, sizeof(double) * (size_t)nc * 3);
    }
  }
  free(dr);
  free(tq);
  s->have_list = s->have_density = s->have_pressure = 0;
  return 0;
}

int orc_get_colloid_state(const orc_state* s, double* x, double* v_hist, double* omega_hist,
                          double* f_hist, double* alpha_hist, double* drag, double* torque,
                          double* rot, double* acc, double* theta) {
  const int d = s->d, nc = s->cp.num_colloid, AB = s->cd.integrate_AB;
  if (x) memcpy(x, s->cx, sizeof(double) * (size_t)nc * d);
  if (!s->cdyn) return 0;
  if (v_hist) memcpy(v_hist, s->cvh, sizeof(double) * (size_t)nc * d * AB);
  if (omega_hist) memcpy(omega_hist, s->comh, sizeof(double) * (size_t)nc * 3 * AB);
  if (f_hist) memcpy(f_hist, s->cfh, sizeof(double) * (size_t)nc * d * AB);
  if (alpha_hist) memcpy(alpha_hist, s->calh, sizeof(double) * (size_t)nc * 3 * AB);
  if (drag) memcpy(drag, s->cdrag, sizeof(double) * (size_t)nc * d);
  if (torque) memcpy(torque, s->ctorque, sizeof(double) * (size_t)nc * 3);
  if (rot) memcpy(rot, s->crot, sizeof(double) * (size_t)nc * 9);
  if (acc) memcpy(acc, s->cacc, sizeof(double) * (size_t)nc * 9);
  if (theta) memcpy(theta, s->ctheta, sizeof(double) * (size_t)nc * 3);
  return 0;
}

static void density_pair(orc_state* s, int64_t ip, int64_t jp, void* ctx) {
  (void)ctx;
  const int d = s->d;
  const int32_t si = s->sid[ip], sj = s->sid[jp];
  if (!s->p.symmetry && !dyn_rho(s, si)) return;
  if (si != 0 && sj != 0 && !dyn_rho(s, si) && !dyn_rho(s, sj)) return;
  double dij = 0.0;
  for (int a = 0; a < d; ++a) {
    const double r = s->x[ip * d + a] - s->x[jp * d + a];
    dij = dij + r * r;
  }
  if (dij >= s->cut_off2) return;
  dij = sqrt(dij);
  const double w = kernel_eval(s, dij, NULL);
  double rhoi, rhoj;
  if (s->p.rhs_density_type == 1) {
    rhoi = w * s->m[jp];
    rhoj = w * s->m[ip];
  } else {
    rhoi = w;
    rhoj = w;
  }
  if (dyn_rho(s, si)) s->rho[ip] = s->rho[ip] + rhoi;
  if (s->p.symmetry && dyn_rho(s, sj)) s->rho[jp] = s->rho[jp] + rhoj;
}

int orc_compute_density(orc_state* s) {
  if (!s->have_list) return fail(s, "orc_compute_density: build the list first");
  const double t0 = now_s();
  const double w0 = kernel_eval(s, 0.0, NULL);
  for (int64_t j = 0; j < s->nall; ++j) s->rho[j] = 0.0;
  for (int64_t j = 0; j < s->nreal; ++j) {
    const int32_t sid = s->sid[j];
    if (sid == 0 || dyn_rho(s, sid)) {
      s->rho[j] = (s->p.rhs_density_type == 1) ? w0 * s->m[j] : w0;
    } else {
      if (s->m[j] < s->machine_zero) return fail(s, "orc_compute_density: zero mass");
      s->rho[j] = (s->p.rhs_density_type == 1) ? s->p.init_density
                                                 : s->p.init_density / s->m[j];
    }
  }
  for_all_pairs(s, density_pair, NULL);
  if (s->p.symmetry)
    for (int64_t g = s->nreal; g < s->nall; ++g) {
      const int64_t o = s->owner[g];
      if (dyn_rho(s, s->sid[o])) s->rho[o] = s->rho[o] + s->rho[g];
    }
  if (s->cp.num_colloid > 0) /* marching_integrate_VV.F90:1074 */
    for (int64_t j = 0; j < s->nreal; ++j)
      if (s->sid[j] > 0) colloid_particle_velocity(s, &s->x[j * s->d], s->sid[j] - 1, &s->v[j * s->d]);
  ghost_refresh(s);
  s->have_density = 1;
  s->timers[1] += now_s() - t0;
  return 0;
}

/* the second ghost get of marching_integrate_VV.F90:1128 for a subdomain:
 * densities of the real particles from the caller, then the periodic ghost
 * copies refreshed from them */
int orc_update_density(orc_state* s, const double* rho) {
  if (!s->have_density) return fail(s, "orc_update_density: no density");
  memcpy(s->rho, rho, sizeof(double) * (size_t)s->nreal);
  ghost_refresh(s);
  s->have_pressure = 0;
  return 0;
}

/* ------------------------------------------------------------------------
 * Pressure: particles_compute_pressure.F90:66-95 ->
 * stateEquation_compute_pressure.F90:147-180 (vector forms).
 * ---------------------------------------------------------------------- */
int orc_compute_pressure(orc_state* s) {
  if (!s->have_density) return fail(s, "orc_compute_pressure: no density");
  const double t0 = now_s();
  for (int64_t j = 0; j < s->nall; ++j) {
    const double r = (s->p.rhs_density_type == 1) ? s->rho[j] : s->rho[j] * s->m[j];
    if (s->p.stateEquation_type == 1)
      s->pr[j] = (s->p.c * s->p.c) * (pow(r, s->p.gamma) - s->p.rho_ref);
    else
      s->pr[j] = s->p0 * (pow(r / s->p.rho_ref, s->p.gamma) - 1.0);
  }
  s->have_pressure = 1;
  s->timers[2] += now_s() - t0;
  return 0;
}

/* ------------------------------------------------------------------------
 * Pair forces: rhs_force_ff_Newtonian_{Morris,Espanol,HuAdams,
 * HuAdams_angular}.F90; accelerations (force per unit mass).
 * ---------------------------------------------------------------------- */
typedef struct {
  int64_t step;
  int noise;
  double sqdt;
} force_ctx;

static void noise_matrix(const orc_state* s, const float* z, double dW[3][3],
                         double* trace_out) {
  const int d = s->d;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) dW[a][b] = 0.0;
  double trace = 0.0;
  for (int a = 0; a < d; ++a) {
    dW[a][a] = (double)z[a];
    trace = trace + dW[a][a];
  }
  trace = trace / d;
  if (d == 3) {
    dW[0][1] = dW[1][0] = (double)z[3] * 0.70710678118654752440;
    dW[0][2] = dW[2][0] = (double)z[4] * 0.70710678118654752440;
    dW[1][2] = dW[2][1] = (double)z[5] * 0.70710678118654752440;
  } else {
    dW[0][1] = dW[1][0] = (double)z[2] * 0.70710678118654752440;
  }
  *trace_out = trace;
  for (int a = 0; a < d; ++a) dW[a][a] = dW[a][a] - trace;
}

/* We = dW e of the Hu-Adams random force (rhs_force_ff_Newtonian_HuAdams.F90:
 * 176-239): MCF uses its symmetric traceless dW only through this vector, a
 * Gaussian with variance 1 - 1/d along e and 1/2 across e, so it is drawn
 * directly, We = s (ca (e.g) e + cb (g - (e.g) e)), ca = sqrt(1 - 1/d),
 * cb = sqrt(1/2), from the first d normals g of the pair's stream and
 * s = +1 if pid_i < pid_j else -1 (the pair's two sides get opposite We). */
static void pair_we(const orc_state* s, int64_t step, int32_t pidi, int32_t pidj,
                    const double* e, double* We) {
  const int d = s->d;
  float z[6];
  orc_pair_normals(s->p.seed, step, pidi, pidj, d, z);
  const double cb = 0.70710678118654752440;
  const double ca = (d == 3) ? 0.81649658092772603273 : cb;
  const double sg = (pidi < pidj) ? 1.0 : -1.0;
  double eg = 0.0;
  for (int a = 0; a < d; ++a) eg = eg + e[a] * (double)z[a];
  for (int a = 0; a < d; ++a)
    We[a] = sg * ((ca - cb) * eg * e[a] + cb * (double)z[a]);
}

int orc_pair_we(const orc_state* s, int64_t step, int32_t pidi, int32_t pidj, const double* e,
                double* We) {
  pair_we(s, step, pidi, pidj, e, We);
  return 0;
}

static void rhs_force_ff(orc_state* s, const force_ctx* fc, const double* xi,
                         const double* xj, double dij, const double* vi,
                         const double* vj, double numi, double numj, double pi,
                         double pj, double mi, double mj, double gradw,
                         int32_t pidi, int32_t pidj, double* fi, double* fj) {
  const int d = s->d;
  double eij[3], vij[3];
  for (int a = 0; a < d; ++a) {
    fi[a] = 0.0;
    fj[a] = 0.0;
    eij[a] = (xi[a] - xj[a]) / dij;
    vij[a] = vi[a] - vj[a];
  }
  const double eta = s->p.eta, kt = s->p.kt;
  const int brown = fc->noise;
  switch (s->p.rhs_force_type) {
    case 1: { /* Morris, rhs_force_ff_Newtonian_Morris.F90:89-133 */
      const double f_c = (pi / (numi * numi) + pj / (numj * numj)) * gradw;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] - mj * f_c * eij[a];
        fj[a] = fj[a] + mi * f_c * eij[a];
      }
      const double f_d = 2.0 * eta * gradw / numi / numj / dij;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] + mj * f_d * vij[a];
        fj[a] = fj[a] - mi * f_d * vij[a];
      }
      break;
    }
    case 2: { /* Espanol-Revenga, rhs_force_ff_Newtonian_Espanol.F90:130-247 */
      double ev = 0.0;
      for (int a = 0; a < d; ++a) ev = ev + eij[a] * vij[a];
      const double f_c = (pi / (numi * numi) + pj / (numj * numj)) * gradw;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] - f_c * eij[a] / mi;
        fj[a] = fj[a] + f_c * eij[a] / mj;
      }
      const double f_d1 = (2.0 - 1.0 / d) * eta * gradw / numi / numj / dij;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] + f_d1 * vij[a] / mi;
        fj[a] = fj[a] - f_d1 * vij[a] / mj;
      }
      const double f_d2 = eta * (d + 2) / d * gradw * ev / numi / numj / dij;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] + f_d2 * eij[a] / mi;
        fj[a] = fj[a] - f_d2 * eij[a] / mj;
      }
      if (brown) {
        float z[6];
        double dW[3][3], trace;
        orc_pair_normals(s->p.seed, fc->step, pidi, pidj, d, z);
        noise_matrix(s, z, dW, &trace);
        const double Zij = 4.0 * kt * gradw / dij / numi / numj;
        const double aa = 5.0 * eta / 3.0;
        const double bb = ((double)d + 2.0) * eta / 3.0;
        const double Aij = sqrt(-Zij * aa);
        const double Bij = sqrt(-Zij * (double)d / 2.0 * (bb + aa * (2.0 / (double)d - 1.0)));
        for (int a = 0; a < d; ++a) {
          double We = 0.0;
          for (int b = 0; b < d; ++b) We = We + dW[a][b] * eij[b];
          const double fr = (Aij * We + Bij * trace * eij[a]) / fc->sqdt;
          fi[a] = fi[a] + fr / mi;
          fj[a] = fj[a] - fr / mj;
        }
      }
      break;
    }
    case 3: { /* Hu-Adams, rhs_force_ff_Newtonian_HuAdams.F90:124-237 */
      const double f_c = (pi / (numi * numi) + pj / (numj * numj)) * gradw;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] - f_c * eij[a] / mi;
        fj[a] = fj[a] + f_c * eij[a] / mj;
      }
      const double f_d = eta * (1.0 / (numi * numi) + 1.0 / (numj * numj)) * gradw / dij;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] + f_d * vij[a] / mi;
        fj[a] = fj[a] - f_d * vij[a] / mj;
      }
      if (brown) {
        double We[3];
        pair_we(s, fc->step, pidi, pidj, eij, We);
        const double f_r = sqrt(-4.0 * kt * f_d) / fc->sqdt;
        for (int a = 0; a < d; ++a) {
          fi[a] = fi[a] + f_r * We[a] / mi;
          fj[a] = fj[a] - f_r * We[a] / mj;
        }
      }
      break;
    }
    case 4: { /* Hu-Adams angular, ..._HuAdams_angular.F90:152-229 */
      double ev = 0.0;
      for (int a = 0; a < d; ++a) ev = ev + eij[a] * vij[a];
      const double pij = (pi + pj) / 2.0;
      const double Aij = (1.0 / (numi * numi) + 1.0 / (numj * numj)) * gradw;
      const double f_c = Aij * pij;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] - f_c * eij[a] / mi;
        fj[a] = fj[a] + f_c * eij[a] / mj;
      }
      const double f_d = s->p.eta_coef * eta * Aij * ev / dij;
      for (int a = 0; a < d; ++a) {
        fi[a] = fi[a] + f_d * eij[a] / mi;
        fj[a] = fj[a] - f_d * eij[a] / mj;
      }
      if (brown) {
        float z[6];
        orc_pair_normals(s->p.seed, fc->step, pidi, pidj, d, z);
        const double eps = (double)z[0];
        const double f_r = eps * sqrt(2.0 * kt * eta) * sqrt(-s->p.eta_coef * Aij / dij) / fc->sqdt;
        for (int a = 0; a < d; ++a) {
          fi[a] = fi[a] + f_r * eij[a] / mi;
          fj[a] = fj[a] - f_r * eij[a] / mj;
        }
      }
      break;
    }
  }
}

/* Morris no-slip velocity of a wall particle,
 * boundary_noslip_solid.F90:40-95,137-240; wall sid = -face (1..2d). */
static void wall_noslip(const orc_state* s, const double* xf, const double* xw,
                        const double* vf, double* vw, int32_t sid_w) {
  const int d = s->d;
  const int index_w = sid_w < 0 ? -sid_w : sid_w;
  const double* sv = s->shear_v[index_w - 1];
  if (s->p.wall_noslip_type <= 1) {
    for (int a = 0; a < d; ++a) vw[a] = sv[a];
    return;
  }
  int index;
  double x_sur;
  if (index_w % 2 == 1) {
    index = (index_w + 1) / 2 - 1;
    x_sur = s->p.min_phys[index];
  } else {
    index = index_w / 2 - 1;
    x_sur = s->p.max_phys[index];
  }
  double f_sur = xf[index] - x_sur;
  double w_sur = xw[index] - x_sur;
  if (f_sur * w_sur >= 0.0) {
    for (int a = 0; a < d; ++a) vw[a] = sv[a];
  } else {
    f_sur = fabs(f_sur);
    w_sur = fabs(w_sur);
    double corr = w_sur / f_sur;
    if (corr > 0.5) corr = 0.5; /* mcf_wall_dist_ratio, mcf_header.F90:282 */
    for (int a = 0; a < d; ++a) vw[a] = -corr * (vf[a] - sv[a]) + sv[a];
  }
}

/* particles_compute_pressure_tensor.F90:88-133: pt(i,j) = -G ct(i,j) +
 * delta_ij (p + G), G = n_p kt_p; pt[i + d*j] */
static void pressure_tensor(const orc_state* s, int64_t k, double* pt) {
  const int d = s->d;
  const double G = s->p.n_p * s->p.kt_p;
  for (int j = 0; j < d; ++j)
    for (int i = 0; i < d; ++i) {
      pt[i + d * j] = -G * s->ct[k * d * d + i + d * j];
      if (i == j) pt[i + d * j] = pt[i + d * j] + s->pr[k] + G;
    }
}

/* rhs_force_ff_non_Newtonian_HuAdams.F90:95-201 */
static void rhs_force_nn(orc_state* s, const force_ctx* fc, const double* xi, const double* xj,
                         double dij, const double* vi, const double* vj, double numi,
                         double numj, const double* pti, const double* ptj, double mi, double mj,
                         double gradw, int32_t pidi, int32_t pidj, double* fi, double* fj) {
  const int d = s->d;
  double eij[3], vij[3], f_c[3];
  for (int a = 0; a < d; ++a) {
    fi[a] = 0.0;
    fj[a] = 0.0;
    eij[a] = (xi[a] - xj[a]) / dij;
    vij[a] = vi[a] - vj[a];
    f_c[a] = 0.0;
  }
  for (int j = 0; j < d; ++j)
    for (int i = 0; i < d; ++i)
      f_c[j] = f_c[j] + pti[i + d * j] * eij[i] / (numi * numi) +
               ptj[i + d * j] * eij[i] / (numj * numj);
  for (int a = 0; a < d; ++a) {
    fi[a] = fi[a] - f_c[a] * gradw / mi;
    fj[a] = fj[a] + f_c[a] * gradw / mj;
  }
  const double f_d = s->p.eta * (1.0 / (numi * numi) + 1.0 / (numj * numj)) * gradw / dij;
  for (int a = 0; a < d; ++a) {
    fi[a] = fi[a] + f_d * vij[a] / mi;
    fj[a] = fj[a] - f_d * vij[a] / mj;
  }
  if (fc->noise) {
    double We[3];
    pair_we(s, fc->step, pidi, pidj, eij, We);
    const double f_r = sqrt(-4.0 * s->p.kt * f_d) / fc->sqdt;
    for (int a = 0; a < d; ++a) {
      fi[a] = fi[a] + f_r * We[a] / mi;
      fj[a] = fj[a] - f_r * We[a] / mj;
    }
  }
}

static void force_pair(orc_state* s, int64_t ip, int64_t jp, void* ctx) {
  const force_ctx* fc = (const force_ctx*)ctx;
  const int d = s->d;
  const int32_t si = s->sid[ip], sj = s->sid[jp];
  if (si < 0 && sj < 0) return; /* w-w: no interaction */
  if (si > 0 && sj > 0 && (si == sj || !s->cp.pp_interact_cc)) return; /* c-c */
  if ((si > 0 && sj < 0) || (si < 0 && sj > 0)) return; /* c-w off */
  double rij[3];
  double dij = 0.0;
  for (int a = 0; a < d; ++a) {
    rij[a] = s->x[ip * d + a] - s->x[jp * d + a];
    dij = dij + rij[a] * rij[a];
  }
  if (dij >= s->cut_off2) return; /* pp_interaction.inc:37-50 */
  dij = sqrt(dij);
  double gradw;
  kernel_eval(s, dij, &gradw);
  double vi[3], vj[3];
  for (int a = 0; a < d; ++a) {
    vi[a] = s->v[ip * d + a];
    vj[a] = s->v[jp * d + a];
  }
  double pi = s->pr[ip], pj = s->pr[jp];
  if (si == 0 && sj < 0) { /* pp_interaction_fw.inc */
    wall_noslip(s, &s->x[ip * d], &s->x[jp * d], vi, vj, sj);
    pj = pi;
  } else if (si < 0 && sj == 0) { /* pp_interaction_wf.inc */
    wall_noslip(s, &s->x[jp * d], &s->x[ip * d], vj, vi, si);
    pi = pj;
  } else if (si == 0 && sj > 0) { /* pp_interaction_fc.inc */
    if (s->cp.noslip_type == 2) colloid_noslip(s, &s->x[ip * d], &s->x[jp * d], vi, sj - 1, vj);
    pj = pi;
  } else if (si > 0 && sj == 0) { /* pp_interaction_cf.inc */
    if (s->cp.noslip_type == 2) colloid_noslip(s, &s->x[jp * d], &s->x[ip * d], vj, si - 1, vi);
    pi = pj;
  }
  double fi[3], fj[3];
  if (s->p.Newtonian) {
    rhs_force_ff(s, fc, &s->x[ip * d], &s->x[jp * d], dij, vi, vj, s->rho[ip], s->rho[jp], pi,
                 pj, s->m[ip], s->m[jp], gradw, s->pid[ip], s->pid[jp], fi, fj);
  } else {
    /* pp_interaction_ff/fw/wf.inc, non-Newtonian branch: a boundary
     * partner takes the fluid particle's density and pressure tensor */
    const int64_t pf = (si != 0) ? jp : ip; /* the fluid one of a fluid-boundary pair */
    const double rho_ip = (si == 0 && sj == 0) ? s->rho[ip] : s->rho[pf];
    const double rho_jp = (si == 0 && sj == 0) ? s->rho[jp] : s->rho[pf];
    /* pp_vgt_ip.inc / pp_vgt_jp.inc */
    const int d2v = d * d;
    for (int b = 0; b < d; ++b)
      for (int a = 0; a < d; ++a) {
        s->vgt[ip * d2v + a + d * b] += (vj[a] - vi[a]) * rij[b] * gradw / rho_ip / dij;
        if (s->p.symmetry)
          s->vgt[jp * d2v + a + d * b] += (vi[a] - vj[a]) * (-rij[b]) * gradw / rho_jp / dij;
      }
    double pti[9], ptj[9];
    const int64_t ci_ = (si == 0 && sj == 0) ? ip : pf;
    const int64_t cj_ = (si == 0 && sj == 0) ? jp : pf;
    pressure_tensor(s, ci_, pti);
    pressure_tensor(s, cj_, ptj);
    rhs_force_nn(s, fc, &s->x[ip * d], &s->x[jp * d], dij, vi, vj, rho_ip, rho_jp, pti, ptj,
                 s->m[ip], s->m[jp], gradw, s->pid[ip], s->pid[jp], fi, fj);
  }
  for (int a = 0; a < d; ++a) s->f[ip * d + a] = s->f[ip * d + a] + fi[a];
  {
    double ni = 0.0, nj = 0.0;
    for (int a = 0; a < d; ++a) {
      ni += fi[a] * fi[a];
      nj += fj[a] * fj[a];
    }
    s->fabs_sum[ip] += sqrt(ni);
    if (s->p.symmetry) s->fabs_sum[jp] += sqrt(nj);
  }
  const int d2 = d * d;
  if (s->p.stress_tensor) {
    /* pp_interaction_ff.inc:83-93: sip = rij(a)*fip(b)/2, sjp = sip */
    for (int b = 0; b < d; ++b)
      for (int a = 0; a < d; ++a) {
        const double sab = rij[a] * fi[b] / 2.0;
        s->s[ip * d2 + b * d + a] = s->s[ip * d2 + b * d + a] + sab;
        if (s->p.symmetry) s->s[jp * d2 + b * d + a] = s->s[jp * d2 + b * d + a] + sab;
      }
  }
  if (s->p.symmetry)
    for (int a = 0; a < d; ++a) s->f[jp * d + a] = s->f[jp * d + a] + fj[a];
}

int orc_compute_interaction(orc_state* s, int64_t step) {
  if (!s->have_pressure) return fail(s, "orc_compute_interaction: no pressure");
  const double t0 = now_s();
  const int d = s->d, d2 = d * d;
  ghost_refresh(s);
  for (int64_t j = 0; j < s->nall * d; ++j) s->f[j] = 0.0;
  for (int64_t j = 0; j < s->nall * d2; ++j) s->s[j] = 0.0;
  for (int64_t j = 0; j < s->nall; ++j) s->fabs_sum[j] = 0.0;
  if (!s->p.Newtonian)
    for (int64_t j = 0; j < s->nall * d2; ++j) s->vgt[j] = 0.0;
  force_ctx fc;
  fc.step = step;
  fc.noise = s->p.Brownian && s->p.kt > s->machine_zero;
  fc.sqdt = 0.0;
  if (fc.noise) fc.sqdt = sqrt(s->p.dt);
  for_all_pairs(s, force_pair, &fc);
  if (s->p.symmetry)
    for (int64_t g = s->nreal; g < s->nall; ++g) {
      const int64_t o = s->owner[g];
      for (int a = 0; a < d; ++a) s->f[o * d + a] = s->f[o * d + a] + s->f[g * d + a];
      s->fabs_sum[o] += s->fabs_sum[g];
      if (!s->p.Newtonian)
        for (int a = 0; a < d2; ++a) s->vgt[o * d2 + a] = s->vgt[o * d2 + a] + s->vgt[g * d2 + a];
      if (s->p.stress_tensor)
        for (int a = 0; a < d2; ++a) s->s[o * d2 + a] = s->s[o * d2 + a] + s->s[g * d2 + a];
    }
  s->timers[2] += now_s() - t0;
  return 0;
}

/* ------------------------------------------------------------------------
 * Body force, particles_apply_body_force.F90:96-353.
 * ---------------------------------------------------------------------- */
int orc_apply_body_force(orc_state* s) {
  const int d = s->d;
  const double* g = s->p.body_force;
  switch (s->p.body_force_type) {
    case 0:
      break;
    case 1:
      for (int i = 0; i < d; ++i)
        if (fabs(g[i]) > s->machine_zero)
          for (int64_t j = 0; j < s->nreal; ++j)
            if (s->sid[j] == 0) s->f[j * d + i] = s->f[j * d + i] + g[i];
      break;
    case 2:
      for (int64_t j = 0; j < s->nreal; ++j) {
        if (!(fabs(g[0]) > s->machine_zero)) continue;
        const double half = s->p.max_phys[d - 1] * 0.5;
        const double xl = s->x[j * d + d - 1];
        if (xl < half && s->sid[j] == 0)
          s->f[j * d] = s->f[j * d] + g[0];
        else if (xl > half && s->sid[j] == 0)
          s->f[j * d] = s->f[j * d] - g[0];
      }
      break;
    case 3: {
      const double k = 2.0 * MK_PI / (s->p.max_phys[1] - s->p.min_phys[1]);
      if (fabs(g[0]) > s->machine_zero)
        for (int64_t j = 0; j < s->nreal; ++j)
          if (s->sid[j] == 0) s->f[j * d] = s->f[j * d] + g[0] * sin(k * s->x[j * d + 1]);
      break;
    }
    default:
      return fail(s, "orc_apply_body_force: body_force_type must be 0..3");
  }
  return 0;
}

/* particles_integrate_velocity.F90:84-94 */
int orc_integrate_velocity(orc_state* s, double dt, double lambda) {
  const int d = s->d;
  for (int64_t j = 0; j < s->nreal; ++j)
    if (s->sid[j] == 0)
      for (int a = 0; a < d; ++a) s->v[j * d + a] = s->v[j * d + a] + lambda * s->f[j * d + a] * dt;
  return 0;
}

/* particles_integrate_position.F90:82-111 (order 1) */
int orc_integrate_position(orc_state* s, double dt) {
  const int d = s->d;
  for (int64_t j = 0; j < s->nreal; ++j)
    if (s->sid[j] == 0)
      for (int a = 0; a < d; ++a) s->x[j * d + a] = s->x[j * d + a] + s->v[j * d + a] * dt;
  return 0;
}

static void set_dt(orc_state* s, double dt) { s->p.dt = dt; }

/* particles_compute_act.F90:112-156: act = c L^T + L c - (c - I)/tau with
 * L = vgt, L(a,b) = vgt[a + d*b] */
static void compute_act(orc_state* s) {
  const int d = s->d, d2 = d * d;
  const double tau = s->p.tau;
  for (int64_t p = 0; p < s->nreal; ++p) {
    const double* c_ = &s->ct[p * d2];
    const double* L = &s->vgt[p * d2];
    for (int j = 0; j < d; ++j)
      for (int i = 0; i < d; ++i) {
        double t_act = 0.0;
        for (int k = 0; k < d; ++k)
          t_act = t_act + c_[i + d * k] * L[j + d * k] + L[i + d * k] * c_[k + d * j];
        s->act[p * d2 + i + d * j] = t_act - (c_[i + d * j] - (i == j ? 1.0 : 0.0)) / tau;
      }
  }
}

/* particles_integrate_ct.F90:66-68 */
static void integrate_ct(orc_state* s, double dt, double lambda) {
  const int d2 = s->d * s->d;
  for (int64_t p = 0; p < s->nreal * d2; ++p) s->ct[p] = s->ct[p] + s->act[p] * dt * lambda;
}

static int rhs(orc_state* s, int64_t step) {
  int rc;
  if ((rc = orc_build_list(s))) return rc;
  if ((rc = orc_compute_density(s))) return rc;
  if ((rc = orc_compute_pressure(s))) return rc;
  if ((rc = orc_compute_interaction(s, step))) return rc;
  const double t0 = now_s();
  rc = orc_apply_body_force(s);
  if (!s->p.Newtonian) compute_act(s); /* marching_integrate_VV.F90:1496 */
  s->timers[3] += now_s() - t0;
  return rc;
}

/* marching_marching.F90:528-911 (initial right-hand side), boundaries
 * updated at time_current first (:437) */
int orc_init_force(orc_state* s, int64_t step) {
  if (s->walls || s->le) boundary_update(s, s->time_current, s->time_current);
  int rc = orc_adjust_particles(s);
  if (rc) return rc;
  rc = rhs(s, step);
  if (rc) return rc;
  if (s->cdyn && s->cp.num_colloid > 0) return colloid_initial_accel(s);
  return 0;
}

/* marching_integrate_VV.F90:303-1620; time_current advanced first
 * (marching_marching.F90:1393) */
int orc_step_vv(orc_state* s, int64_t step, double dt) {
  set_dt(s, dt);
  s->time_current = s->time_current + dt;
  const double time = s->time_current;
  const int d = s->d;
  double t0 = now_s();
  orc_integrate_velocity(s, dt, 0.5);
  orc_integrate_position(s, dt);
  if (!s->p.Newtonian) integrate_ct(s, dt, 0.5); /* marching_integrate_VV.F90:413 */
  if (s->cdyn && s->cp.num_colloid > 0) {
    /* :455-765 */
    int rcc = orc_colloid_integrate(s, step, dt);
    if (rcc) return rcc;
  }
  if (s->walls || s->le) {
    /* :783-806: boundary update, wall particles x + v dt
     * (particles_integrate_boundary_position.F90) */
    boundary_update(s, time + dt, time + 0.5 * dt);
    for (int64_t j = 0; j < s->nreal; ++j)
      if (s->sid[j] < 0)
        for (int a = 0; a < d; ++a) s->x[j * d + a] = s->x[j * d + a] + s->v[j * d + a] * dt;
  }
  orc_adjust_particles(s);
  s->timers[3] += now_s() - t0;
  int rc = rhs(s, step);
  if (rc) return rc;
  t0 = now_s();
  if (!s->p.Newtonian) integrate_ct(s, dt, 0.5); /* :1511 */
  orc_integrate_velocity(s, dt, 0.5);
  if (s->walls || s->le) {
    /* :1650-1675: boundary update at the end of the step, wall particles
     * take their face's shear_v (particles_set_boundary_velocity.F90) */
    boundary_update(s, time + dt, time + dt);
    for (int64_t j = 0; j < s->nreal; ++j)
      if (s->sid[j] < 0) {
        const int f = -s->sid[j] - 1;
        for (int a = 0; a < d; ++a) s->v[j * d + a] = s->shear_v[f][a];
      }
  }
  s->timers[3] += now_s() - t0;
  return 0;
}

int orc_run_vv(orc_state* s, int64_t step0, int32_t nsteps, double dt) {
  for (int32_t k = 1; k <= nsteps; ++k) {
    int rc = orc_step_vv(s, step0 + k, dt);
    if (rc) return rc;
  }
  return 0;
}

int orc_download(orc_state* s, double* x, double* v, double* rho, double* p,
                 double* f, double* ct, double* s_out) {
  const int d = s->d, d2 = d * d;
  const int64_t n = s->nreal;
  if (x) memcpy(x, s->x, sizeof(double) * (size_t)(n * d));
  if (v) memcpy(v, s->v, sizeof(double) * (size_t)(n * d));
  if (rho) memcpy(rho, s->rho, sizeof(double) * (size_t)n);
  if (p) memcpy(p, s->pr, sizeof(double) * (size_t)n);
  if (f) memcpy(f, s->f, sizeof(double) * (size_t)(n * d));
  if (ct) memcpy(ct, s->ct, sizeof(double) * (size_t)(n * d2));
  if (s_out) memcpy(s_out, s->s, sizeof(double) * (size_t)(n * d2));
  return 0;
}

/* statistic_compute_statistic.F90:230-303 over the first n_owned reals (a
 * rank's own particles: the sums MCF all-reduces over the ranks at
 * statistic_compute_statistic.F90:348-403) */
int orc_statistics_owned(orc_state* s, int64_t n_owned, double* k_energy, double* momentum,
                         double* stress) {
  const int d = s->d, d2 = d * d;
  double ke = 0.0, mom[3] = {0, 0, 0}, st[9] = {0};
  const int64_t nown = n_owned < s->nreal ? n_owned : s->nreal;
  for (int64_t j = 0; j < nown; ++j) {
    if (s->sid[j] == 0) {
      double v2 = 0.0;
      for (int a = 0; a < d; ++a) v2 = v2 + s->v[j * d + a] * s->v[j * d + a];
      ke = ke + 0.5 * s->m[j] * v2;
      for (int a = 0; a < d; ++a) mom[a] = mom[a] + s->m[j] * s->v[j * d + a];
    }
    if (s->p.stress_tensor && s->sid[j] >= 0)
      for (int a = 0; a < d2; ++a) st[a] = st[a] + s->s[j * d2 + a];
  }
  if (k_energy) *k_energy = ke;
  if (momentum)
    for (int a = 0; a < 3; ++a) momentum[a] = mom[a];
  if (stress)
    for (int a = 0; a < 9; ++a) stress[a] = a < d2 ? st[a] : 0.0;
  return 0;
}

/* statistic_compute_statistic.F90:230-303 */
int orc_statistics(orc_state* s, double* k_energy, double* momentum, double* stress) {
  return orc_statistics_owned(s, s->nreal, k_energy, momentum, stress);
}

int orc_force_scale(const orc_state* s, double* out) {
  memcpy(out, s->fabs_sum, sizeof(double) * (size_t)s->nreal);
  return 0;
}

int orc_counts(const orc_state* s, int64_t* counts) {
  counts[0] = s->nreal;
  counts[1] = s->nall - s->nreal;
  counts[2] = s->npairs;
  return 0;
}

int orc_timers(const orc_state* s, double* t) {
  for (int i = 0; i < 4; ++i) t[i] = s->timers[i];
  return 0;
}

/* particles_init_global_inter_cubic.F90 / _square: lattice by repeated
 * addition starting at min + dx/2 */
int64_t orc_lattice(int dim, const double* min_t, const double* max_t, const double* dx,
                    double* x_out, int64_t cap) {
  int64_t num = 0;
  double sx[3];
  if (dim == 3) {
    sx[2] = min_t[2] + 0.5 * dx[2];
    while (sx[2] < max_t[2]) {
      sx[1] = min_t[1] + 0.5 * dx[1];
      while (sx[1] < max_t[1]) {
        sx[0] = min_t[0] + 0.5 * dx[0];
        while (sx[0] < max_t[0]) {
          if (x_out && num < cap)
            for (int a = 0; a < 3; ++a) x_out[num * 3 + a] = sx[a];
          num++;
          sx[0] = sx[0] + dx[0];
        }
        sx[1] = sx[1] + dx[1];
      }
      sx[2] = sx[2] + dx[2];
    }
  } else {
    sx[1] = min_t[1] + 0.5 * dx[1];
    while (sx[1] < max_t[1]) {
      sx[0] = min_t[0] + 0.5 * dx[0];
      while (sx[0] < max_t[0]) {
        if (x_out && num < cap)
          for (int a = 0; a < 2; ++a) x_out[num * 2 + a] = sx[a];
        num++;
        sx[0] = sx[0] + dx[0];
      }
      sx[1] = sx[1] + dx[1];
    }
  }
  return num;
}
