// colloid.cu -- rigid-body dynamics of the colloids on the device.
//
// MCF integrates its colloids on the host (Class_Colloid, O(N_c) work) inside
// every VV step, marching_integrate_VV.F90:455-765: the fluid's drag and
// torque are summed from the boundary particles' accelerations, then per
// sub-step the rotation vector, rotation matrix and accumulated orientation,
// the angular velocity, the centre and the velocity are advanced by explicit
// Adams-Bashforth steps (orders 1-5, ramping up after step_start), the
// colloid-colloid repulsion is evaluated at the new centres, the body force
// added, both accelerations recorded in their histories, the centres wrapped
// back into the box, and every boundary particle is turned with its colloid
// and put at the new centre.  Here that runs as three kernels per sub-step
// with no host round trip: k_colloid_drag (update.cu, one warp per colloid),
// k_colloid_rigid (one block, a thread per colloid, the O(N_c) and O(N_c^2)
// parts) and k_colloid_follow (a warp per colloid over its boundary
// particles, which also commits the colloid's new centre, velocity and
// angular velocity to the table the pair sweeps read).  All arithmetic is
// FP64 in the operation order of the Fortran (no fused multiply-add), so the
// state follows the CPU restatement to rounding.
#include <cmath>
#include <vector>

#include "mcfg_internal.cuh"
#include "sph.cuh"

#ifndef TRY
#define TRY(expr)        \
  do {                   \
    int _rc = (expr);    \
    if (_rc) return _rc; \
  } while (0)
#endif

namespace mcfg {

namespace {

// Per-colloid record of the dynamics, kCollRec doubles:
//   m | mmi(3) | theta(3) | drag(3) | torque(3) | rot_matrix(9) |
//   acc_matrix(9) | v(3, AB) | omega(3, AB) | f(3, AB) | alpha(3, AB)
// matrices column-major (i + 3 j), histories level-major, level 1 first.
constexpr int kRecM = 0, kRecMmi = 1, kRecTheta = 4, kRecDrag = 7, kRecTorque = 10,
              kRecRot = 13, kRecAcc = 22, kRecV = 31, kRecOm = 46, kRecF = 61, kRecAl = 76;
constexpr int kMaxAB = 5;
static_assert(kRecAl + 3 * kMaxAB <= kCollRec, "colloid record too small");

struct RigidArgs {
  double* rec;          // [nc][kCollRec]
  double* xnew;         // [nc][3] centres after the sub-step
  const double* fluid;  // [nc][6] fluid drag (3) and torque (3), k_colloid_drag
  const int64_t* step_ptr;
  int64_t step_arg;
  int64_t step_start;
  int isub;      // sub-step 1..sub_time_step
  int mode;      // 0: a sub-step; 1: the initial accelerations only
  int ab;        // integrate_AB
  int translate, rotate;
  int body_force_type;
  double g[3];
  int repul_type;
  double F0, hn, hm;
  double dts;
  double machine_zero;
};

__device__ __forceinline__ int ab_order(int64_t step, int itype) {
  return step < itype ? (int)step : itype;
}

// Adams-Bashforth increment over a history whose level q sits at h[3 q]:
// coefficients times levels left to right, times dt, over the divisor, as
// colloid_integrate_translate_position/_velocity.F90 write it
__device__ __forceinline__ double ab_incr(int order, const double* h, double dt) {
  double s;
  switch (order) {
    case 1:
      return __dmul_rn(h[0], dt);
    case 2:
      s = __dsub_rn(__dmul_rn(3.0, h[0]), h[3]);
      return __ddiv_rn(__dmul_rn(s, dt), 2.0);
    case 3:
      s = __dsub_rn(__dmul_rn(23.0, h[0]), __dmul_rn(16.0, h[3]));
      s = __dadd_rn(s, __dmul_rn(5.0, h[6]));
      return __ddiv_rn(__dmul_rn(s, dt), 12.0);
    case 4:
      s = __dsub_rn(__dmul_rn(55.0, h[0]), __dmul_rn(59.0, h[3]));
      s = __dadd_rn(s, __dmul_rn(37.0, h[6]));
      s = __dsub_rn(s, __dmul_rn(9.0, h[9]));
      return __ddiv_rn(__dmul_rn(s, dt), 24.0);
    default:
      s = __dsub_rn(__dmul_rn(1901.0, h[0]), __dmul_rn(2774.0, h[3]));
      s = __dadd_rn(s, __dmul_rn(2616.0, h[6]));
      s = __dsub_rn(s, __dmul_rn(1274.0, h[9]));
      s = __dadd_rn(s, __dmul_rn(251.0, h[12]));
      return __ddiv_rn(__dmul_rn(s, dt), 720.0);
  }
}

// "h(:,:,i) = h(:,:,i-1), i = itype..2" for one colloid's 3-vector history
__device__ __forceinline__ void ab_shift(double* h, int itype) {
  for (int q = itype - 1; q >= 1; --q)
#pragma unroll
    for (int a = 0; a < 3; ++a) h[3 * q + a] = h[3 * (q - 1) + a];
}

// tool_rotation_matrix.F90, rm(i,j) at rm[i + 3 j]
__device__ __forceinline__ void rotation_matrix(const double* ax, double phi, double* rm) {
  const double cp = cos(phi), cp1 = __dsub_rn(1.0, cp), sp = sin(phi);
  auto d = [&](int i, int j) { return __dmul_rn(__dmul_rn(ax[i], ax[j]), cp1); };
  rm[0 + 3 * 0] = __dadd_rn(d(0, 0), cp);
  rm[0 + 3 * 1] = __dsub_rn(d(0, 1), __dmul_rn(ax[2], sp));
  rm[0 + 3 * 2] = __dadd_rn(d(0, 2), __dmul_rn(ax[1], sp));
  rm[1 + 3 * 0] = __dadd_rn(d(1, 0), __dmul_rn(ax[2], sp));
  rm[1 + 3 * 1] = __dadd_rn(d(1, 1), cp);
  rm[1 + 3 * 2] = __dsub_rn(d(1, 2), __dmul_rn(ax[0], sp));
  rm[2 + 3 * 0] = __dsub_rn(d(2, 0), __dmul_rn(ax[1], sp));
  rm[2 + 3 * 1] = __dadd_rn(d(2, 1), __dmul_rn(ax[0], sp));
  rm[2 + 3 * 2] = __dadd_rn(d(2, 2), cp);
}

// One block, a thread per colloid (strided).  mode 0, one sub-step of
// marching_integrate_VV.F90:494-760:
//   A  colloid_compute_rotation_vector / _rotation_matrix /
//      _accumulation_matrix, colloid_integrate_rotate_velocity,
//      colloid_integrate_translate_position / _velocity;
//   B  colloid_compute_interaction (fluid drag + colloid-colloid repulsion
//      at the new centres, colloid_compute_repulsion_cc.F90, partners in
//      index order), colloid_apply_body_force,
//      colloid_compute_translate_acceleration;
//   C  colloid_adjust_colloid (after every thread has read the unwrapped
//      centres), colloid_compute_rotate_acceleration.
// mode 1, the initial accelerations of marching_marching.F90:995-1110: B at
// the current centres, then the rotate acceleration.
template <int D>
__global__ void k_colloid_rigid(Consts k, RigidArgs a) {
  const int nc = k.ncoll;
  const int64_t step = a.step_ptr ? *a.step_ptr : a.step_arg;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    double* r = a.rec + (size_t)c * kCollRec;
    const double* cd = k.coll + (size_t)c * 12;
    double xn[3] = {cd[0], cd[1], cd[2]};
    if (a.mode == 0) {
      const int oa = ab_order(step - 1 + a.isub - a.step_start, a.ab);
      // colloid_integrate_rotate_velocity is handed step-1+i+step_start
      const int orr = ab_order(step - 1 + a.isub + a.step_start, a.ab);
      if (a.rotate) {
        double ax[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) ax[q] = ab_incr(oa, r + kRecOm + q, a.dts);
        double phi = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(ax[0], ax[0]), __dmul_rn(ax[1], ax[1])),
                                    __dmul_rn(ax[2], ax[2])));
        if (phi < a.machine_zero) {
          phi = 0.0;
          ax[0] = 1.0;
          ax[1] = ax[2] = 0.0;
        } else {
#pragma unroll
          for (int q = 0; q < 3; ++q) ax[q] = __ddiv_rn(ax[q], phi);
        }
        r[kRecTheta + 2] = __dadd_rn(r[kRecTheta + 2], phi);
        double* rm = r + kRecRot;
        rotation_matrix(ax, phi, rm);
        double acc[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            double t = 0.0;
#pragma unroll
            for (int q = 0; q < 3; ++q)
              t = __dadd_rn(t, __dmul_rn(rm[i + 3 * q], r[kRecAcc + q + 3 * j]));
            acc[i + 3 * j] = t;
          }
#pragma unroll
        for (int q = 0; q < 9; ++q) r[kRecAcc + q] = acc[q];
        ab_shift(r + kRecOm, a.ab);
#pragma unroll
        for (int q = 0; q < 3; ++q)
          r[kRecOm + q] = __dadd_rn(r[kRecOm + q], ab_incr(orr, r + kRecAl + q, a.dts));
      }
      if (a.translate) {
#pragma unroll
        for (int q = 0; q < D; ++q) xn[q] = __dadd_rn(xn[q], ab_incr(oa, r + kRecV + q, a.dts));
        ab_shift(r + kRecV, a.ab);
#pragma unroll
        for (int q = 0; q < D; ++q)
          r[kRecV + q] = __dadd_rn(r[kRecV + q], ab_incr(oa, r + kRecF + q, a.dts));
      }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) a.xnew[(size_t)c * 3 + q] = xn[q];
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    double* r = a.rec + (size_t)c * kCollRec;
    const double rad_c = k.coll[(size_t)c * 12 + 9];
    double xc[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < D; ++q) xc[q] = a.xnew[(size_t)c * 3 + q];
    double rep[3] = {0.0, 0.0, 0.0};
    if (a.repul_type >= 1) {
      for (int j = 0; j < nc; ++j) {
        if (j == c) continue;
        double R12[3] = {0.0, 0.0, 0.0}, rr = 0.0;
#pragma unroll
        for (int q = 0; q < D; ++q) {
          double t = __dsub_rn(xc[q], a.xnew[(size_t)j * 3 + q]);
          if (k.periodic[q]) {
            if (t > 0.5 * k.len[q])
              t = __dsub_rn(t, k.len[q]);
            else if (t < -0.5 * k.len[q])
              t = __dadd_rn(t, k.len[q]);
          }
          R12[q] = t;
          rr = __dadd_rn(rr, __dmul_rn(t, t));
        }
        const double rd = sqrt(rr);
        double hgap = __dsub_rn(rd, __dadd_rn(rad_c, k.coll[(size_t)j * 12 + 9]));
        if (!(hgap < 5.0 * a.hn)) continue;
        double F = 0.0;
        if (a.repul_type == 1) {  // Hookean
          if (hgap < a.hn) {
            if (hgap < a.hm) hgap = a.hm;
            F = __dsub_rn(a.F0, __ddiv_rn(__dmul_rn(a.F0, hgap), a.hn));
          }
        } else {  // DLVO
          if (hgap < a.hm) hgap = a.hm;
          const double e1 = exp(__ddiv_rn(-hgap, a.hn)), e5 = exp(-5.0);
          F = __dsub_rn(__ddiv_rn(__dmul_rn(__ddiv_rn(a.F0, a.hn), e1), __dsub_rn(1.0, e1)),
                        __ddiv_rn(__dmul_rn(__ddiv_rn(a.F0, a.hn), e5), __dsub_rn(1.0, e5)));
        }
#pragma unroll
        for (int q = 0; q < D; ++q) rep[q] = __dadd_rn(rep[q], __dmul_rn(F, __ddiv_rn(R12[q], rd)));
      }
    }
    const double m = r[kRecM];
#pragma unroll
    for (int q = 0; q < D; ++q) {
      double dr = __dadd_rn(a.fluid[(size_t)c * 6 + q], rep[q]);
      if (a.body_force_type == 1) dr = __dadd_rn(dr, __dmul_rn(a.g[q], m));
      r[kRecDrag + q] = dr;
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) r[kRecTorque + q] = a.fluid[(size_t)c * 6 + 3 + q];
    ab_shift(r + kRecF, a.ab);
#pragma unroll
    for (int q = 0; q < D; ++q) r[kRecF + q] = a.translate ? __ddiv_rn(r[kRecDrag + q], m) : 0.0;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    double* r = a.rec + (size_t)c * kCollRec;
    if (a.mode == 0) {
      const double rad_c = k.coll[(size_t)c * 12 + 9];
#pragma unroll
      for (int q = 0; q < D; ++q) {
        double x = a.xnew[(size_t)c * 3 + q];
        const double lo = k.min_phys[q], hi = k.max_phys[q], L = __dsub_rn(hi, lo);
        if (x < lo) {
          if (k.bc_lo[q] == MCFG_BC_PERIODIC) {
            const int nover = (int)__ddiv_rn(__dsub_rn(hi, x), L);
            x = __dadd_rn(x, __dmul_rn(L, (double)nover));
          } else if (k.bc_lo[q] == MCFG_BC_WALL_SOLID) {
            x = __dadd_rn(lo, rad_c);
            r[kRecV + q] = 0.0;
          }
        }
        if (x >= hi) {
          if (k.bc_hi[q] == MCFG_BC_PERIODIC) {
            const int nover = (int)__ddiv_rn(__dsub_rn(x, lo), L);
            x = __dsub_rn(x, __dmul_rn(L, (double)nover));
          } else if (k.bc_hi[q] == MCFG_BC_WALL_SOLID) {
            x = __dsub_rn(__dsub_rn(hi, rad_c), a.machine_zero);
            r[kRecV + q] = 0.0;
          }
        }
        a.xnew[(size_t)c * 3 + q] = x;
      }
    }
    ab_shift(r + kRecAl, a.ab);
    if (a.rotate) {
      if (D == 2) {
        r[kRecAl + 2] = __ddiv_rn(r[kRecTorque + 2], r[kRecMmi + 2]);
      } else {
#pragma unroll
        for (int q = 0; q < 3; ++q) r[kRecAl + q] = __ddiv_rn(r[kRecTorque + q], r[kRecMmi + q]);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 3; ++q) r[kRecAl + q] = 0.0;
    }
  }
}

// particles_compute_colloid_relative_position.F90 and _absolute_position.F90
// around one sub-step: each boundary particle relative to the nearest image
// of its colloid's old centre, turned by the sub-step's rotation matrix, put
// at the new centre in the same periodic image as before (so list reuse sees
// a small displacement); then lane 0 writes the colloid's new centre,
// velocity and angular velocity into the table the sweeps read.  One warp per
// colloid: the warp reads only its own colloid's table row.
template <int D>
__global__ void k_colloid_follow(Consts k, const int* __restrict__ cstart,
                                 const int* __restrict__ cmem, const int* __restrict__ slot_of,
                                 const double* __restrict__ rec, const double* __restrict__ xnew,
                                 int rotate, double4_32a* __restrict__ x) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= k.ncoll) return;
  double* cd = const_cast<double*>(k.coll) + (size_t)c * 12;
  const double* r = rec + (size_t)c * kCollRec;
  for (int q = cstart[c] + lane; q < cstart[c + 1]; q += 32) {
    const int s = slot_of[cmem[q]];
    const double4_32a xv = x[s];
    const double xs[3] = {xv.x, xv.y, xv.z};
    double rx[3] = {0.0, 0.0, 0.0};
    colloid_rx<D>(k, xs, c, rx);
    double rb[3] = {rx[0], rx[1], rx[2]};
    if (rotate) {
#pragma unroll
      for (int i = 0; i < D; ++i) {
        double t = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) t = __dadd_rn(t, __dmul_rn(r[kRecRot + i + 3 * j], rx[j]));
        rb[i] = t;
      }
    }
    double xo[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < D; ++i) {
      const double img = (xs[i] - rx[i]) - cd[i];
      double xn = __dadd_rn(rb[i], xnew[(size_t)c * 3 + i]);
      if (k.periodic[i] && fabs(img) > 0.5 * k.len[i])
        xn = __dadd_rn(xn, img > 0.0 ? k.len[i] : -k.len[i]);
      xo[i] = xn;
    }
    x[s] = make_double4_32a(xo[0], xo[1], D == 3 ? xo[2] : 0.0, 0.0);
  }
  __syncwarp();
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      cd[i] = xnew[(size_t)c * 3 + i];
      cd[3 + i] = (i < D) ? r[kRecV + i] : 0.0;
      cd[6 + i] = r[kRecOm + i];
    }
  }
}

RigidArgs rigid_args(Handle* h, int64_t step, int isub, int mode, double dts) {
  RigidArgs a;
  a.rec = h->crec;
  a.xnew = h->cxnew;
  a.fluid = h->coll_out;
  a.step_ptr = h->graph_capturing ? h->d_step : nullptr;
  a.step_arg = step;
  a.step_start = h->cdp.step_start;
  a.isub = isub;
  a.mode = mode;
  a.ab = h->cdp.integrate_AB;
  a.translate = h->cp.translate;
  a.rotate = h->cp.rotate;
  a.body_force_type = h->cdp.body_force_type;
  for (int q = 0; q < 3; ++q) a.g[q] = h->cdp.body_force[q];
  a.repul_type = h->cp.cc_repul_type;
  a.F0 = h->cp.cc_repul_F0;
  a.hn = h->cp.cc_repul_cut_off;
  a.hm = h->cp.cc_repul_cut_on;
  a.dts = dts;
  a.machine_zero = h->k.machine_zero;
  return a;
}

int launch_rigid(Handle* h, const RigidArgs& a) {
  const int nc = h->k.ncoll;
  const int bs = nc >= 1024 ? 1024 : ((nc + 31) / 32) * 32;
  if (h->k.d == 3)
    k_colloid_rigid<3><<<1, bs, 0, h->stream>>>(h->k, a);
  else
    k_colloid_rigid<2><<<1, bs, 0, h->stream>>>(h->k, a);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "colloid rigid-body launch") ? MCFG_ECUDA : MCFG_OK;
}

int launch_follow(Handle* h) {
  const int nc = h->k.ncoll;
  const int warps_per_block = 4;
  const int g = (nc + warps_per_block - 1) / warps_per_block;
  if (h->k.d == 3)
    k_colloid_follow<3><<<g, 32 * warps_per_block, 0, h->stream>>>(
        h->k, h->coll_start, h->coll_mem, h->slot_of, h->crec, h->cxnew, h->cp.rotate, h->x);
  else
    k_colloid_follow<2><<<g, 32 * warps_per_block, 0, h->stream>>>(
        h->k, h->coll_start, h->coll_mem, h->slot_of, h->crec, h->cxnew, h->cp.rotate, h->x);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "colloid follow launch") ? MCFG_ECUDA : MCFG_OK;
}

}  // namespace

// the colloid part of a VV step (marching_integrate_VV.F90:455-765)
int colloid_section(Handle* h, int64_t step, double dt) {
  if (!h->cdyn || h->k.ncoll == 0) return MCFG_OK;
  TRY(colloid_drag_launch(h));
  if (!(h->cp.translate || h->cp.rotate)) return MCFG_OK;
  const int nsub = h->cdp.sub_time_step;
  const double dts = dt / (double)nsub;
  for (int i = 1; i <= nsub; ++i) {
    TRY(launch_rigid(h, rigid_args(h, step, i, 0, dts)));
    TRY(launch_follow(h));
  }
  h->coll_host_stale = true;
  return MCFG_OK;
}

// the initial colloid accelerations after the first right-hand side
// (marching_marching.F90:995-1110)
int colloid_initial(Handle* h) {
  if (!h->cdyn || h->k.ncoll == 0) return MCFG_OK;
  TRY(colloid_drag_launch(h));
  TRY(launch_rigid(h, rigid_args(h, 0, 1, 1, 0.0)));
  return MCFG_OK;
}

// host copies of the colloid table (centres, velocities, angular
// velocities) after device-side dynamics
int colloid_sync_host(Handle* h) {
  if (!h->coll_host_stale) return MCFG_OK;
  const int nc = h->k.ncoll, d = h->p.num_dim;
  std::vector<double> buf((size_t)nc * 12);
  if (cuda_check(h, cudaMemcpyAsync(buf.data(), h->coll, sizeof(double) * buf.size(),
                                    cudaMemcpyDeviceToHost, h->stream), "colloid table") ||
      cuda_check(h, cudaStreamSynchronize(h->stream), "colloid table"))
    return MCFG_ECUDA;
  for (int c = 0; c < nc; ++c) {
    for (int a = 0; a < d; ++a) {
      h->cx[(size_t)c * d + a] = buf[(size_t)c * 12 + a];
      h->cv[(size_t)c * d + a] = buf[(size_t)c * 12 + 3 + a];
    }
    for (int a = 0; a < 3; ++a) h->com[(size_t)c * 3 + a] = buf[(size_t)c * 12 + 6 + a];
  }
  h->coll_host_stale = false;
  return MCFG_OK;
}

}  // namespace mcfg
