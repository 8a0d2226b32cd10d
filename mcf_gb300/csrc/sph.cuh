// sph.cuh -- SPH kernel, equation of state and pair force forms, templated
// on the arithmetic type (double: FP64 path, float: FP32-mixed path).
#pragma once
#include "mcfg_internal.cuh"

namespace mcfg {

// Does a particle of species sid sum its density over its pairs?  Fluid
// always; walls with wall_rho_type 1 and colloid boundary particles with
// coll_rho_type 1 (dynamic); the others keep init_density
// (particles_compute_density.F90:700-771, :812-815).
__device__ __forceinline__ bool dyn_rho(const Consts& k, int sid) {
  if (sid == 0) return true;
  if (sid < 0) return k.wall_rho_type == 1;
  return k.coll_rho_type == 1;
}

template <typename T>
struct KC;  // kernel and pair constants in T
template <>
struct KC<double> {
  // the kernel's argument s = r / h as MCF divides it
  // (kernel_kernel_quintic_spline.F90:69,177): near the cut-off W and W'
  // amplify a rounding difference of s by 4-5 s / (3 - s), so the FP64 path
  // keeps MCF's division
  __device__ static double arg(const Consts& k, double r) { return r / k.h; }
  __device__ static double inv_h(const Consts& k) { return k.inv_h; }
  __device__ static double coef(const Consts& k) { return k.coef; }
  __device__ static double coef_grad(const Consts& k) { return k.coef_grad; }
  __device__ static double eta(const Consts& k) { return k.eta; }
  __device__ static double kt(const Consts& k) { return k.kt; }
  __device__ static double eta_coef(const Consts& k) { return k.eta_coef; }
};
template <>
struct KC<float> {
  __device__ static float arg(const Consts& k, float r) { return r * k.inv_hf; }
  __device__ static float inv_h(const Consts& k) { return k.inv_hf; }
  __device__ static float coef(const Consts& k) { return k.coeff; }
  __device__ static float coef_grad(const Consts& k) { return k.coef_gradf; }
  __device__ static float eta(const Consts& k) { return k.etaf; }
  __device__ static float kt(const Consts& k) { return k.ktf; }
  __device__ static float eta_coef(const Consts& k) { return k.eta_coeff; }
};

// W(r): kernel_kernel_quintic_spline.F90:69-99 (h = rc/3, W = coef*[(3-s)^5
// - 6(2-s)^5 + 15(1-s)^5] piecewise) and kernel_kernel_Lucy.F90:68-78.
template <typename T>
__device__ __forceinline__ T kernel_w(const Consts& k, T r) {
  const T s = KC<T>::arg(k, r);
  if (k.kernel_type == 1) {
    const T s3 = T(3) - s, s2 = T(2) - s, s1 = T(1) - s;
    T a3 = s3 * s3;
    a3 = a3 * a3 * s3;
    T w = T(0);
    if (s < T(3)) w = a3;
    if (s < T(2)) {
      T a2 = s2 * s2;
      a2 = a2 * a2 * s2;
      w = w - T(6) * a2;
    }
    if (s < T(1)) {
      T a1 = s1 * s1;
      a1 = a1 * a1 * s1;
      w = w + T(15) * a1;
    }
    return KC<T>::coef(k) * w;
  } else {
    if (s > T(1)) return T(0);
    const T om = T(1) - s;
    return KC<T>::coef(k) * (T(1) + T(3) * s) * (om * om * om);
  }
}

// dW/dr: kernel_kernel_quintic_spline.F90:177-215, kernel_kernel_Lucy.F90:155-168
template <typename T>
__device__ __forceinline__ T kernel_gradw(const Consts& k, T r) {
  const T s = KC<T>::arg(k, r);
  if (k.kernel_type == 1) {
    const T s3 = T(3) - s, s2 = T(2) - s, s1 = T(1) - s;
    T g = T(0);
    if (s < T(3)) {
      const T a = s3 * s3;
      g = T(5) * (a * a);
    }
    if (s < T(2)) {
      const T a = s2 * s2;
      g = g - T(30) * (a * a);
    }
    if (s < T(1)) {
      const T a = s1 * s1;
      g = g + T(75) * (a * a);
    }
    return KC<T>::coef_grad(k) * g;
  } else {
    if (s > T(1)) return T(0);
    const T om = T(1) - s;
    return KC<T>::coef_grad(k) * T(12) * s * (om * om);
  }
}

// d2W/dr2 for the adjoint: the derivative in r of kernel_gradw's
// polynomials (quintic: coef/h^2 [20(3-s)^3 - 120(2-s)^3 + 300(1-s)^3]
// piecewise; Lucy: -12 coef/h^2 (1-s)(1-3s)).
template <typename T>
__device__ __forceinline__ T kernel_grad2w(const Consts& k, T r) {
  const T s = r * KC<T>::inv_h(k);
  const T cg = KC<T>::coef_grad(k) * KC<T>::inv_h(k);  // -coef/h^2
  if (k.kernel_type == 1) {
    const T s3 = T(3) - s, s2 = T(2) - s, s1 = T(1) - s;
    T g = T(0);
    if (s < T(3)) g = T(-20) * (s3 * s3 * s3);
    if (s < T(2)) g = g + T(120) * (s2 * s2 * s2);
    if (s < T(1)) g = g - T(300) * (s1 * s1 * s1);
    return cg * g;
  } else {
    if (s > T(1)) return T(0);
    return cg * T(12) * (T(1) - s) * (T(1) - T(3) * s);
  }
}

// dW/dr and d2W/dr2 together (the adjoint evaluates both per pair): the
// same polynomials as kernel_gradw and kernel_grad2w sharing their powers
template <typename T>
__device__ __forceinline__ void kernel_gradw2(const Consts& k, T r, T& gw, T& g2) {
  const T s = r * KC<T>::inv_h(k);
  const T cgr = KC<T>::coef_grad(k);
  if (k.kernel_type == 1) {
    const T s3 = T(3) - s, s2 = T(2) - s, s1 = T(1) - s;
    T a = T(0), b = T(0);
    if (s < T(3)) {
      const T q = s3 * s3;
      a = T(5) * (q * q);
      b = T(-20) * (q * s3);
    }
    if (s < T(2)) {
      const T q = s2 * s2;
      a = a - T(30) * (q * q);
      b = b + T(120) * (q * s2);
    }
    if (s < T(1)) {
      const T q = s1 * s1;
      a = a + T(75) * (q * q);
      b = b - T(300) * (q * s1);
    }
    gw = cgr * a;
    g2 = cgr * KC<T>::inv_h(k) * b;
  } else {
    if (s > T(1)) {
      gw = T(0);
      g2 = T(0);
      return;
    }
    const T om = T(1) - s;
    gw = cgr * T(12) * s * (om * om);
    g2 = cgr * KC<T>::inv_h(k) * T(12) * om * (T(1) - T(3) * s);
  }
}

// Pressure, stateEquation_compute_pressure.F90:147-180 (vector forms):
// Morris p = c^2 (rho^gamma - rho_ref), Batchelor p = p0((rho/rho_ref)^gamma - 1).
__device__ __forceinline__ double eos_pressure(const Consts& k, double rho) {
  if (k.eos_type == 1) {
    const double rg = (k.gamma == 1.0) ? rho : pow(rho, k.gamma);
    return k.c2 * (rg - k.rho_ref);
  }
  const double q = rho / k.rho_ref;
  const double qg = (k.gamma == 1.0) ? q : pow(q, k.gamma);
  return k.p0 * (qg - 1.0);
}

// Per-particle pair coefficients (A, B, C) of each force form so that the
// pair loop does no division by per-particle quantities:
//   type 1 Morris      : A = p/rho^2, B = 1/rho, C = m
//   type 2 Espanol     : A = p/n^2,   B = 1/n,   C = 1/m
//   type 3 Hu-Adams    : A = p/n^2,   B = 1/n^2, C = 1/m
//   type 4 HA angular  : A = p,       B = 1/n^2, C = 1/m
__device__ __forceinline__ double4_32a pair_coeffs(const Consts& k, double rho, double p, double m) {
  const double inv = 1.0 / rho;
  double4_32a r;
  switch (k.rhs_force_type) {
    case 1:
      r = make_double4_32a(p * inv * inv, inv, m, p);
      break;
    case 2:
      r = make_double4_32a(p * inv * inv, inv, 1.0 / m, p);
      break;
    case 3:
      r = make_double4_32a(p * inv * inv, inv * inv, 1.0 / m, p);
      break;
    default:
      r = make_double4_32a(p, inv * inv, 1.0 / m, p);
      break;
  }
  return r;
}

// A coefficient of a boundary particle whose pressure is replaced by the
// fluid partner's (pp_interaction_fw.inc: this%p(jp) = this%p(ip)).
template <typename T>
__device__ __forceinline__ T boundary_A(int type, T p_fluid, T B) {
  switch (type) {
    case 1:
    case 2:
      return p_fluid * B * B;
    case 3:
      return p_fluid * B;
    default:
      return p_fluid;
  }
}

template <typename T>
__device__ __forceinline__ T my_sqrt(T a);
template <>
__device__ __forceinline__ double my_sqrt<double>(double a) { return sqrt(a); }
template <>
__device__ __forceinline__ float my_sqrt<float>(float a) { return sqrtf(a); }

// Pair force of rhs_force_ff_Newtonian_{Morris,Espanol,HuAdams,
// HuAdams_angular}.F90 before the mass factor: the acceleration of i is
// g * scale_i, that of j is -g * scale_j, with (scale_i, scale_j) =
// (m_j, m_i) for Morris (C = m) and (1/m_i, 1/m_j) otherwise (C = 1/m); see
// pair_scales.  r = x_i - x_j (image), inv_d = 1/|r|, vij = v_i - v_j.
template <typename T, int D>
__device__ __forceinline__ void pair_force(const Consts& k, const T* r, T inv_d, const T* vij,
                                           T Ai, T Bi, T Aj, T Bj, T gw, bool noise,
                                           const float* z, T inv_sqdt, T* g) {
  T e[3];
#pragma unroll
  for (int a = 0; a < D; ++a) e[a] = r[a] * inv_d;
  const T eta = KC<T>::eta(k);
  const T kt = KC<T>::kt(k);
  const T eta_coef = KC<T>::eta_coef(k);
  switch (k.rhs_force_type) {
    case 1: {
      const T f_c = (Ai + Aj) * gw;
      const T f_d = T(2) * eta * gw * Bi * Bj * inv_d;
#pragma unroll
      for (int a = 0; a < D; ++a) g[a] = f_d * vij[a] - f_c * e[a];
      break;
    }
    case 2: {
      T ev = T(0);
#pragma unroll
      for (int a = 0; a < D; ++a) ev += e[a] * vij[a];
      const T f_c = (Ai + Aj) * gw;
      const T bb = Bi * Bj * gw * inv_d * eta;
      const T f_d1 = (T(2) - T(1) / T(D)) * bb;
      const T f_d2 = (T(D + 2) / T(D)) * bb * ev;
#pragma unroll
      for (int a = 0; a < D; ++a) g[a] = f_d1 * vij[a] + (f_d2 - f_c) * e[a];
      if (noise) {
        T dW[3][3];
        T tr = T(0);
#pragma unroll
        for (int a = 0; a < D; ++a) {
          dW[a][a] = (T)z[a];
          tr += dW[a][a];
        }
        tr = tr / T(D);
        const T s2 = T(0.70710678118654752440);
        if (D == 3) {
          dW[0][1] = dW[1][0] = (T)z[3] * s2;
          dW[0][2] = dW[2][0] = (T)z[4] * s2;
          dW[1][2] = dW[2][1] = (T)z[5] * s2;
        } else {
          dW[0][1] = dW[1][0] = (T)z[2] * s2;
        }
#pragma unroll
        for (int a = 0; a < D; ++a) dW[a][a] -= tr;
        const T Zij = T(4) * kt * gw * inv_d * Bi * Bj;
        const T aa = T(5) * eta / T(3);
        const T bq = (T(D) + T(2)) * eta / T(3);
        const T Aij = my_sqrt<T>(-Zij * aa);
        const T Bij = my_sqrt<T>(-Zij * T(D) / T(2) * (bq + aa * (T(2) / T(D) - T(1))));
#pragma unroll
        for (int a = 0; a < D; ++a) {
          T We = T(0);
#pragma unroll
          for (int b = 0; b < D; ++b) We += dW[a][b] * e[b];
          g[a] += (Aij * We + Bij * tr * e[a]) * inv_sqdt;
        }
      }
      break;
    }
    case 3: {
      const T f_c = (Ai + Aj) * gw;
      const T f_d = eta * (Bi + Bj) * gw * inv_d;
#pragma unroll
      for (int a = 0; a < D; ++a) g[a] = f_d * vij[a] - f_c * e[a];
      if (noise) {
        // MCF uses its symmetric traceless dW only through We = dW e, a
        // Gaussian vector with variance 1 - 1/d along e and 1/2 across e;
        // drawn directly as s (ca (e.g) e + cb (g - (e.g) e)) from d normals
        // g (pair_draw), s = +-1 by pid order so both sides get opposite We
        const T cb = T(0.70710678118654752440);
        const T ca = (D == 3) ? T(0.81649658092772603273) : cb;  // sqrt(1 - 1/d)
        T eg = T(0);
#pragma unroll
        for (int a = 0; a < D; ++a) eg += e[a] * (T)z[a];
        const T f_r = my_sqrt<T>(T(-4) * kt * f_d) * inv_sqdt * (T)z[5];
        const T fl = f_r * (ca - cb) * eg, ft = f_r * cb;
#pragma unroll
        for (int a = 0; a < D; ++a) g[a] += fl * e[a] + ft * (T)z[a];
      }
      break;
    }
    default: {
      T ev = T(0);
#pragma unroll
      for (int a = 0; a < D; ++a) ev += e[a] * vij[a];
      const T pij = (Ai + Aj) * T(0.5);
      const T Aij = (Bi + Bj) * gw;
      const T f_c = Aij * pij;
      const T f_d = eta_coef * eta * Aij * ev * inv_d;
      T fe = f_d - f_c;
      if (noise) {
        const T eps = (T)z[0];
        fe += eps * my_sqrt<T>(T(2) * kt * eta) * my_sqrt<T>(-eta_coef * Aij * inv_d) * inv_sqdt;
      }
#pragma unroll
      for (int a = 0; a < D; ++a) g[a] = fe * e[a];
      break;
    }
  }
}

// (scale_i, scale_j) of pair_force from the C coefficients
template <typename T>
__device__ __forceinline__ void pair_scales(int type, T Ci, T Cj, T& si, T& sj) {
  if (type == 1) {
    si = Cj;
    sj = Ci;
  } else {
    si = Ci;
    sj = Cj;
  }
}

template <typename T>
struct WallV;
template <>
struct WallV<double> {
  __device__ static double get(const Consts& k, int f, int a) { return k.wall_v[f][a]; }
};
template <>
struct WallV<float> {
  __device__ static float get(const Consts& k, int f, int a) { return k.wall_vf[f][a]; }
};

// Morris no-slip velocity of a solid-wall particle,
// boundary_noslip_solid.F90:40-95 (frozen) and :137-240 (Morris).  Wall
// particles carry sid = -face (face 1..2d: axis (face-1)/2, lower if odd);
// f_sur / w_sur are the fluid / wall coordinates minus the face coordinate
// along that axis.
template <typename T, int D>
__device__ __forceinline__ void wall_noslip_dist(const Consts& k, T f_sur, T w_sur, const T* vf,
                                                 int sid_w, T* vw) {
  // face velocity, selected with constant indices (a dynamic index into the
  // kernel-parameter block would force a local-memory copy of it)
  T sv[3] = {T(0), T(0), T(0)};
  const int fi = -sid_w - 1;
#pragma unroll
  for (int f = 0; f < 6; ++f)
    if (f == fi) {
#pragma unroll
      for (int a = 0; a < 3; ++a) sv[a] = WallV<T>::get(k, f, a);
    }
  if (k.wall_noslip_type <= 1 || f_sur * w_sur >= T(0)) {
#pragma unroll
    for (int a = 0; a < D; ++a) vw[a] = sv[a];
    return;
  }
  T corr = fabs(w_sur) / fabs(f_sur);
  if (corr > T(0.5)) corr = T(0.5);  // mcf_wall_dist_ratio, mcf_header.F90:282
#pragma unroll
  for (int a = 0; a < D; ++a) vw[a] = -corr * (vf[a] - sv[a]) + sv[a];
}

// same from FP64 coordinates along the wall-normal axis
template <typename T, int D>
__device__ __forceinline__ void wall_noslip(const Consts& k, double xf_n, double xw_n,
                                            const T* vf, int sid_w, T* vw) {
  const int index_w = -sid_w;
  const int axis = (index_w - 1) >> 1;
  double x_sur = 0.0;
#pragma unroll
  for (int a = 0; a < D; ++a)
    if (a == axis) x_sur = (index_w & 1) ? k.min_phys[a] : k.max_phys[a];
  wall_noslip_dist<T, D>(k, (T)(xf_n - x_sur), (T)(xw_n - x_sur), vf, sid_w, vw);
}

// ---------------------------------------------------------------------------
// Colloids (spheres in 3D, disks in 2D)
// ---------------------------------------------------------------------------
// colloid_in_nearest_image.F90 (periodic part), FP64: rx = x - nearest image
// of colloid c's centre, looked for within radius + dout per axis
template <int D>
__device__ __forceinline__ void colloid_rx(const Consts& k, const double* x, int c, double* rx) {
  const double* cd = k.coll + (size_t)c * 12;
  const double dmax = cd[9] + k.coll_dout;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    double xi = cd[a];
    const double r = x[a] - xi;
    if (r > dmax && k.periodic[a])
      xi = xi + k.len[a];
    else if (-r > dmax && k.periodic[a])
      xi = xi - k.len[a];
    rx[a] = x[a] - xi;
  }
}

template <typename T>
__device__ __forceinline__ void cross3t(const T* a, const T* b, T* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// Morris no-slip velocity of a colloid boundary particle seen from a fluid
// particle, colloid_noslip_Morris_sphere.F90:129-300 (disk alike in 2D):
// r_xc = boundary particle - colloid image centre, r_fc = fluid - boundary
// particle (pair separation), vf the fluid velocity.
template <typename T, int D>
__device__ __forceinline__ void colloid_noslip(const Consts& k, int c, const T* r_xc,
                                               const T* r_fc, const T* vf, T* vc) {
  const double* cd = k.coll + (size_t)c * 12;
  const T R = (T)cd[9];
  T V[3] = {(T)cd[3], (T)cd[4], (T)cd[5]};
  const T om[3] = {(T)cd[6], (T)cd[7], (T)cd[8]};
  T r_xf[3] = {0, 0, 0};
  T dd = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    r_xf[a] = r_xc[a] + r_fc[a];
    dd += r_xf[a] * r_xf[a];
  }
  const T d_fcoll = my_sqrt<T>(dd);
  if (d_fcoll <= R) {
    T w[3] = {0, 0, 0};
    if (k.coll_rotate) {
      const T r3[3] = {r_xc[0], r_xc[1], D == 3 ? r_xc[2] : T(0)};
      cross3t<T>(om, r3, w);
    }
#pragma unroll
    for (int a = 0; a < D; ++a) vc[a] = V[a] + w[a];
    return;
  }
  T d_cn = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) d_cn += r_xc[a] * r_xf[a] / d_fcoll;
  const T d_cs = R - d_cn;
  const T d_fs = d_fcoll - R;
  T corr;
  if (fabs(d_fs) < (T)k.machine_zero) {
    corr = T(0.5);  // mcf_colloid_dist_ratio_max
  } else {
    corr = d_cs / d_fs;
    if (corr > T(0.5)) corr = T(0.5);
    else if (corr < T(-0.5)) corr = T(-0.5);
  }
  T r_vs[3] = {0, 0, 0};
  if (k.coll_rotate) {
    T r_xs[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) r_xs[a] = R / d_fcoll * r_xf[a];
    cross3t<T>(om, r_xs, r_vs);
  }
#pragma unroll
  for (int a = 0; a < D; ++a) vc[a] = -corr * (vf[a] - V[a] - r_vs[a]) + V[a] + r_vs[a];
}

}  // namespace mcfg
