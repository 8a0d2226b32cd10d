// sweep_common.cuh -- pieces shared by the pair sweeps (pair_kernels.cu,
// sweep32.cu): the Oldroyd-B and colloid arrays handed to the sweeps, the
// boundary particles' rigid velocity, the per-particle pair records written
// after the density sum, the block-shared stencil-slot offsets, and the
// force epilogue (body force, store, second half kick, Oldroyd-B update).
#pragma once
#include "mcfg_internal.cuh"
#include "pair_common.cuh"
#include "sph.cuh"

namespace mcfg {

// Oldroyd-B arrays handed to the sweeps (all null for a Newtonian run).
struct NN {
  const double* ct;  // conformation tensor [d*d][n]
  double* act;       // d(ct)/dt [d*d][n]
  double* vgt;       // velocity gradient [d*d][n]
  void* qq;          // 1/n and G*ct/n^2, [1+d*d][n] in the path's type
};

// colloid arrays handed to the sweeps
struct CollArgs {
  double4_32a* v;      // state velocity (boundary particles get the rigid one)
  double4_32a* rxc;    // FP64 path: boundary particle - colloid image centre
  float4* rxcf;        // FP32 path: same
};

// particles_set_colloid_velocity.F90:73-95 with colloid_particle_velocity.F90:
// the boundary particle moves with its colloid, V + Omega x rx.  Also keeps
// rx for the no-slip pair term.  Returns the new velocity.
template <int D>
__device__ __forceinline__ double4_32a colloid_particle_update(const Consts& k, int i, int si,
                                                               const double4_32a& xi4,
                                                               const CollArgs& ca) {
  const double x[3] = {xi4.x, xi4.y, xi4.z};
  double rx[3] = {0.0, 0.0, 0.0};
  colloid_rx<D>(k, x, si - 1, rx);
  if (ca.rxc) ca.rxc[i] = make_double4_32a(rx[0], rx[1], rx[2], 0.0);
  if (ca.rxcf) ca.rxcf[i] = make_float4((float)rx[0], (float)rx[1], (float)rx[2], 0.f);
  double vn[3] = {0.0, 0.0, 0.0};
  if (k.coll_translate || k.coll_rotate) {
    const double* cd = k.coll + (size_t)(si - 1) * 12;
    vn[0] = cd[3];
    vn[1] = cd[4];
    vn[2] = D == 3 ? cd[5] : 0.0;
    if (k.coll_rotate) {
      const double r3[3] = {rx[0], rx[1], D == 3 ? rx[2] : 0.0};
      const double om[3] = {cd[6], cd[7], cd[8]};
      double w[3];
      cross3t<double>(om, r3, w);
#pragma unroll
      for (int a = 0; a < D; ++a) vn[a] += w[a];
    }
  }
  const double4_32a out = make_double4_32a(vn[0], vn[1], D == 3 ? vn[2] : 0.0, 0.0);
  ca.v[i] = out;
  return out;
}

// Per-particle prologue of the force sweep: pressure from the equation of
// state and the pair coefficients (fused into k_density or run as
// k_pressure).  The FP32 path forms them in FP32.
template <bool FP64>
__device__ __forceinline__ void write_particle_records(const Consts& k, int i, double rho, double m,
                                                       int pid, const double4_32a& v,
                                                       double* __restrict__ pr,
                                                       double4_32a* __restrict__ pc,
                                                       float4* __restrict__ pcf,
                                                       float4* __restrict__ vf, const NN& nn) {
  if (!k.newtonian) {
    // Oldroyd-B: pressure tensor (p + G) I - G c
    // (particles_compute_pressure_tensor.F90:88-133) as A = (p + G)/n^2 and
    // Q = G c / n^2, with 1/n for the velocity gradient
    const double r_eos = (k.rhs_density_type == 1) ? rho : rho * m;
    const double p = eos_pressure(k, r_eos);
    pr[i] = p;
    const double inv = 1.0 / rho;
    const double inv2 = inv * inv;
    const int n = k.n, d2 = k.d * k.d;
    if (FP64) {
      pc[i] = make_double4_32a((p + k.G) * inv2, inv2, 1.0 / m, p);
      double* q = (double*)nn.qq;
      q[i] = inv;
      for (int cc = 0; cc < d2; ++cc) q[(size_t)(1 + cc) * n + i] = k.G * nn.ct[(size_t)cc * n + i] * inv2;
    } else {
      pcf[i] = make_float4((float)((p + k.G) * inv2), (float)inv2, (float)(1.0 / m), (float)p);
      vf[i] = make_float4((float)v.x, (float)v.y, (float)v.z, __int_as_float(pid));
      float* q = (float*)nn.qq;
      q[i] = (float)inv;
      for (int cc = 0; cc < d2; ++cc)
        q[(size_t)(1 + cc) * n + i] = (float)(k.G * nn.ct[(size_t)cc * n + i] * inv2);
    }
    return;
  }
  if (FP64) {
    const double r_eos = (k.rhs_density_type == 1) ? rho : rho * m;
    const double p = eos_pressure(k, r_eos);
    pr[i] = p;
    pc[i] = pair_coeffs(k, rho, p, m);
  } else {
    const float rf = (float)rho, mf = (float)m;
    const float r_eos = (k.rhs_density_type == 1) ? rf : rf * mf;
    float p;
    if (k.eos_type == 1) {
      const float rg = (k.gamma == 1.0) ? r_eos : powf(r_eos, (float)k.gamma);
      p = (float)k.c2 * (rg - (float)k.rho_ref);
    } else {
      const float q = r_eos / (float)k.rho_ref;
      const float qg = (k.gamma == 1.0) ? q : powf(q, (float)k.gamma);
      p = (float)k.p0 * (qg - 1.0f);
    }
    pr[i] = (double)p;
    const float inv = 1.0f / rf;
    float4 cc;
    switch (k.rhs_force_type) {
      case 1: cc = make_float4(p * inv * inv, inv, mf, p); break;
      case 2: cc = make_float4(p * inv * inv, inv, 1.0f / mf, p); break;
      case 3: cc = make_float4(p * inv * inv, inv * inv, 1.0f / mf, p); break;
      default: cc = make_float4(p, inv * inv, 1.0f / mf, p); break;
    }
    pcf[i] = cc;
    vf[i] = make_float4((float)v.x, (float)v.y, (float)v.z, __int_as_float(pid));
  }
}

constexpr int kReuseTPB = 128;
// below this many particles the FP32 force sweep runs 4 lanes per particle
constexpr int64_t kSplitBelow = 50000;

// FP32 offset of each stencil slot (the neighbour cell's origin minus the
// home cell's, w = Lees-Edwards velocity jump), build_table's t.o, in a
// block-shared table of kSlotTable entries: slot s of a home cell in
// Lees-Edwards state st at st * kMaxStencil + s.  The block's first threads
// fill it, then __syncthreads.
constexpr int kSlotTable = 3 * kMaxStencil;
static_assert(kSlotTable <= kReuseTPB, "one thread per slot-table entry");
template <int D>
__device__ __forceinline__ void fill_slot_offsets(const Consts& k, float4* s_slot) {
  const int e = threadIdx.x;
  if (e < kSlotTable) s_slot[e] = slot_offset<D>(k, e % kMaxStencil, e / kMaxStencil);
}

// Physical list row of logical entry p of a list in two segments: entries
// below nff from row 0 up, the others from row cap-1 down (the FP32
// candidate and pair lists; an unsplit list has nff = its count).
__device__ __forceinline__ int cand_row(int p, int nff, int cap) {
  return p < nff ? p : cap - 1 - (p - nff);
}

// slot offsets of the Lees-Edwards row state of the home cell
__device__ __forceinline__ const float4* slot_table(const Consts& k, const float4* s_slot,
                                                   int cell) {
  if (!k.le || cell >= k.ncell) return s_slot;
  return s_slot + le_state(k, (cell / k.nm[0]) % k.nm[1]) * kMaxStencil;
}

// ---------------------------------------------------------------------------
// Epilogue shared by both force sweeps: body force, store, second half kick.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void force_epilogue(const Consts& k, int i, int si, const double* xi,
                                               double ax, double ay, double az,
                                               int fuse_mode, double dt,
                                               const double4_32a* __restrict__ v,
                                               double4_32a* __restrict__ f,
                                               double4_32a* __restrict__ v_out,
                                               unsigned* __restrict__ err) {
  if (!isfinite(ax) || !isfinite(ay) || !isfinite(az)) atomicOr(err, kErrNonFinite);
  if (fuse_mode >= kForceBody && si == 0) {
    // particles_apply_body_force.F90:96-353
    const double g[3] = {k.body_force[0], k.body_force[1], k.body_force[2]};
    if (k.body_force_type == 1) {
      if (fabs(g[0]) > k.machine_zero) ax += g[0];
      if (fabs(g[1]) > k.machine_zero) ay += g[1];
      if (D == 3 && fabs(g[2]) > k.machine_zero) az += g[2];
    } else if (k.body_force_type == 2) {
      if (fabs(g[0]) > k.machine_zero) {
        const double half = k.max_phys[D - 1] * 0.5;
        double xl = xi[D - 1];
        // positions may sit past a periodic face between list rebuilds
        if (k.periodic[D - 1]) {
          if (xl < k.min_phys[D - 1]) xl = __dadd_rn(xl, k.len[D - 1]);
          if (xl >= k.max_phys[D - 1]) xl = __dsub_rn(xl, k.len[D - 1]);
        }
        if (xl < half)
          ax += g[0];
        else if (xl > half)
          ax -= g[0];
      }
    } else if (k.body_force_type == 3) {
      if (fabs(g[0]) > k.machine_zero) {
        const double kw = 2.0 * kPi / (k.max_phys[1] - k.min_phys[1]);
        ax += g[0] * sin(kw * xi[1]);
      }
    }
  }
  f[i] = make_double4_32a(ax, ay, az, 0.0);
  if (fuse_mode == kForceBodyKick) {
    // second half kick, particles_integrate_velocity.F90:84-94
    double4_32a vv = v[i];
    if (si == 0) {
      // rounded like k_integrate and the CPU restatement: v + (0.5 a) dt, no FMA
      vv.x = __dadd_rn(vv.x, __dmul_rn(__dmul_rn(0.5, ax), dt));
      vv.y = __dadd_rn(vv.y, __dmul_rn(__dmul_rn(0.5, ay), dt));
      if (D == 3) vv.z = __dadd_rn(vv.z, __dmul_rn(__dmul_rn(0.5, az), dt));
    } else if (si < 0 && k.walls) {
      // end of the step: the face's shear velocity (moving walls)
      double vs[3] = {vv.x, vv.y, vv.z};
      wall_end_velocity<D>(k, si, vs);
      vv.x = vs[0];
      vv.y = vs[1];
      if (D == 3) vv.z = vs[2];
    }
    v_out[i] = vv;
  }
}

// Oldroyd-B per-particle update after the pair sweep: store the velocity
// gradient L, act = c L^T + L c - (c - I)/tau (particles_compute_act.F90:
// 112-156) and, inside a VV step, the second half step ct += act dt/2
// (particles_integrate_ct.F90:66-68), all in FP64.
template <int D>
__device__ __forceinline__ void nn_epilogue(const Consts& k, const NN& nn, int i, const double* L,
                                            int fuse_mode, double dt) {
  const int n = k.n;
#pragma unroll
  for (int cc = 0; cc < D * D; ++cc) nn.vgt[(size_t)cc * n + i] = L[cc];
  if (fuse_mode < kForceBody) return;
  double cm[D * D];
#pragma unroll
  for (int cc = 0; cc < D * D; ++cc) cm[cc] = nn.ct[(size_t)cc * n + i];
#pragma unroll
  for (int b = 0; b < D; ++b)
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double t = 0.0;
#pragma unroll
      for (int q = 0; q < D; ++q) t = t + cm[a + D * q] * L[b + D * q] + L[a + D * q] * cm[q + D * b];
      const double act = t - (cm[a + D * b] - (a == b ? 1.0 : 0.0)) * k.inv_tau;
      nn.act[(size_t)(a + D * b) * n + i] = act;
      if (fuse_mode == kForceBodyKick)
        ((double*)nn.ct)[(size_t)(a + D * b) * n + i] =
            __dadd_rn(cm[a + D * b], __dmul_rn(__dmul_rn(act, dt), 0.5));
    }
}


}  // namespace mcfg
