// pair_kernels.cu -- the two pair sweeps of the SDPD right-hand side.
//
// Layout: particles sorted by cell (cell_list.cu).  One warp owns one cell
// and walks its particles in chunks of 32 (lane = particle i).  The 27 (3D)
// or 9 (2D) neighbour cells are resolved once per warp into a shared-memory
// table (start, count, periodic image sign per axis).
//
// Sweep 1 (k_density): FP32 candidate test on cell offsets for every
// particle of the neighbour cells (warp-uniform broadcast loads), appending
// candidates to a per-particle neighbour list [capacity][N] of 16-bit
// entries slot<<11 | local index (coalesced across lanes).  Phase 2 walks the
// list: the FP64 path re-tests with the exact FP64 squared distance of MCF
// (so the pair set is MCF's bit for bit) and keeps only pairs inside the
// cut-off; both paths then sum W.  The epilogue evaluates the equation of
// state and writes the per-particle pair coefficients.
//
// Sweep 2 (k_force): walks the neighbour list (no candidate tests, no
// divergence beyond list-length differences) and gathers the pair
// accelerations of particle i.  Each pair is evaluated from both sides, so
// there is no scatter, no atomic and the result is deterministic; the random
// term is keyed by the unordered pid pair, so both sides draw the same dW.
//
// Reference: particles_compute_density.F90:369-867, particles_compute_
// interaction.F90:609-900, pp_interaction*.inc, rhs_force_ff_Newtonian*.F90.
#include <type_traits>

#include "mcfg_internal.cuh"
#include "sph.cuh"

namespace mcfg {

constexpr int kWarpsPerBlock = 4;

struct NbTable {
  int start[kMaxStencil];
  int count[kMaxStencil];
  int shift[kMaxStencil];  // 2 bits per axis: 0 none, 1 image at x+L, 2 at x-L
};

// cell == k.ncell is the bin of particles without a real cell: it has no
// neighbours (PPM gives such particles no box, ppm_util_rank3d.F90:463-473).
template <int D>
__device__ __forceinline__ void build_table(const Consts& k, int cell,
                                            const int* __restrict__ cell_start, NbTable& t) {
  constexpr int NS = (D == 3) ? 27 : 9;
  constexpr int CENTER = (D == 3) ? 13 : 4;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if (cell == k.ncell) {
    if (lane < NS) {
      const int s0 = cell_start[cell];
      t.start[lane] = s0;
      t.count[lane] = (lane == CENTER) ? cell_start[cell + 1] - s0 : 0;
      t.shift[lane] = 0;
    }
    __syncwarp();
    return;
  }
  if (lane < NS) {
    int c[3] = {0, 0, 0};
    int rem = cell;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      c[a] = rem % k.nm[a];
      rem /= k.nm[a];
    }
    const int o[3] = {lane % 3 - 1, (lane / 3) % 3 - 1, lane / 9 - 1};
    int nc = 0, stride = 1, sh = 0;
    bool ok = true;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      int t2 = c[a] + o[a];
      if (t2 < 0) {
        if (k.periodic[a]) {
          t2 += k.nm[a];
          sh |= 2 << (2 * a);
        } else {
          ok = false;
        }
      } else if (t2 >= k.nm[a]) {
        if (k.periodic[a]) {
          t2 -= k.nm[a];
          sh |= 1 << (2 * a);
        } else {
          ok = false;
        }
      }
      nc += t2 * stride;
      stride *= k.nm[a];
    }
    if (ok) {
      const int s0 = cell_start[nc];
      t.start[lane] = s0;
      t.count[lane] = cell_start[nc + 1] - s0;
    } else {
      t.start[lane] = 0;
      t.count[lane] = 0;
    }
    t.shift[lane] = sh;
  }
  __syncwarp();
}

// FP64 separation of MCF's pair (ip, jp) where jp may be a periodic image:
// PPM creates images only at x+L (symmetry=T), so a pair across a boundary
// is evaluated as (x_upper) - (x_lower + L) per axis.  Rounded exactly like
// rij = x(ip) - x(jp) with the ghost coordinate x + len_phys
// (ppm_bcdef_periodic_x.inc), and d2 = ((r0*r0 + r1*r1) + r2*r2) without
// fused multiply-add (pp_interaction.inc:37-50).
template <int D>
__device__ __forceinline__ double exact_sep(const Consts& k, const double* xi, const double* xj,
                                            int sh, double* r) {
  double d2 = 0.0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int s = (sh >> (2 * a)) & 3;
    double ra;
    if (s == 1)
      ra = __dsub_rn(xi[a], __dadd_rn(xj[a], k.len[a]));
    else if (s == 2)
      ra = __dsub_rn(__dadd_rn(xi[a], k.len[a]), xj[a]);
    else
      ra = __dsub_rn(xi[a], xj[a]);
    r[a] = ra;
    d2 = (a == 0) ? __dmul_rn(ra, ra) : __dadd_rn(d2, __dmul_rn(ra, ra));
  }
  return d2;
}

__device__ __forceinline__ bool dyn_rho(const Consts& k, int sid) {
  if (sid == 0) return true;
  if (sid < 0) return k.wall_rho_type == 1;
  return false;
}

// prologue shared by k_density (fused) and k_pressure
template <bool FP64>
__device__ __forceinline__ void write_particle_records(const Consts& k, int i, double rho, double m,
                                                       int sid, int pid, const double4_32a& v,
                                                       double* __restrict__ pr,
                                                       double4_32a* __restrict__ pc,
                                                       float4* __restrict__ pcf,
                                                       float4* __restrict__ vf) {
  const double r_eos = (k.rhs_density_type == 1) ? rho : rho * m;
  const double p = eos_pressure(k, r_eos);
  pr[i] = p;
  const double4_32a c = pair_coeffs(k, rho, p, m);
  if (FP64) {
    pc[i] = c;
  } else {
    pcf[i] = make_float4((float)c.x, (float)c.y, (float)c.z, (float)c.w);
    vf[i] = make_float4((float)v.x, (float)v.y, (float)v.z, __int_as_float(pid));
  }
  (void)sid;
}

template <int D, bool FP64>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_density(Consts k, const int* __restrict__ cell_start, const float4* __restrict__ off,
              const double4_32a* __restrict__ x, const double4_32a* __restrict__ v,
              const double* __restrict__ m, const int* __restrict__ sid,
              const int* __restrict__ pid, uint16_t* __restrict__ nl, int* __restrict__ ncount,
              int cap, double* __restrict__ rho, double* __restrict__ pr,
              double4_32a* __restrict__ pc, float4* __restrict__ pcf, float4* __restrict__ vf,
              int with_pressure, unsigned* __restrict__ err, int* __restrict__ stats,
              unsigned long long* __restrict__ pairs) {
  constexpr int NS = (D == 3) ? 27 : 9;
  constexpr int CENTER = (D == 3) ? 13 : 4;
  __shared__ NbTable tab[kWarpsPerBlock];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = k.n;
  int my_max = 0;
  unsigned long long my_pairs = 0;
  for (int cell = blockIdx.x * kWarpsPerBlock + wib; cell <= k.ncell;
       cell += gridDim.x * kWarpsPerBlock) {
    NbTable& t = tab[wib];
    build_table<D>(k, cell, cell_start, t);
    const int c0 = t.start[CENTER], c1 = c0 + t.count[CENTER];
    for (int base = c0; base < c1; base += 32) {
      const int i = base + lane;
      const bool active = i < c1;
      const float4 oi = active ? off[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float rlim = FP64 ? k.rc2f_hi : k.rc2f;
      int cnt = 0;
      for (int sl = 0; sl < NS; ++sl) {
        const int js = t.start[sl], jn = t.count[sl];
        const float ox = (float)(sl % 3 - 1) * k.csf[0];
        const float oy = (float)((sl / 3) % 3 - 1) * k.csf[1];
        const float oz = (D == 3) ? (float)(sl / 9 - 1) * k.csf[2] : 0.0f;
        for (int q = 0; q < jn; ++q) {
          const float4 oj = off[js + q];
          const float rx = (oi.x - oj.x) - ox;
          const float ry = (oi.y - oj.y) - oy;
          float d2 = rx * rx + ry * ry;
          if (D == 3) {
            const float rz = (oi.z - oj.z) - oz;
            d2 += rz * rz;
          }
          if (active && d2 < rlim && !(sl == CENTER && js + q == i)) {
            if (cnt < cap) nl[(size_t)cnt * n + i] = (uint16_t)((sl << kLocalBits) | q);
            ++cnt;
          }
        }
      }
      if (!active) continue;
      if (cnt > cap) {
        atomicOr(err, kErrNeighOverflow);
        my_max = max(my_max, cnt);
        cnt = cap;
      }
      // phase 2: exact test (FP64) and the density sum
      const int si = sid[i];
      const bool acc_i = dyn_rho(k, si);
      double rho_i;
      int kept = 0;
      if (FP64) {
        const double4_32a xi4 = x[i];
        const double xi[3] = {xi4.x, xi4.y, xi4.z};
        double sum = 0.0;
        for (int e = 0; e < cnt; ++e) {
          const int ent = nl[(size_t)e * n + i];
          const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
          const int j = t.start[sl] + q;
          const double4_32a xj4 = x[j];
          const double xj[3] = {xj4.x, xj4.y, xj4.z};
          double r[3];
          const double d2 = exact_sep<D>(k, xi, xj, t.shift[sl], r);
          if (d2 >= k.rc2) continue;
          nl[(size_t)kept * n + i] = (uint16_t)ent;
          ++kept;
          if (acc_i) {
            const double w = kernel_w<double>(k, sqrt(d2));
            sum += (k.rhs_density_type == 1) ? w * m[j] : w;
          }
        }
        rho_i = sum;
      } else {
        // Kahan-compensated FP32 sum of W
        float sum = 0.0f, comp = 0.0f;
        for (int e = 0; e < cnt; ++e) {
          const int ent = nl[(size_t)e * n + i];
          const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
          const int j = t.start[sl] + q;
          if (acc_i) {
            const float4 oj = off[j];
            const float rx = (oi.x - oj.x) - (float)(sl % 3 - 1) * k.csf[0];
            const float ry = (oi.y - oj.y) - (float)((sl / 3) % 3 - 1) * k.csf[1];
            float d2 = rx * rx + ry * ry;
            if (D == 3) {
              const float rz = (oi.z - oj.z) - (float)(sl / 9 - 1) * k.csf[2];
              d2 += rz * rz;
            }
            float w = kernel_w<float>(k, sqrtf(d2));
            if (k.rhs_density_type == 1) w *= (float)m[j];
            const float y = w - comp;
            const float tt = sum + y;
            comp = (tt - sum) - y;
            sum = tt;
          }
        }
        kept = cnt;
        rho_i = (double)sum;
      }
      ncount[i] = kept;
      my_max = max(my_max, kept);
      my_pairs += (unsigned long long)kept;
      const double mi = m[i];
      double rho_out;
      if (acc_i) {
        rho_out = ((k.rhs_density_type == 1) ? k.w0 * mi : k.w0) + rho_i;
      } else {
        rho_out = (k.rhs_density_type == 1) ? k.init_density : k.init_density / mi;
      }
      rho[i] = rho_out;
      if (!(rho_out > 0.0)) atomicOr(err, kErrZeroDensity);
      if (with_pressure)
        write_particle_records<FP64>(k, i, rho_out, mi, si, pid[i], v[i], pr, pc, pcf, vf);
    }
  }
  // warp reductions of the counters
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    my_max = max(my_max, __shfl_xor_sync(0xffffffffu, my_max, o));
    my_pairs += __shfl_xor_sync(0xffffffffu, my_pairs, o);
  }
  if (lane == 0) {
    atomicMax(&stats[1], my_max);
    atomicAdd(pairs, my_pairs);
  }
}

template <bool FP64>
__global__ void k_pressure(Consts k, const double* __restrict__ rho, const double* __restrict__ m,
                           const int* __restrict__ sid, const int* __restrict__ pid,
                           const double4_32a* __restrict__ v, double* __restrict__ pr,
                           double4_32a* __restrict__ pc, float4* __restrict__ pcf,
                           float4* __restrict__ vf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  write_particle_records<FP64>(k, i, rho[i], m[i], sid[i], pid[i], v[i], pr, pc, pcf, vf);
}

// ---------------------------------------------------------------------------
// Force sweep
// ---------------------------------------------------------------------------
template <int D, bool FP64>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_force(Consts k, const int* __restrict__ cell_start, const uint16_t* __restrict__ nl,
            const int* __restrict__ ncount, const float4* __restrict__ off,
            const double4_32a* __restrict__ x, const double4_32a* __restrict__ v,
            const double4_32a* __restrict__ pc, const float4* __restrict__ pcf,
            const float4* __restrict__ vf, const int* __restrict__ sid,
            const int* __restrict__ pid, double4_32a* __restrict__ f, double* __restrict__ st,
            int fuse_mode, double dt, double4_32a* __restrict__ v_out, uint32_t step,
            double inv_sqdt, unsigned* __restrict__ err) {
  constexpr int CENTER = (D == 3) ? 13 : 4;
  using T = typename std::conditional<FP64, double, float>::type;
  __shared__ NbTable tab[kWarpsPerBlock];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = k.n;
  const bool noise = k.noise != 0;
  const T isq = (T)inv_sqdt;
  for (int cell = blockIdx.x * kWarpsPerBlock + wib; cell <= k.ncell;
       cell += gridDim.x * kWarpsPerBlock) {
    NbTable& t = tab[wib];
    build_table<D>(k, cell, cell_start, t);
    const int c0 = t.start[CENTER], c1 = c0 + t.count[CENTER];
    for (int base = c0; base < c1; base += 32) {
      const int i = base + lane;
      if (i >= c1) continue;
      const int si = sid[i];
      const int pidi = pid[i];
      T ri[3], vi[3];
      T Ai, Bi, Ci, Pi;
      const double4_32a xi4 = x[i];
      const double xi[3] = {xi4.x, xi4.y, xi4.z};
      if (FP64) {
        const double4_32a v4 = v[i];
        vi[0] = (T)v4.x; vi[1] = (T)v4.y; vi[2] = (T)v4.z;
        const double4_32a c = pc[i];
        Ai = (T)c.x; Bi = (T)c.y; Ci = (T)c.z; Pi = (T)c.w;
      } else {
        const float4 o = off[i];
        ri[0] = (T)o.x; ri[1] = (T)o.y; ri[2] = (T)o.z;
        const float4 v4 = vf[i];
        vi[0] = (T)v4.x; vi[1] = (T)v4.y; vi[2] = (T)v4.z;
        const float4 c = pcf[i];
        Ai = (T)c.x; Bi = (T)c.y; Ci = (T)c.z; Pi = (T)c.w;
      }
      T acc[3] = {T(0), T(0), T(0)};
      T comp[3] = {T(0), T(0), T(0)};  // Kahan terms (FP32 path)
      T sacc[9];
#pragma unroll
      for (int a = 0; a < 9; ++a) sacc[a] = T(0);
      const int cnt = ncount[i];
      for (int e = 0; e < cnt; ++e) {
        const int ent = nl[(size_t)e * n + i];
        const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
        const int j = t.start[sl] + q;
        T r[3], vj[3];
        T Aj, Bj, Cj, Pj;
        T d;
        int sj, pidj = 0;
        if (FP64) {
          sj = sid[j];
          if (si != 0 && sj != 0) continue;  // w-w, c-c, c-w: no interaction here
          const double4_32a xj4 = x[j];
          const double xj[3] = {xj4.x, xj4.y, xj4.z};
          double rr[3];
          const double d2 = exact_sep<D>(k, xi, xj, t.shift[sl], rr);
#pragma unroll
          for (int a = 0; a < D; ++a) r[a] = (T)rr[a];
          d = (T)sqrt(d2);
          const double4_32a v4 = v[j];
          vj[0] = (T)v4.x; vj[1] = (T)v4.y; vj[2] = (T)v4.z;
          const double4_32a c = pc[j];
          Aj = (T)c.x; Bj = (T)c.y; Cj = (T)c.z; Pj = (T)c.w;
          if (noise) pidj = pid[j];
        } else {
          const float4 oj = off[j];
          sj = __float_as_int(oj.w);
          if (si != 0 && sj != 0) continue;
          r[0] = (ri[0] - (T)oj.x) - (T)(sl % 3 - 1) * (T)k.csf[0];
          r[1] = (ri[1] - (T)oj.y) - (T)((sl / 3) % 3 - 1) * (T)k.csf[1];
          r[2] = (D == 3) ? (ri[2] - (T)oj.z) - (T)(sl / 9 - 1) * (T)k.csf[2] : T(0);
          T d2 = r[0] * r[0] + r[1] * r[1];
          if (D == 3) d2 += r[2] * r[2];
          d = my_sqrt<T>(d2);
          const float4 v4 = vf[j];
          vj[0] = (T)v4.x; vj[1] = (T)v4.y; vj[2] = (T)v4.z;
          pidj = __float_as_int(v4.w);
          const float4 c = pcf[j];
          Aj = (T)c.x; Bj = (T)c.y; Cj = (T)c.z; Pj = (T)c.w;
        }
        T vi_save[3] = {vi[0], vi[1], vi[2]};
        T Ai_save = Ai;
        if (si < 0 || sj < 0) {
          // fluid-wall pair: the wall particle takes the Morris no-slip
          // velocity and the fluid particle's pressure
          // (pp_interaction_fw.inc, pp_interaction_wf.inc)
          const int sw = (sj < 0) ? sj : si;
          const int axis = (-sw - 1) >> 1;
          const double4_32a xj4 = x[j];
          const double xjn = axis == 0 ? xj4.x : axis == 1 ? xj4.y : xj4.z;
          const double xin = axis == 0 ? xi[0] : axis == 1 ? xi[1] : xi[2];
          T vw[3];
          int ax_unused;
          if (sj < 0) {
            wall_noslip<T, D>(k, xin, xjn, vi, sj, vw, ax_unused);
#pragma unroll
            for (int a = 0; a < D; ++a) vj[a] = vw[a];
            Aj = boundary_A<T>(k.rhs_force_type, Pi, Bj);
          } else {
            wall_noslip<T, D>(k, xjn, xin, vj, si, vw, ax_unused);
#pragma unroll
            for (int a = 0; a < D; ++a) vi[a] = vw[a];
            Ai = boundary_A<T>(k.rhs_force_type, Pj, Bi);
          }
        }
        const T gw = kernel_gradw<T>(k, d);
        T vij[3];
#pragma unroll
        for (int a = 0; a < D; ++a) vij[a] = vi[a] - vj[a];
        float z[6];
        if (noise) pair_normals<D>(k.key0, k.key1, step, pidi, pidj, z);
        T pa[3];
        pair_accel<T, D>(k, r, d, vij, Ai, Bi, Ci, Aj, Bj, Cj, gw, noise, z, isq, pa);
        vi[0] = vi_save[0]; vi[1] = vi_save[1]; vi[2] = vi_save[2];
        Ai = Ai_save;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          if (FP64) {
            acc[a] += pa[a];
          } else {
            const T y = pa[a] - comp[a];
            const T tt = acc[a] + y;
            comp[a] = (tt - acc[a]) - y;
            acc[a] = tt;
          }
        }
        if (k.stress) {
          // pp_interaction_ff.inc:83-93: s_ab += r_a * f_b / 2
#pragma unroll
          for (int b = 0; b < D; ++b)
#pragma unroll
            for (int a = 0; a < D; ++a) sacc[b * D + a] += r[a] * pa[b] * T(0.5);
        }
      }
      double ax = (double)acc[0], ay = (double)acc[1], az = (D == 3) ? (double)acc[2] : 0.0;
      if (!isfinite(ax) || !isfinite(ay) || !isfinite(az)) atomicOr(err, kErrNonFinite);
      if (fuse_mode >= kForceBody && si == 0) {
        // particles_apply_body_force.F90:96-353
        const double* g = k.body_force;
        if (k.body_force_type == 1) {
          if (fabs(g[0]) > k.machine_zero) ax += g[0];
          if (fabs(g[1]) > k.machine_zero) ay += g[1];
          if (D == 3 && fabs(g[2]) > k.machine_zero) az += g[2];
        } else if (k.body_force_type == 2) {
          if (fabs(g[0]) > k.machine_zero) {
            const double half = k.max_phys[D - 1] * 0.5;
            const double xl = xi[D - 1];
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
      if (k.stress) {
#pragma unroll
        for (int a = 0; a < D * D; ++a) st[(size_t)a * n + i] = (double)sacc[a];
      }
      if (fuse_mode == kForceBodyKick) {
        // second half kick, particles_integrate_velocity.F90:84-94
        double4_32a vv = v[i];
        if (si == 0) {
          vv.x = vv.x + 0.5 * ax * dt;
          vv.y = vv.y + 0.5 * ay * dt;
          if (D == 3) vv.z = vv.z + 0.5 * az * dt;
        }
        v_out[i] = vv;
      }
    }
  }
}

static int grid_for(Handle* h) {
  const int warps = h->k.ncell + 1;  // + bin of particles without a cell
  int g = (warps + kWarpsPerBlock - 1) / kWarpsPerBlock;
  return g < 1 ? 1 : g;
}

int compute_density(Handle* h, bool with_pressure) {
  Consts& k = h->k;
  cudaStream_t s = h->stream;
  if (cuda_check(h, cudaMemsetAsync(h->d_stats, 0, sizeof(int) * 4, s), "memset stats"))
    return MCFG_ECUDA;
  if (cuda_check(h, cudaMemsetAsync(h->d_pairs, 0, sizeof(unsigned long long), s), "memset pairs"))
    return MCFG_ECUDA;
  const int g = grid_for(h);
  const bool fp64 = h->p.precision == MCFG_PRECISION_FP64;
#define LAUNCH_D(DD, PP)                                                                       \
  k_density<DD, PP><<<g, kWarpsPerBlock * 32, 0, s>>>(                                          \
      k, h->cell_start, h->off, h->x, h->v, h->m, h->sid, h->pid, h->nl, h->ncount,            \
      h->neigh_cap, h->rho, h->pr, h->pc, h->pcf, h->vf, with_pressure ? 1 : 0, h->d_err,      \
      h->d_stats, h->d_pairs)
  if (k.d == 3) {
    if (fp64) LAUNCH_D(3, true); else LAUNCH_D(3, false);
  } else {
    if (fp64) LAUNCH_D(2, true); else LAUNCH_D(2, false);
  }
#undef LAUNCH_D
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "density launch")) return MCFG_ECUDA;
  return MCFG_OK;
}

int compute_pressure(Handle* h) {
  const int n = (int)h->n;
  if (n == 0) return MCFG_OK;
  const int tb = 256, gb = (n + tb - 1) / tb;
  if (h->p.precision == MCFG_PRECISION_FP64)
    k_pressure<true><<<gb, tb, 0, h->stream>>>(h->k, h->rho, h->m, h->sid, h->pid, h->v, h->pr,
                                               h->pc, h->pcf, h->vf);
  else
    k_pressure<false><<<gb, tb, 0, h->stream>>>(h->k, h->rho, h->m, h->sid, h->pid, h->v, h->pr,
                                                h->pc, h->pcf, h->vf);
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "pressure launch")) return MCFG_ECUDA;
  return MCFG_OK;
}

int compute_force(Handle* h, int64_t step, int fuse_mode, double dt) {
  Consts& k = h->k;
  cudaStream_t s = h->stream;
  const int g = grid_for(h);
  const bool fp64 = h->p.precision == MCFG_PRECISION_FP64;
  const double inv_sqdt = (k.noise && dt > 0.0) ? 1.0 / sqrt(dt) : 0.0;
  if (k.noise && !(dt > 0.0)) return set_error(h, MCFG_EINVAL, "random force needs dt > 0");
#define LAUNCH_F(DD, PP)                                                                       \
  k_force<DD, PP><<<g, kWarpsPerBlock * 32, 0, s>>>(                                            \
      k, h->cell_start, h->nl, h->ncount, h->off, h->x, h->v, h->pc, h->pcf, h->vf, h->sid,     \
      h->pid, h->f, h->st, fuse_mode, dt, h->v2, (uint32_t)step, inv_sqdt, h->d_err)
  if (k.d == 3) {
    if (fp64) LAUNCH_F(3, true); else LAUNCH_F(3, false);
  } else {
    if (fp64) LAUNCH_F(2, true); else LAUNCH_F(2, false);
  }
#undef LAUNCH_F
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "force launch")) return MCFG_ECUDA;
  if (fuse_mode == kForceBodyKick) std::swap(h->v, h->v2);
  return MCFG_OK;
}

}  // namespace mcfg
