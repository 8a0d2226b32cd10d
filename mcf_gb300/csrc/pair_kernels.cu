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
#include <algorithm>
#include <type_traits>

#include "mcfg_internal.cuh"
#include "pair_common.cuh"
#include "sph.cuh"
#include "sweep_common.cuh"

namespace mcfg {

constexpr int kStage = 64;      // neighbour-cell offsets staged per pass
constexpr int kListStage = 96;  // neighbour entries staged in shared memory per lane

template <int D, bool FP64>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_density(Consts k, const int* __restrict__ cell_start, const float4* __restrict__ off,
              const double4_32a* __restrict__ x, const double4_32a* __restrict__ v,
              const double* __restrict__ m, const int* __restrict__ sid,
              const int* __restrict__ pid, uint16_t* __restrict__ nl, int* __restrict__ ncount,
              int* __restrict__ nhs, int cap, double* __restrict__ rho, double* __restrict__ pr,
              double4_32a* __restrict__ pc, float4* __restrict__ pcf, float4* __restrict__ vf,
              int with_pressure, unsigned* __restrict__ err, int* __restrict__ stats,
              unsigned long long* __restrict__ pairs, NN nn, CollArgs ca) {
  constexpr int CENTER = (D == 3) ? 13 : 4;
  __shared__ NbTable tab[kWarpsPerBlock];
  __shared__ float4 sb[kWarpsPerBlock][kStage];
  __shared__ uint16_t ls[kWarpsPerBlock][kListStage][32];
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
      // phase 1: candidate scan, offsets of each neighbour cell staged in
      // shared memory by coalesced loads, then broadcast to the lanes
      for (int sl = 0; sl < k.ns; ++sl) {
        const int js = t.start[sl], jn = t.count[sl];
        const float4 so = t.o[sl];
        const float px = oi.x - so.x, py = oi.y - so.y, pz = oi.z - so.z;
        for (int b2 = 0; b2 < jn; b2 += kStage) {
          const int mm = min(kStage, jn - b2);
          __syncwarp();
          for (int q = lane; q < mm; q += 32) sb[wib][q] = off[js + b2 + q];
          __syncwarp();
#pragma unroll 4
          for (int q2 = 0; q2 < mm; ++q2) {
            const float4 oj = sb[wib][q2];
            const float rx = px - oj.x, ry = py - oj.y;
            float d2 = rx * rx + ry * ry;
            if (D == 3) {
              const float rz = pz - oj.z;
              d2 += rz * rz;
            }
            const int q = b2 + q2;
            if (active && d2 < rlim && !(sl == CENTER && js + q == i)) {
              const uint16_t ent = (uint16_t)((sl << kLocalBits) | q);
              if (cnt < kListStage)
                ls[wib][cnt][lane] = ent;
              else if (cnt < cap)
                nl[(size_t)cnt * n + i] = ent;
              ++cnt;
            }
          }
        }
      }
      if (active && cnt > cap) {
        atomicOr(err, kErrNeighOverflow);
        my_max = max(my_max, cnt);
      }
      cnt = min(cnt, cap);
      // phase 2: exact test (FP64 path), density sum, final list rows
      const int si = active ? sid[i] : 0;
      const bool acc_i = dyn_rho(k, si);
      const int li = i - c0;  // local index in the cell
      double rho_i = 0.0;
      int kept = 0;
      int hs = -1;  // first entry of the forward half (pairs this particle owns)
      if (FP64) {
        double4_32a xi4 = active ? x[i] : make_double4_32a(0, 0, 0, 0);
        const double xi[3] = {xi4.x, xi4.y, xi4.z};
        double sum = 0.0;
        for (int e = 0; e < cnt; ++e) {
          const int ent = (e < kListStage) ? ls[wib][e][lane] : nl[(size_t)e * n + i];
          const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
          const int j = t.start[sl] + q;
          const double4_32a xj4 = x[j];
          const double xj[3] = {xj4.x, xj4.y, xj4.z};
          double r[3];
          const double d2 = exact_sep<D>(k, xi, xj, t.shift[sl], r);
          if (d2 >= k.rc2) continue;
          if (hs < 0 && (sl > CENTER || (sl == CENTER && q > li))) hs = kept;
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
        const bool mass = k.rhs_density_type == 1;
        for (int e = 0; e < cnt; ++e) {
          const int ent = (e < kListStage) ? ls[wib][e][lane] : nl[(size_t)e * n + i];
          if (e < kListStage) nl[(size_t)e * n + i] = (uint16_t)ent;
          const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
          if (hs < 0 && (sl > CENTER || (sl == CENTER && q > li))) hs = e;
          if (!acc_i) continue;
          const int j = t.start[sl] + q;
          const float4 oj = off[j];
          const float4 so = t.o[sl];
          const float rx = (oi.x - oj.x) - so.x;
          const float ry = (oi.y - oj.y) - so.y;
          float d2 = rx * rx + ry * ry;
          if (D == 3) {
            const float rz = (oi.z - oj.z) - so.z;
            d2 += rz * rz;
          }
          float w = kernel_w<float>(k, sqrtf(d2));
          if (mass) w *= (float)m[j];
          const float y = w - comp;
          const float tt = sum + y;
          comp = (tt - sum) - y;
          sum = tt;
        }
        kept = cnt;
        rho_i = (double)sum;
      }
      if (!active) continue;
      ncount[i] = kept;
      nhs[i] = (hs < 0) ? kept : hs;
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
      if (with_pressure) {
        const double4_32a vi4 =
            (si > 0 && k.ncoll > 0) ? colloid_particle_update<D>(k, i, si, x[i], ca) : v[i];
        write_particle_records<FP64>(k, i, rho_out, mi, pid[i], vi4, pr, pc, pcf, vf, nn);
      }
    }
  }
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

// ---------------------------------------------------------------------------
// List-reuse mode: the candidate list (gated rebuild) and the density sweep
// over it.
// ---------------------------------------------------------------------------

// Candidates within rc + skin of every particle: k_density's FP32 scan of
// the 27/9 neighbour cells with the larger bound, written to vl.  Returns at
// once unless a rebuild is due.
template <int D>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_verlet_build(Consts k, const int* __restrict__ gate, const int* __restrict__ cell_start,
                   const float4* __restrict__ off, uint16_t* __restrict__ vl,
                   int* __restrict__ vcount, int vcap, int partition,
                   unsigned* __restrict__ err) {
  if (*gate == 0) return;
  constexpr int CENTER = (D == 3) ? 13 : 4;
  __shared__ NbTable tab[kWarpsPerBlock];
  __shared__ float4 sb[kWarpsPerBlock][kStage];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = k.n;
  for (int cell = blockIdx.x * kWarpsPerBlock + wib; cell <= k.ncell;
       cell += gridDim.x * kWarpsPerBlock) {
    NbTable& t = tab[wib];
    build_table<D>(k, cell, cell_start, t);
    const int c0 = t.start[CENTER], c1 = c0 + t.count[CENTER];
    for (int base = c0; base < c1; base += 32) {
      const int i = base + lane;
      const bool active = i < c1;
      const float4 oi = active ? off[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      const bool fluid_i = __float_as_int(oi.w) == 0;
      int cnt = 0, cnt_o = 0;  // cnt_o: partitioned lists' second segment
      for (int sl = 0; sl < k.ns; ++sl) {
        const int js = t.start[sl], jn = t.count[sl];
        const float4 so = t.o[sl];
        const float px = oi.x - so.x, py = oi.y - so.y, pz = oi.z - so.z;
        for (int b2 = 0; b2 < jn; b2 += kStage) {
          const int mm = min(kStage, jn - b2);
          __syncwarp();
          for (int q = lane; q < mm; q += 32) sb[wib][q] = off[js + b2 + q];
          __syncwarp();
#pragma unroll 4
          for (int q2 = 0; q2 < mm; ++q2) {
            const float4 oj = sb[wib][q2];
            const float rx = px - oj.x, ry = py - oj.y;
            float d2 = rx * rx + ry * ry;
            if (D == 3) {
              const float rz = pz - oj.z;
              d2 += rz * rz;
            }
            const int q = b2 + q2;
            if (active && d2 < k.rv2f && !(sl == CENTER && js + q == i)) {
              const uint16_t ent = (uint16_t)((sl << kLocalBits) | q);
              if (partition && !(fluid_i && __float_as_int(oj.w) == 0)) {
                // FP32 lists: pairs with a boundary particle from the last row down
                if (cnt + cnt_o < vcap) vl[(size_t)(vcap - 1 - cnt_o) * n + i] = ent;
                ++cnt_o;
              } else {
                if (cnt + cnt_o < vcap) vl[(size_t)cnt * n + i] = ent;
                ++cnt;
              }
            }
          }
        }
      }
      if (active) {
        if (cnt + cnt_o > vcap) {
          atomicOr(err, kErrNeighOverflow);
          cnt = min(cnt, vcap);
          cnt_o = min(cnt_o, vcap - cnt);
        }
        // partitioned: fluid-fluid count | other count << 16
        vcount[i] = partition ? (cnt | (cnt_o << 16)) : cnt;
      }
    }
  }
}

// end of a gated rebuild: count it and lower the flag
__global__ void k_rebuild_done(int* __restrict__ flag) {
  if (flag[0] != 0) flag[1] += 1;
  flag[0] = 0;
}

// FP64 density over the candidate list, one thread per particle: the step's
// exact pair test with MCF's FP64 separation, the step's neighbour list for
// the force sweeps (nhs: the first entry of the forward half the symmetric
// sweep owns), the W sum and the epilogue of k_density.  The FP32 path runs
// k_density_list (sweep32.cu).
template <int D>
__global__ void __launch_bounds__(kReuseTPB)
    k_density_reuse(Consts k, const int* __restrict__ cell_start, const int* __restrict__ cell_of,
                    const double4_32a* __restrict__ x, const double4_32a* __restrict__ v,
                    const double* __restrict__ m, const int* __restrict__ sid,
                    const int* __restrict__ pid, const uint16_t* __restrict__ vl,
                    const int* __restrict__ vcount, uint16_t* __restrict__ nl,
                    int* __restrict__ ncount, int* __restrict__ nhs, int cap,
                    double* __restrict__ rho, double* __restrict__ pr,
                    double4_32a* __restrict__ pc, float4* __restrict__ pcf,
                    float4* __restrict__ vf, int with_pressure, unsigned* __restrict__ err,
                    int* __restrict__ stats, unsigned long long* __restrict__ pairs, NN nn,
                    CollArgs ca) {
  constexpr int CENTER = (D == 3) ? 13 : 4;
  __shared__ int s_start[kMaxStencil * kReuseTPB];
  __shared__ int s_shift[kMaxStencil * kReuseTPB];
  const int n = k.n, tid = threadIdx.x;
  const int i = blockIdx.x * kReuseTPB + tid;
  int my_max = 0;
  unsigned long long my_pairs = 0;
  if (i < n) {
    const int celli = cell_of[i];
    build_lane_table<D, kReuseTPB>(k, celli, cell_start, s_start, s_shift);
    const int li = i - s_start[CENTER * kReuseTPB + tid];
    const int si = sid[i];
    const bool acc_i = dyn_rho(k, si);
    const int cnt = vcount[i];
    const double4_32a xi4 = x[i];
    const double xi[3] = {xi4.x, xi4.y, xi4.z};
    double sum = 0.0;
    int kept = 0, hs = -1;
    for (int e = 0; e < cnt; ++e) {
      const int ent = vl[(size_t)e * n + i];
      const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
      const int j = s_start[sl * kReuseTPB + tid] + q;
      const double4_32a xj4 = x[j];
      const double xj[3] = {xj4.x, xj4.y, xj4.z};
      double r[3];
      const double d2 = exact_sep<D>(k, xi, xj, s_shift[sl * kReuseTPB + tid], r);
      if (d2 >= k.rc2) continue;
      if (hs < 0 && (sl > CENTER || (sl == CENTER && q > li))) hs = kept;
      if (kept < cap) nl[(size_t)kept * n + i] = (uint16_t)ent;
      ++kept;
      if (acc_i) {
        const double w = kernel_w<double>(k, sqrt(d2));
        sum += (k.rhs_density_type == 1) ? w * m[j] : w;
      }
    }
    if (kept > cap) atomicOr(err, kErrNeighOverflow);
    my_max = kept;
    kept = min(kept, cap);
    ncount[i] = kept;
    nhs[i] = (hs < 0 || hs > kept) ? kept : hs;
    my_pairs = (unsigned long long)kept;
    const double mi = m[i];
    double rho_out;
    if (acc_i) {
      rho_out = ((k.rhs_density_type == 1) ? k.w0 * mi : k.w0) + sum;
    } else {
      rho_out = (k.rhs_density_type == 1) ? k.init_density : k.init_density / mi;
    }
    rho[i] = rho_out;
    if (!(rho_out > 0.0)) atomicOr(err, kErrZeroDensity);
    if (with_pressure) {
      const double4_32a vi4 =
          (si > 0 && k.ncoll > 0) ? colloid_particle_update<D>(k, i, si, x[i], ca) : v[i];
      write_particle_records<true>(k, i, rho_out, mi, pid[i], vi4, pr, pc, pcf, vf, nn);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    my_max = max(my_max, __shfl_xor_sync(0xffffffffu, my_max, o));
    my_pairs += __shfl_xor_sync(0xffffffffu, my_pairs, o);
  }
  if ((tid & 31) == 0) {
    atomicMax(&stats[1], my_max);
    atomicAdd(pairs, my_pairs);
  }
}

template <int D, bool FP64>
__global__ void k_pressure(Consts k, const double* __restrict__ rho, const double* __restrict__ m,
                           const int* __restrict__ pid, const double4_32a* __restrict__ v,
                           double* __restrict__ pr, double4_32a* __restrict__ pc,
                           float4* __restrict__ pcf, float4* __restrict__ vf, NN nn,
                           const int* __restrict__ sid, const double4_32a* __restrict__ x,
                           CollArgs ca) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  const int si = sid[i];
  const double4_32a vi4 =
      (si > 0 && k.ncoll > 0) ? colloid_particle_update<D>(k, i, si, x[i], ca) : v[i];
  write_particle_records<FP64>(k, i, rho[i], m[i], pid[i], vi4, pr, pc, pcf, vf, nn);
}

// ---------------------------------------------------------------------------
// FP64 force sweep
// ---------------------------------------------------------------------------
template <int D, bool NNW>
__global__ void __launch_bounds__(kReuseTPB)
    k_force64(Consts k, const int* __restrict__ cell_start, const int* __restrict__ cell_of,
              const uint16_t* __restrict__ nl,
              const int* __restrict__ ncount, const double4_32a* __restrict__ x,
              const double4_32a* __restrict__ v, const double4_32a* __restrict__ pc,
              const int* __restrict__ sid, const int* __restrict__ pid,
              double4_32a* __restrict__ f, double* __restrict__ st, int fuse_mode, double dt,
              double4_32a* __restrict__ v_out, uint32_t step_arg,
              const int64_t* __restrict__ step_ptr, double inv_sqdt,
              unsigned* __restrict__ err, NN nn, CollArgs ca) {
  constexpr int D2 = D * D;
  using T = double;
  // the Philox counter's step: the argument, or the device step counter
  // when the sweep runs inside a captured graph
  const uint32_t step = step_ptr ? (uint32_t)*step_ptr : step_arg;
  __shared__ int s_start[kMaxStencil * kReuseTPB];
  __shared__ int s_shift[kMaxStencil * kReuseTPB];
  const int n = k.n;
  const bool noise = k.noise != 0;
  const int i = blockIdx.x * kReuseTPB + threadIdx.x;
  if (i >= n) return;
  build_lane_table<D, kReuseTPB>(k, cell_of[i], cell_start, s_start, s_shift);
  const int si = sid[i];
  const int pidi = pid[i];
  const double4_32a xi4 = x[i];
  const double xi[3] = {xi4.x, xi4.y, xi4.z};
  const double4_32a v4i = v[i];
  const double4_32a ci = pc[i];
  constexpr bool nnw = NNW;  // Oldroyd-B terms compiled only when used
  const double* qq = (const double*)nn.qq;
  T qi[1 + D2], L[D2];
#pragma unroll
  for (int cc = 0; cc < D2; ++cc) L[cc] = 0;
  if (nnw) {
#pragma unroll
    for (int cc = 0; cc <= D2; ++cc) qi[cc] = qq[(size_t)cc * n + i];
  }
  T acc[3] = {0, 0, 0};
  T sacc[9];
#pragma unroll
  for (int a = 0; a < 9; ++a) sacc[a] = 0;
  const int cnt = ncount[i];
  for (int e = 0; e < cnt; ++e) {
    const int ent = nl[(size_t)e * n + i];
    const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
    const int j = s_start[sl * kReuseTPB + threadIdx.x] + q;
    const int sj = sid[j];
    // pp_interaction.inc:63-223: w-w and c-w never interact, c-c only
    // between different colloids with pp_interact_cc
    if (si != 0 && sj != 0 && !(si > 0 && sj > 0 && si != sj && k.pp_cc)) continue;
    const double4_32a xj4 = x[j];
    const double xj[3] = {xj4.x, xj4.y, xj4.z};
    T r[3];
    const int shj = s_shift[sl * kReuseTPB + threadIdx.x];
    const double d2 = exact_sep<D>(k, xi, xj, shj, r);
    // the kernel's argument is MCF's SQRT(DOT_PRODUCT(rij, rij)), correctly
    // rounded: near the cut-off W'(d) ~ (3 - d/h)^4 amplifies any rounding
    // difference of d by 4 d / (3h - d); 1/d only scales well-conditioned terms
    const T inv_d = rsqrt(d2);
    const T d = sqrt(d2);
    const double4_32a v4 = v[j];
    T vi[3] = {v4i.x, v4i.y, v4i.z};
    T vj[3] = {v4.x, v4.y, v4.z};
    if (shj >= kLeUp) le_velocity<T>(k, shj, vi, vj);
    const double4_32a cj = pc[j];
    T Ai = ci.x, Aj = cj.x, Bi = ci.y, Bj = cj.y;
    T qj[1 + D2], qie[1 + D2];
    if (nnw) {
#pragma unroll
      for (int cc = 0; cc <= D2; ++cc) {
        qj[cc] = qq[(size_t)cc * n + j];
        qie[cc] = qi[cc];
      }
    }
    if (si < 0 || sj < 0) {
      // fluid-wall pair: wall particle takes the Morris no-slip velocity
      // and the fluid pressure (pp_interaction_fw.inc / _wf.inc); in the
      // Oldroyd-B model also the fluid density and pressure tensor
      const int sw = (sj < 0) ? sj : si;
      const int axis = (-sw - 1) >> 1;
      const double xin = axis == 0 ? xi[0] : axis == 1 ? xi[1] : xi[2];
      const double xjn = axis == 0 ? xj[0] : axis == 1 ? xj[1] : xj[2];
      T vw[3];
      if (sj < 0) {
        wall_noslip<T, D>(k, xin, xjn, vi, sj, vw);
#pragma unroll
        for (int a = 0; a < D; ++a) vj[a] = vw[a];
        if (nnw) {
          Aj = Ai;
          Bj = Bi;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qj[cc] = qi[cc];
        } else {
          Aj = boundary_A<T>(k.rhs_force_type, ci.w, cj.y);
        }
      } else {
        wall_noslip<T, D>(k, xjn, xin, vj, si, vw);
#pragma unroll
        for (int a = 0; a < D; ++a) vi[a] = vw[a];
        if (nnw) {
          Ai = Aj;
          Bi = Bj;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qie[cc] = qj[cc];
        } else {
          Ai = boundary_A<T>(k.rhs_force_type, cj.w, ci.y);
        }
      }
    } else if ((si > 0) != (sj > 0)) {
      // fluid-colloid pair (pp_interaction_fc.inc / _cf.inc): the
      // boundary particle takes the Morris no-slip velocity and the
      // fluid pressure (Oldroyd-B: also its density and pressure tensor)
      if (sj > 0) {
        if (k.coll_noslip == 2) {
          const double4_32a rc4 = ca.rxc[j];
          const T rxc_[3] = {rc4.x, rc4.y, rc4.z};
          T vw[3];
          colloid_noslip<T, D>(k, sj - 1, rxc_, r, vi, vw);
#pragma unroll
          for (int a = 0; a < D; ++a) vj[a] = vw[a];
        }
        if (nnw) {
          Aj = Ai;
          Bj = Bi;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qj[cc] = qi[cc];
        } else {
          Aj = boundary_A<T>(k.rhs_force_type, ci.w, cj.y);
        }
      } else {
        if (k.coll_noslip == 2) {
          const double4_32a rc4 = ca.rxc[i];
          const T rxc_[3] = {rc4.x, rc4.y, rc4.z};
          const T rfc[3] = {-r[0], -r[1], -r[2]};
          T vw[3];
          colloid_noslip<T, D>(k, si - 1, rxc_, rfc, vj, vw);
#pragma unroll
          for (int a = 0; a < D; ++a) vi[a] = vw[a];
        }
        if (nnw) {
          Ai = Aj;
          Bi = Bj;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qie[cc] = qj[cc];
        } else {
          Ai = boundary_A<T>(k.rhs_force_type, cj.w, ci.y);
        }
      }
    }
    const T gw = kernel_gradw<T>(k, d);
    T vij[3];
#pragma unroll
    for (int a = 0; a < D; ++a) vij[a] = vi[a] - vj[a];
    float z[6];
    if (noise) pair_draw<D>(k.rhs_force_type, k.rk, step, pidi, pid[j], z);
    T pa[3], si_s, sj_s;
    pair_force<T, D>(k, r, inv_d, vij, Ai, Bi, Aj, Bj, gw, noise, z, inv_sqdt, pa);
    if (nnw) {
      // polymer part of the pressure-tensor force,
      // rhs_force_ff_non_Newtonian_HuAdams.F90:95-110, and the velocity
      // gradient of pp_vgt_ip.inc
#pragma unroll
      for (int b = 0; b < D; ++b) {
        T s_ = 0;
#pragma unroll
        for (int a = 0; a < D; ++a) s_ += (qie[1 + a + D * b] + qj[1 + a + D * b]) * r[a];
        pa[b] += gw * inv_d * s_;
      }
      const T fac = gw * qie[0] * inv_d;
#pragma unroll
      for (int b = 0; b < D; ++b)
#pragma unroll
        for (int a = 0; a < D; ++a) L[a + D * b] += (vj[a] - vi[a]) * r[b] * fac;
    }
    pair_scales<T>(k.rhs_force_type, ci.z, cj.z, si_s, sj_s);
#pragma unroll
    for (int a = 0; a < D; ++a) pa[a] *= si_s;
#pragma unroll
    for (int a = 0; a < D; ++a) acc[a] += pa[a];
    if (k.stress) {
      // pp_interaction_ff.inc:83-93: s_ab += r_a * f_b / 2
#pragma unroll
      for (int b = 0; b < D; ++b)
#pragma unroll
        for (int a = 0; a < D; ++a) sacc[b * D + a] += r[a] * pa[b] * T(0.5);
    }
  }
  if (k.stress) {
#pragma unroll
    for (int a = 0; a < D * D; ++a) st[(size_t)a * n + i] = sacc[a];
  }
  if (nnw) nn_epilogue<D>(k, nn, i, L, fuse_mode, dt);
  force_epilogue<D>(k, i, si, xi, acc[0], acc[1], D == 3 ? acc[2] : 0.0, fuse_mode, dt, v,
                    f, v_out, err);
}

// ---------------------------------------------------------------------------
// FP32-mixed force sweep: pair arithmetic in FP32 on cell offsets, Kahan
// sums, the next pair's data loaded while the current one is computed.
// ---------------------------------------------------------------------------
struct JData {
  float4 o, v, c;
  int sl, j;
};

template <int D>
__device__ __forceinline__ JData load_j(const int* __restrict__ s_start, int ent,
                                        const float4* __restrict__ off,
                                        const float4* __restrict__ vf,
                                        const float4* __restrict__ pcf) {
  JData d;
  d.sl = ent >> kLocalBits;
  d.j = s_start[d.sl * kReuseTPB + threadIdx.x] + (ent & (kMaxCellCount - 1));
  d.o = off[d.j];
  d.v = vf[d.j];
  d.c = pcf[d.j];
  return d;
}

// S lanes per particle (1, or 4 for small systems, where one thread per
// particle leaves most of the GPU idle and each thread's serial pair loop
// sets the time): lane l takes list entries l, l + S, ...; the lanes' sums
// are added in lane order by the first lane, which runs the epilogue.
// STRESS: the per-particle stress s_i += r_ij (x) a_ij / 2 is accumulated
// (a compile-time switch: its nine sums would otherwise stay live across
// the pair loop of every run).  The 3D Oldroyd-B instances take 4 blocks
// per SM: at 5 (96 registers) they spill the polymer terms.
template <int D, bool NNW, int S, bool STRESS>
__global__ void __launch_bounds__(kReuseTPB, (NNW && D == 3) ? 4 : 5)
    k_force32(Consts k, const int* __restrict__ cell_start, const int* __restrict__ cell_of,
              const uint16_t* __restrict__ nl, const int* __restrict__ ncount, int cap,
              const float4* __restrict__ off,
              const double4_32a* __restrict__ x, const double4_32a* __restrict__ v,
              const float4* __restrict__ pcf, const float4* __restrict__ vf,
              const float2* __restrict__ wd, double4_32a* __restrict__ f,
              double* __restrict__ st, int fuse_mode, double dt,
              double4_32a* __restrict__ v_out, uint32_t step_arg,
              const int64_t* __restrict__ step_ptr, float inv_sqdt,
              unsigned* __restrict__ err, NN nn, CollArgs ca) {
  constexpr int D2 = D * D;
  using T = float;
  const uint32_t step = step_ptr ? (uint32_t)*step_ptr : step_arg;
  // one thread per particle, whatever its cell: per-thread neighbour-cell
  // tables keep every lane busy (2D cells hold ~9 particles)
  __shared__ int s_start[kMaxStencil * kReuseTPB];
  const int n = k.n;
  const bool noise = k.noise != 0;
  const bool walls = k.wall_axis != -1;
  __shared__ float4 s_slot[kSlotTable];
  fill_slot_offsets<D>(k, s_slot);
  __syncthreads();
  const int gt = blockIdx.x * kReuseTPB + threadIdx.x;
  const int i = gt / S, lane_s = gt % S;
  if (i >= n) return;  // the S lanes of a particle leave together
  const int celli = cell_of[i];
  build_lane_table<D, kReuseTPB, false>(k, celli, cell_start, s_start, nullptr);
  const float4* slot_tab = slot_table(k, s_slot, celli);
  const float4 oi = off[i];
  const int si = __float_as_int(oi.w);
  const float4 v4i = vf[i];
  const int pidi = __float_as_int(v4i.w);
  const float4 ci = pcf[i];
  const float2 wdi = (walls && k.wall_axis >= 0) ? wd[i] : make_float2(0.f, 0.f);
  constexpr bool nnw = NNW;  // Oldroyd-B terms compiled only when used
  const float* qq = (const float*)nn.qq;
  T qi[1 + D2], L[D2];
#pragma unroll
  for (int cc = 0; cc < D2; ++cc) L[cc] = 0.f;
  if (nnw) {
#pragma unroll
    for (int cc = 0; cc <= D2; ++cc) qi[cc] = qq[(size_t)cc * n + i];
  }
  T acc[3] = {0.f, 0.f, 0.f}, comp[3] = {0.f, 0.f, 0.f};
  T sacc[9];
#pragma unroll
  for (int a = 0; a < 9; ++a) sacc[a] = 0.f;
  // the list's two segments (fluid-fluid pairs from row 0 up, the others
  // from row cap-1 down; a per-step list has only the first)
  const int nc = ncount[i];
  const int nff = nc & 0xffff, cnt = nff + (nc >> 16);
  JData nxt;
  int ent_n1 = 0;
  if (lane_s < cnt)
    nxt = load_j<D>(s_start, nl[(size_t)cand_row(lane_s, nff, cap) * n + i], off, vf, pcf);
  if (lane_s + S < cnt) ent_n1 = nl[(size_t)cand_row(lane_s + S, nff, cap) * n + i];
  for (int e = lane_s; e < cnt; e += S) {
    const JData cur = nxt;
    if (e + S < cnt) {
      nxt = load_j<D>(s_start, ent_n1, off, vf, pcf);
      if (e + 2 * S < cnt) ent_n1 = nl[(size_t)cand_row(e + 2 * S, nff, cap) * n + i];
    }
    const int sj = __float_as_int(cur.o.w);
    if (si != 0 && sj != 0 && !(si > 0 && sj > 0 && si != sj && k.pp_cc)) continue;
    const int sl = cur.sl;
    T r[3];
    const float4 so = slot_tab[sl];
    r[0] = (oi.x - cur.o.x) - so.x;
    r[1] = (oi.y - cur.o.y) - so.y;
    r[2] = (D == 3) ? (oi.z - cur.o.z) - so.z : 0.f;
    T d2 = r[0] * r[0] + r[1] * r[1];
    if (D == 3) d2 += r[2] * r[2];
    const T inv_d = rsqrtf(d2);
    const T d = d2 * inv_d;
    T vi[3] = {v4i.x, v4i.y, v4i.z};
    T vj[3] = {cur.v.x + so.w, cur.v.y, cur.v.z};
    T Ai = ci.x, Aj = cur.c.x, Bi = ci.y, Bj = cur.c.y;
    T qj[1 + D2], qie[1 + D2];
    if (nnw) {
#pragma unroll
      for (int cc = 0; cc <= D2; ++cc) {
        qj[cc] = qq[(size_t)cc * n + cur.j];
        qie[cc] = qi[cc];
      }
    }
    if (si < 0 || sj < 0) {
      // fluid-wall pair: the wall particle takes the Morris no-slip
      // velocity and the fluid pressure (pp_interaction_fw.inc / _wf.inc),
      // in the Oldroyd-B model also the fluid density and pressure
      // tensor; face distances come from the FP64-rounded per-particle
      // values (one wall axis) or from the FP64 positions (several)
      const int sw = (sj < 0) ? sj : si;
      const int face = -sw;
      const bool lower = (face & 1) != 0;
      float df, dw;
      if (k.wall_axis >= 0) {
        const float2 wj = wd[cur.j];
        const float di = lower ? wdi.x : wdi.y, dj = lower ? wj.x : wj.y;
        df = (sj < 0) ? di : dj;
        dw = (sj < 0) ? dj : di;
      } else {
        const int axis = (face - 1) >> 1;
        const double x_sur = axis == 0 ? (lower ? k.min_phys[0] : k.max_phys[0])
                             : axis == 1 ? (lower ? k.min_phys[1] : k.max_phys[1])
                                         : (lower ? k.min_phys[2] : k.max_phys[2]);
        const double4_32a a4 = x[i], b4 = x[cur.j];
        const double xa = axis == 0 ? a4.x : axis == 1 ? a4.y : a4.z;
        const double xb = axis == 0 ? b4.x : axis == 1 ? b4.y : b4.z;
        df = (float)(((sj < 0) ? xa : xb) - x_sur);
        dw = (float)(((sj < 0) ? xb : xa) - x_sur);
      }
      T vw[3];
      if (sj < 0) {
        wall_noslip_dist<T, D>(k, df, dw, vi, sj, vw);
#pragma unroll
        for (int a = 0; a < D; ++a) vj[a] = vw[a];
        if (nnw) {
          Aj = Ai;
          Bj = Bi;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qj[cc] = qi[cc];
        } else {
          Aj = boundary_A<T>(k.rhs_force_type, ci.w, cur.c.y);
        }
      } else {
        wall_noslip_dist<T, D>(k, df, dw, vj, si, vw);
#pragma unroll
        for (int a = 0; a < D; ++a) vi[a] = vw[a];
        if (nnw) {
          Ai = Aj;
          Bi = Bj;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qie[cc] = qj[cc];
        } else {
          Ai = boundary_A<T>(k.rhs_force_type, cur.c.w, ci.y);
        }
      }
    } else if ((si > 0) != (sj > 0)) {
      // fluid-colloid pair (pp_interaction_fc.inc / _cf.inc)
      if (sj > 0) {
        if (k.coll_noslip == 2) {
          const float4 rc4 = ca.rxcf[cur.j];
          const T rxc_[3] = {rc4.x, rc4.y, rc4.z};
          T vw[3];
          colloid_noslip<T, D>(k, sj - 1, rxc_, r, vi, vw);
#pragma unroll
          for (int a = 0; a < D; ++a) vj[a] = vw[a];
        }
        if (nnw) {
          Aj = Ai;
          Bj = Bi;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qj[cc] = qi[cc];
        } else {
          Aj = boundary_A<T>(k.rhs_force_type, ci.w, cur.c.y);
        }
      } else {
        if (k.coll_noslip == 2) {
          const float4 rc4 = ca.rxcf[i];
          const T rxc_[3] = {rc4.x, rc4.y, rc4.z};
          const T rfc[3] = {-r[0], -r[1], -r[2]};
          T vw[3];
          colloid_noslip<T, D>(k, si - 1, rxc_, rfc, vj, vw);
#pragma unroll
          for (int a = 0; a < D; ++a) vi[a] = vw[a];
        }
        if (nnw) {
          Ai = Aj;
          Bi = Bj;
#pragma unroll
          for (int cc = 0; cc <= D2; ++cc) qie[cc] = qj[cc];
        } else {
          Ai = boundary_A<T>(k.rhs_force_type, cur.c.w, ci.y);
        }
      }
    }
    const T gw = kernel_gradw<T>(k, d);
    T vij[3];
#pragma unroll
    for (int a = 0; a < D; ++a) vij[a] = vi[a] - vj[a];
    float z[6];
    if (noise)
      pair_draw<D>(k.rhs_force_type, k.rk, step, pidi, __float_as_int(cur.v.w), z);
    T pa[3], si_s, sj_s;
    pair_force<T, D>(k, r, inv_d, vij, Ai, Bi, Aj, Bj, gw, noise, z, inv_sqdt, pa);
    if (nnw) {
      // polymer pressure-tensor force and velocity gradient (FP32 pairs)
#pragma unroll
      for (int b = 0; b < D; ++b) {
        T s_ = 0.f;
#pragma unroll
        for (int a = 0; a < D; ++a) s_ += (qie[1 + a + D * b] + qj[1 + a + D * b]) * r[a];
        pa[b] += gw * inv_d * s_;
      }
      const T fac = gw * qie[0] * inv_d;
#pragma unroll
      for (int b = 0; b < D; ++b)
#pragma unroll
        for (int a = 0; a < D; ++a) L[a + D * b] += (vj[a] - vi[a]) * r[b] * fac;
    }
    pair_scales<T>(k.rhs_force_type, ci.z, cur.c.z, si_s, sj_s);
#pragma unroll
    for (int a = 0; a < D; ++a) pa[a] *= si_s;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const T y = pa[a] - comp[a];
      const T tt = acc[a] + y;
      comp[a] = (tt - acc[a]) - y;
      acc[a] = tt;
    }
    if (STRESS) {
#pragma unroll
      for (int b = 0; b < D; ++b)
#pragma unroll
        for (int a = 0; a < D; ++a) sacc[b * D + a] += r[a] * pa[b] * 0.5f;
    }
  }
  if (S > 1) {
    // the lanes' sums, added in lane order by lane 0 of the group
    const unsigned gmask = ((1u << S) - 1u) << ((threadIdx.x & 31) & ~(S - 1));
    const int base = (threadIdx.x & 31) & ~(S - 1);
    T part[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) part[a] = acc[a] - comp[a];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      T tot = part[a];
      for (int q = 1; q < S; ++q) tot += __shfl_sync(gmask, part[a], base + q);
      acc[a] = tot;
      comp[a] = 0.f;
    }
    if (nnw) {
#pragma unroll
      for (int cc = 0; cc < D2; ++cc) {
        T tot = L[cc];
        for (int q = 1; q < S; ++q) tot += __shfl_sync(gmask, L[cc], base + q);
        L[cc] = tot;
      }
    }
    if (STRESS) {
#pragma unroll
      for (int a = 0; a < 9; ++a) {
        T tot = sacc[a];
        for (int q = 1; q < S; ++q) tot += __shfl_sync(gmask, sacc[a], base + q);
        sacc[a] = tot;
      }
    }
    if (lane_s != 0) return;
  }
  if (STRESS) {
#pragma unroll
    for (int a = 0; a < D * D; ++a) st[(size_t)a * n + i] = (double)sacc[a];
  }
  const double4_32a xi4 = x[i];
  const double xi[3] = {xi4.x, xi4.y, xi4.z};
  if (nnw) {
    double Ld[D2];
#pragma unroll
    for (int cc = 0; cc < D2; ++cc) Ld[cc] = (double)L[cc];
    nn_epilogue<D>(k, nn, i, Ld, fuse_mode, dt);
  }
  force_epilogue<D>(k, i, si, xi, (double)acc[0], (double)acc[1],
                    D == 3 ? (double)acc[2] : 0.0, fuse_mode, dt, v, f, v_out, err);
}

// ---------------------------------------------------------------------------
// Symmetric force sweep: every pair is evaluated once, by the particle whose
// cell owns it (partner in one of the 13 forward cells, or later in the same
// cell: the half-shell of ppm_neighlist_MkNeighIdx.F90:198-249).  The owner
// keeps its share in registers (Kahan in FP32); the partner's share is
// summed per (forward slot, partner) in shared memory.  Lanes of a round that
// hit the same partner are combined with __match_any_sync, in lane order,
// by the lowest such lane, so every sum has a fixed order and the result is
// deterministic without atomics.  The per-slot partial sums go to planes
// jp[slot][c][n] that k_force_gather adds up per particle.
// ---------------------------------------------------------------------------
template <bool FP64>
struct SymT;
template <>
struct SymT<true> {
  using T = double;
  static constexpr int CC = 32;  // partners per slot held in shared memory
};
template <>
struct SymT<false> {
  using T = float;
  static constexpr int CC = 64;
};


// Per-warp dynamic shared memory of k_force_sym (bytes), see the layout in
// the kernel.
template <int D, bool FP64>
__host__ __device__ constexpr int sym_warp_bytes() {
  using T = typename SymT<FP64>::T;
  constexpr int NSF = (D == 3) ? 14 : 5;
  constexpr int CC = SymT<FP64>::CC;
  constexpr int part = NSF * 3 * CC * (int)sizeof(T);
  constexpr int accs = 2 * 3 * 32 * (int)sizeof(T);
  constexpr int idx = 96 * 4;  // ex[33], e0[32], pad
  constexpr int own = FP64 ? (3 * 32 * 32 + 2 * 32 * 4) : (3 * 32 * 16 + 32 * 8);
  return ((part + accs + idx + own) + 31) / 32 * 32;
}

template <int D, bool FP64>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_force_sym(Consts k, const int* __restrict__ cell_start, const uint16_t* __restrict__ nl,
                const int* __restrict__ ncount, const int* __restrict__ nhs,
                const float4* __restrict__ off, const double4_32a* __restrict__ x,
                const double4_32a* __restrict__ v, const double4_32a* __restrict__ pc,
                const float4* __restrict__ pcf, const float4* __restrict__ vf,
                const float2* __restrict__ wd, const int* __restrict__ sid,
                const int* __restrict__ pid, typename SymT<FP64>::T* __restrict__ jp,
                uint32_t step_arg, const int64_t* __restrict__ step_ptr,
                typename SymT<FP64>::T inv_sqdt) {
  // the Philox counter's step: the argument, or the device step counter
  // when the sweep runs inside a captured graph
  const uint32_t step = step_ptr ? (uint32_t)*step_ptr : step_arg;
  using T = typename SymT<FP64>::T;
  constexpr int CC = SymT<FP64>::CC;
  constexpr int CENTER = (D == 3) ? 13 : 4;
  constexpr int NSF = (D == 3) ? 14 : 5;  // forward slots CENTER..NS-1
  extern __shared__ __align__(32) unsigned char smem_raw[];
  __shared__ NbTable tab[kWarpsPerBlock];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per-warp layout: part[NSF][3][CC] | acc[3][32] | comp[3][32] | ex[33] e0[32] |
  //                  owner data (FP32: off, vf, pcf float4 + wd float2;
  //                              FP64: x, v, pc double4 + sid, pid int)
  unsigned char* wb = smem_raw + (size_t)wib * sym_warp_bytes<D, FP64>();
  T* part = reinterpret_cast<T*>(wb);
  T* acc_s = part + NSF * 3 * CC;
  T* comp_s = acc_s + 3 * 32;
  int* ex = reinterpret_cast<int*>(comp_s + 3 * 32);
  int* e0s = ex + 33;
  unsigned char* own = reinterpret_cast<unsigned char*>(ex + 96);
  const int n = k.n;
  const bool noise = k.noise != 0;
  const bool walls = k.wall_axis != -1;
  for (int cell = blockIdx.x * kWarpsPerBlock + wib; cell <= k.ncell;
       cell += gridDim.x * kWarpsPerBlock) {
    NbTable& t = tab[wib];
    build_table<D>(k, cell, cell_start, t);
    // zero the partner sums this cell owns (shared, or global when a cell
    // holds more than CC particles)
    for (int s = 0; s < NSF; ++s) {
      const int cs_ = t.count[CENTER + s], st_ = t.start[CENTER + s];
      for (int q = lane; q < cs_; q += 32)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          if (cs_ <= CC)
            part[(s * 3 + a) * CC + q] = T(0);
          else
            jp[((size_t)s * 3 + a) * n + st_ + q] = T(0);
        }
    }
    const int c0 = t.start[CENTER], c1 = c0 + t.count[CENTER];
    for (int base = c0; base < c1; base += 32) {
      const int i = base + lane;
      const bool act = i < c1;
      const int e0 = act ? nhs[i] : 0, e1 = act ? ncount[i] : 0;
      const int len = e1 - e0;
      // owner data and accumulators of this chunk in shared memory
      if (FP64) {
        double4_32a* ox = reinterpret_cast<double4_32a*>(own);
        double4_32a* ov = ox + 32;
        double4_32a* oc = ov + 32;
        int* os = reinterpret_cast<int*>(oc + 32);
        int* op = os + 32;
        if (act) {
          ox[lane] = x[i];
          ov[lane] = v[i];
          oc[lane] = pc[i];
          os[lane] = sid[i];
          op[lane] = pid[i];
        }
      } else {
        float4* oo = reinterpret_cast<float4*>(own);
        float4* ov = oo + 32;
        float4* oc = ov + 32;
        float2* ow = reinterpret_cast<float2*>(oc + 32);
        if (act) {
          oo[lane] = off[i];
          ov[lane] = vf[i];
          oc[lane] = pcf[i];
          if (walls && k.wall_axis >= 0) ow[lane] = wd[i];
        }
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        acc_s[a * 32 + lane] = T(0);
        comp_s[a * 32 + lane] = T(0);
      }
      // exclusive prefix of the owned-pair counts: the warp's pairs are
      // spread evenly over the lanes, 32 per round
      int incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int tt = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += tt;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      ex[lane] = incl - len;
      e0s[lane] = e0;
      if (lane == 31) ex[32] = total;
      __syncwarp();
      const int rounds = (total + 31) >> 5;
      for (int r = 0; r < rounds; ++r) {
        const int fidx = r * 32 + lane;
        const bool valid = fidx < total;
        int ow_l = 0;
#pragma unroll
        for (int stp = 16; stp > 0; stp >>= 1)
          if (ex[ow_l + stp] <= fidx) ow_l += stp;
        bool has = false;
        int keyj = 0, jsl = 0, jq = 0;
        T vjs[3] = {0, 0, 0}, vis[3] = {0, 0, 0};
        if (valid) {
          const int ii = base + ow_l;
          const int e = e0s[ow_l] + (fidx - ex[ow_l]);
          const int ent = nl[(size_t)e * n + ii];
          jsl = ent >> kLocalBits;
          jq = ent & (kMaxCellCount - 1);
          const int j = t.start[jsl] + jq;
          T rr[3], vi[3], vj[3];
          T Ai, Bi, Ci, Pi, Aj, Bj, Cj, Pj, inv_d, d;
          int si, sj, pidi, pidj;
          double xi[3] = {0.0, 0.0, 0.0}, xj[3] = {0.0, 0.0, 0.0};
          float2 wdi = make_float2(0.f, 0.f);
          if (FP64) {
            const double4_32a* ox = reinterpret_cast<const double4_32a*>(own);
            const int* os = reinterpret_cast<const int*>(ox + 96);
            const double4_32a x4 = ox[ow_l], v4 = ox[32 + ow_l], c4 = ox[64 + ow_l];
            si = os[ow_l];
            pidi = os[32 + ow_l];
            xi[0] = x4.x; xi[1] = x4.y; xi[2] = x4.z;
            vi[0] = (T)v4.x; vi[1] = (T)v4.y; vi[2] = (T)v4.z;
            Ai = (T)c4.x; Bi = (T)c4.y; Ci = (T)c4.z; Pi = (T)c4.w;
            sj = sid[j];
            const double4_32a xj4 = x[j];
            xj[0] = xj4.x; xj[1] = xj4.y; xj[2] = xj4.z;
            double r64[3];
            const double d2 = exact_sep<D>(k, xi, xj, t.shift[jsl], r64);
#pragma unroll
            for (int a = 0; a < 3; ++a) rr[a] = (T)r64[a];
            // MCF's correctly rounded SQRT for the kernel's argument (see
            // k_force64)
            inv_d = (T)rsqrt(d2);
            d = (T)sqrt(d2);
            const double4_32a vj4 = v[j], cj4 = pc[j];
            vj[0] = (T)vj4.x; vj[1] = (T)vj4.y; vj[2] = (T)vj4.z;
            Aj = (T)cj4.x; Bj = (T)cj4.y; Cj = (T)cj4.z; Pj = (T)cj4.w;
            pidj = noise ? pid[j] : 0;
          } else {
            const float4* oo = reinterpret_cast<const float4*>(own);
            const float2* ow = reinterpret_cast<const float2*>(oo + 96);
            const float4 o4 = oo[ow_l], v4 = oo[32 + ow_l], c4 = oo[64 + ow_l];
            si = __float_as_int(o4.w);
            pidi = __float_as_int(v4.w);
            vi[0] = (T)v4.x; vi[1] = (T)v4.y; vi[2] = (T)v4.z;
            Ai = (T)c4.x; Bi = (T)c4.y; Ci = (T)c4.z; Pi = (T)c4.w;
            if (walls && k.wall_axis >= 0) wdi = ow[ow_l];
            const float4 oj = off[j], vj4 = vf[j], cj4 = pcf[j];
            sj = __float_as_int(oj.w);
            const float4 so = t.o[jsl];
            rr[0] = (T)((o4.x - oj.x) - so.x);
            rr[1] = (T)((o4.y - oj.y) - so.y);
            rr[2] = (D == 3) ? (T)((o4.z - oj.z) - so.z) : T(0);
            T d2 = rr[0] * rr[0] + rr[1] * rr[1];
            if (D == 3) d2 += rr[2] * rr[2];
            inv_d = (T)rsqrtf((float)d2);
            d = d2 * inv_d;
            vj[0] = (T)vj4.x; vj[1] = (T)vj4.y; vj[2] = (T)vj4.z;
            Aj = (T)cj4.x; Bj = (T)cj4.y; Cj = (T)cj4.z; Pj = (T)cj4.w;
            pidj = __float_as_int(vj4.w);
          }
          has = !(si != 0 && sj != 0);  // w-w, c-c, c-w: no interaction here
          if (has) {
            if (si < 0 || sj < 0) {
              // fluid-wall pair (pp_interaction_fw.inc / _wf.inc)
              const int sw = (sj < 0) ? sj : si;
              const int face = -sw;
              const bool lower = (face & 1) != 0;
              const int axis = (face - 1) >> 1;
              T df, dw;
              if (!FP64 && k.wall_axis >= 0) {
                const float2 wj = wd[j];
                const float a_ = lower ? wdi.x : wdi.y, b_ = lower ? wj.x : wj.y;
                df = (T)((sj < 0) ? a_ : b_);
                dw = (T)((sj < 0) ? b_ : a_);
              } else {
                const double x_sur = axis == 0 ? (lower ? k.min_phys[0] : k.max_phys[0])
                                     : axis == 1 ? (lower ? k.min_phys[1] : k.max_phys[1])
                                                 : (lower ? k.min_phys[2] : k.max_phys[2]);
                double xa, xb;
                if (FP64) {
                  xa = axis == 0 ? xi[0] : axis == 1 ? xi[1] : xi[2];
                  xb = axis == 0 ? xj[0] : axis == 1 ? xj[1] : xj[2];
                } else {
                  const double4_32a a4 = x[ii], b4 = x[j];
                  xa = axis == 0 ? a4.x : axis == 1 ? a4.y : a4.z;
                  xb = axis == 0 ? b4.x : axis == 1 ? b4.y : b4.z;
                }
                df = (T)(((sj < 0) ? xa : xb) - x_sur);
                dw = (T)(((sj < 0) ? xb : xa) - x_sur);
              }
              T vw[3];
              if (sj < 0) {
                wall_noslip_dist<T, D>(k, df, dw, vi, sj, vw);
#pragma unroll
                for (int a = 0; a < D; ++a) vj[a] = vw[a];
                Aj = boundary_A<T>(k.rhs_force_type, Pi, Bj);
              } else {
                wall_noslip_dist<T, D>(k, df, dw, vj, si, vw);
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
            if (noise) pair_draw<D>(k.rhs_force_type, k.rk, step, pidi, pidj, z);
            T g[3], s_i, s_j;
            pair_force<T, D>(k, rr, inv_d, vij, Ai, Bi, Aj, Bj, gw, noise, z, inv_sqdt, g);
            pair_scales<T>(k.rhs_force_type, Ci, Cj, s_i, s_j);
#pragma unroll
            for (int a = 0; a < D; ++a) {
              vis[a] = g[a] * s_i;
              vjs[a] = -g[a] * s_j;
            }
            keyj = (jsl - CENTER) * kMaxCellCount + jq;
          }
        }
        // deterministic combination: lanes of this round with the same
        // target are summed in lane order by the lowest of them
        const unsigned amask = __ballot_sync(0xffffffffu, has);
        if (has) {
          // partner side
          {
            const unsigned peers = __match_any_sync(amask, keyj);
            T s0 = vjs[0], s1 = vjs[1], s2 = vjs[2];
            if (peers != (1u << lane)) {
              s0 = s1 = s2 = T(0);
              for (unsigned mm = peers; mm; mm &= mm - 1) {
                const int src = __ffs(mm) - 1;
                s0 += __shfl_sync(peers, vjs[0], src);
                s1 += __shfl_sync(peers, vjs[1], src);
                s2 += __shfl_sync(peers, vjs[2], src);
              }
            }
            if (lane == __ffs(peers) - 1) {
              const int s = jsl - CENTER;
              if (t.count[jsl] <= CC) {
                part[(s * 3 + 0) * CC + jq] += s0;
                part[(s * 3 + 1) * CC + jq] += s1;
                part[(s * 3 + 2) * CC + jq] += s2;
              } else {
                const size_t b0 = (size_t)t.start[jsl] + jq;
                jp[((size_t)s * 3 + 0) * n + b0] += s0;
                jp[((size_t)s * 3 + 1) * n + b0] += s1;
                jp[((size_t)s * 3 + 2) * n + b0] += s2;
              }
            }
          }
          // owner side (Kahan-compensated in FP32)
          {
            const unsigned peers = __match_any_sync(amask, ow_l);
            T s0 = vis[0], s1 = vis[1], s2 = vis[2];
            if (peers != (1u << lane)) {
              s0 = s1 = s2 = T(0);
              for (unsigned mm = peers; mm; mm &= mm - 1) {
                const int src = __ffs(mm) - 1;
                s0 += __shfl_sync(peers, vis[0], src);
                s1 += __shfl_sync(peers, vis[1], src);
                s2 += __shfl_sync(peers, vis[2], src);
              }
            }
            if (lane == __ffs(peers) - 1) {
              const T sv[3] = {s0, s1, s2};
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                T& acc = acc_s[a * 32 + ow_l];
                if (FP64) {
                  acc += sv[a];
                } else {
                  T& cmp = comp_s[a * 32 + ow_l];
                  const T y = sv[a] - cmp;
                  const T tt = acc + y;
                  cmp = (tt - acc) - y;
                  acc = tt;
                }
              }
            }
          }
        }
        __syncwarp();
      }
      if (act) {
#pragma unroll
        for (int a = 0; a < 3; ++a) jp[((size_t)NSF * 3 + a) * n + i] = acc_s[a * 32 + lane];
      }
      __syncwarp();
    }
    __syncwarp();
    for (int s = 0; s < NSF; ++s) {
      const int cs_ = t.count[CENTER + s], st_ = t.start[CENTER + s];
      if (cs_ > CC) continue;
      for (int q = lane; q < cs_; q += 32)
#pragma unroll
        for (int a = 0; a < 3; ++a)
          jp[((size_t)s * 3 + a) * n + st_ + q] = part[(s * 3 + a) * CC + q];
    }
    __syncwarp();
  }
}

// Sum of the per-slot partner shares and the owner share of every particle
// (fixed order, Kahan in FP32), then body force and the second half kick.
template <int D, bool FP64>
__global__ void k_force_gather(Consts k, const int* __restrict__ cell_of,
                               const typename SymT<FP64>::T* __restrict__ jp,
                               const double4_32a* __restrict__ x,
                               const double4_32a* __restrict__ v, const int* __restrict__ sid,
                               double4_32a* __restrict__ f, int fuse_mode, double dt,
                               double4_32a* __restrict__ v_out, unsigned* __restrict__ err) {
  using T = typename SymT<FP64>::T;
  constexpr int CENTER = (D == 3) ? 13 : 4;
  constexpr int NSF = (D == 3) ? 14 : 5;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = k.n;
  if (j >= n) return;
  const int cj = cell_of[j];
  int cc[3] = {0, 0, 0};
  if (cj < k.ncell) {
    int rem = cj;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      cc[a] = rem % k.nm[a];
      rem /= k.nm[a];
    }
  }
  T acc[3], comp[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < 3; ++a) acc[a] = jp[((size_t)NSF * 3 + a) * n + j];
  if (cj < k.ncell) {
#pragma unroll
    for (int s = 0; s < NSF; ++s) {
      // the owner cell of plane s is cell(j) - offset(CENTER + s)
      const int sl = CENTER + s;
      const int o[3] = {sl % 3 - 1, (sl / 3) % 3 - 1, sl / 9 - 1};
      bool ok = true;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const int h = cc[a] - o[a];
        if ((h < 0 || h >= k.nm[a]) && !k.periodic[a]) ok = false;
      }
      if (!ok) continue;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const T val = jp[((size_t)s * 3 + a) * n + j];
        if (FP64) {
          acc[a] += val;
        } else {
          const T y = val - comp[a];
          const T tt = acc[a] + y;
          comp[a] = (tt - acc[a]) - y;
          acc[a] = tt;
        }
      }
    }
  }
  const double4_32a x4 = x[j];
  const double xj[3] = {x4.x, x4.y, x4.z};
  force_epilogue<D>(k, j, sid[j], xj, (double)acc[0], (double)acc[1],
                    D == 3 ? (double)acc[2] : 0.0, fuse_mode, dt, v, f, v_out, err);
}

static int grid_for(Handle* h) {
  const int warps = h->k.ncell + 1;  // + bin of particles without a cell
  int g = (warps + kWarpsPerBlock - 1) / kWarpsPerBlock;
  return g < 1 ? 1 : g;
}

int verlet_build_gated(Handle* h) {
  Consts& k = h->k;
  const int g = grid_for(h);
  if (k.d == 3)
    k_verlet_build<3><<<g, kWarpsPerBlock * 32, 0, h->stream>>>(
        k, h->d_rebuild, h->cell_start, h->off, h->vl, h->vcount, h->vcap, h->partitioned ? 1 : 0,
        h->d_err);
  else
    k_verlet_build<2><<<g, kWarpsPerBlock * 32, 0, h->stream>>>(
        k, h->d_rebuild, h->cell_start, h->off, h->vl, h->vcount, h->vcap, h->partitioned ? 1 : 0,
        h->d_err);
  k_rebuild_done<<<1, 1, 0, h->stream>>>(h->d_rebuild);
  h->launches += 2;
  return cuda_check(h, cudaGetLastError(), "candidate list launch") ? MCFG_ECUDA : MCFG_OK;
}

int compute_density(Handle* h, bool with_pressure, bool reuse) {
  Consts& k = h->k;
  cudaStream_t s = h->stream;
  if (cuda_check(h, cudaMemsetAsync(h->d_stats, 0, sizeof(int) * 4, s), "memset stats"))
    return MCFG_ECUDA;
  if (cuda_check(h, cudaMemsetAsync(h->d_pairs, 0, sizeof(unsigned long long), s), "memset pairs"))
    return MCFG_ECUDA;
  const int g = grid_for(h);
  const bool fp64 = h->p.precision == MCFG_PRECISION_FP64;
  // FP32 with list reuse: the compact two-segment pair list (sweep32.cu)
  if (reuse && !fp64) return density_list(h, with_pressure);
  if (reuse) {
    const int n = (int)h->n;
    if (n == 0) return MCFG_OK;
    const int gr = (n + kReuseTPB - 1) / kReuseTPB;
#define LAUNCH_R(DD)                                                                            \
  k_density_reuse<DD><<<gr, kReuseTPB, 0, s>>>(                                                 \
      k, h->cell_start, h->cell_of, h->x, h->v, h->m, h->sid, h->pid, h->vl, h->vcount, h->nl,  \
      h->ncount, h->nhs, h->neigh_cap, h->rho, h->pr, h->pc, h->pcf, h->vf,                     \
      with_pressure ? 1 : 0, h->d_err, h->d_stats, h->d_pairs, NN{h->ct, h->act, h->vgt, h->qq}, \
      CollArgs{h->v, h->rxc, h->rxcf})
    if (k.d == 3)
      LAUNCH_R(3);
    else
      LAUNCH_R(2);
#undef LAUNCH_R
    h->launches++;
    return cuda_check(h, cudaGetLastError(), "density launch") ? MCFG_ECUDA : MCFG_OK;
  }
#define LAUNCH_D(DD, PP)                                                                       \
  k_density<DD, PP><<<g, kWarpsPerBlock * 32, 0, s>>>(                                          \
      k, h->cell_start, h->off, h->x, h->v, h->m, h->sid, h->pid, h->nl, h->ncount, h->nhs,    \
      h->neigh_cap, h->rho, h->pr, h->pc, h->pcf, h->vf, with_pressure ? 1 : 0, h->d_err,      \
      h->d_stats, h->d_pairs, NN{h->ct, h->act, h->vgt, h->qq}, CollArgs{h->v, h->rxc, h->rxcf})
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
  const NN nn{h->ct, h->act, h->vgt, h->qq};
  const CollArgs ca{h->v, h->rxc, h->rxcf};
#define LAUNCH_P(DD, PP)                                                                        \
  k_pressure<DD, PP><<<gb, tb, 0, h->stream>>>(h->k, h->rho, h->m, h->pid, h->v, h->pr, h->pc,   \
                                               h->pcf, h->vf, nn, h->sid, h->x, ca)
  if (h->p.precision == MCFG_PRECISION_FP64) {
    if (h->k.d == 3) LAUNCH_P(3, true); else LAUNCH_P(2, true);
  } else {
    if (h->k.d == 3) LAUNCH_P(3, false); else LAUNCH_P(2, false);
  }
#undef LAUNCH_P
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "pressure launch")) return MCFG_ECUDA;
  return MCFG_OK;
}

int compute_force(Handle* h, int64_t step, int fuse_mode, double dt) {
  Consts& k = h->k;
  cudaStream_t s = h->stream;
  const int g = grid_for(h);
  const bool fp64 = h->p.precision == MCFG_PRECISION_FP64;
  if (k.noise && !(dt > 0.0)) return set_error(h, MCFG_EINVAL, "random force needs dt > 0");
  const double inv_sqdt = (k.noise && dt > 0.0) ? 1.0 / sqrt(dt) : 0.0;
  const int bs = kWarpsPerBlock * 32;
  const NN nn{h->ct, h->act, h->vgt, h->qq};
  const CollArgs ca{h->v, h->rxc, h->rxcf};
  const int gp = std::max(1, ((int)h->n + kReuseTPB - 1) / kReuseTPB);
  const int64_t* step_ptr = h->graph_capturing ? h->d_step : nullptr;
  // small systems: 4 lanes per particle in the FP32 sweep
  const bool split = h->n < kSplitBelow;
  const int gp4 = std::max(1, (int)((h->n * 4 + kReuseTPB - 1) / kReuseTPB));
  if (!k.stress && h->jp && fp64 && k.newtonian && k.ncoll == 0 && !k.le) {
    // symmetric sweep + per-particle gather: halves the FP64 pair work; the
    // FP32 path keeps the two-sided sweep, which is faster there (the
    // symmetric sweep's shared-memory partner sums cap its occupancy)
    const int n = (int)h->n;
    const int gbn = (n + 255) / 256;
    // the attribute is per device: set it for the handle's (a host call)
    if (k.d == 3)
      cudaFuncSetAttribute(k_force_sym<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kWarpsPerBlock * sym_warp_bytes<3, true>());
    else
      cudaFuncSetAttribute(k_force_sym<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kWarpsPerBlock * sym_warp_bytes<2, true>());
    double* jp = (double*)h->jp;
    if (k.d == 3) {
      k_force_sym<3, true><<<g, bs, kWarpsPerBlock * sym_warp_bytes<3, true>(), s>>>(
          k, h->cell_start, h->nl, h->ncount, h->nhs, h->off, h->x, h->v, h->pc, h->pcf, h->vf,
          h->wd, h->sid, h->pid, jp, (uint32_t)step, step_ptr, inv_sqdt);
      if (n > 0)
        k_force_gather<3, true><<<gbn, 256, 0, s>>>(k, h->cell_of, jp, h->x, h->v, h->sid, h->f,
                                                    fuse_mode, dt, h->v2, h->d_err);
    } else {
      k_force_sym<2, true><<<g, bs, kWarpsPerBlock * sym_warp_bytes<2, true>(), s>>>(
          k, h->cell_start, h->nl, h->ncount, h->nhs, h->off, h->x, h->v, h->pc, h->pcf, h->vf,
          h->wd, h->sid, h->pid, jp, (uint32_t)step, step_ptr, inv_sqdt);
      if (n > 0)
        k_force_gather<2, true><<<gbn, 256, 0, s>>>(k, h->cell_of, jp, h->x, h->v, h->sid, h->f,
                                                    fuse_mode, dt, h->v2, h->d_err);
    }
    h->launches++;
  } else if (fp64) {
#define LAUNCH_F64(DD, NW)                                                                      \
  k_force64<DD, NW><<<gp, kReuseTPB, 0, s>>>(k, h->cell_start, h->cell_of, h->nl, h->ncount,     \
                                            h->x, h->v, h->pc,                                 \
                                     h->sid, h->pid, h->f, h->st, fuse_mode, dt, h->v2,          \
                                     (uint32_t)step, step_ptr, inv_sqdt, h->d_err, nn, ca)
    if (k.d == 3) {
      if (k.newtonian) LAUNCH_F64(3, false); else LAUNCH_F64(3, true);
    } else {
      if (k.newtonian) LAUNCH_F64(2, false); else LAUNCH_F64(2, true);
    }
#undef LAUNCH_F64
  } else {
#define LAUNCH_F32(DD, NW, ST)                                                                  \
  do {                                                                                           \
    if (split)                                                                                   \
      k_force32<DD, NW, 4, ST><<<gp4, kReuseTPB, 0, s>>>(                                        \
          k, h->cell_start, h->cell_of, h->nl, h->ncount, h->neigh_cap, h->off, h->x, h->v,      \
          h->pcf, h->vf, h->wd, h->f, h->st, fuse_mode, dt, h->v2, (uint32_t)step, step_ptr,     \
          (float)inv_sqdt, h->d_err, nn, ca);                                                    \
    else                                                                                         \
      k_force32<DD, NW, 1, ST><<<gp, kReuseTPB, 0, s>>>(                                         \
          k, h->cell_start, h->cell_of, h->nl, h->ncount, h->neigh_cap, h->off, h->x, h->v,      \
          h->pcf, h->vf, h->wd, h->f, h->st, fuse_mode, dt, h->v2, (uint32_t)step, step_ptr,     \
          (float)inv_sqdt, h->d_err, nn, ca);                                                    \
  } while (0)
#define PICK_F32_ST(DD, NW)                   \
  do {                                        \
    if (k.stress) LAUNCH_F32(DD, NW, true);   \
    else LAUNCH_F32(DD, NW, false);           \
  } while (0)
    if (k.d == 3) {
      if (k.newtonian) PICK_F32_ST(3, false); else PICK_F32_ST(3, true);
    } else {
      if (k.newtonian) PICK_F32_ST(2, false); else PICK_F32_ST(2, true);
    }
#undef PICK_F32_ST
#undef LAUNCH_F32
  }
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "force launch")) return MCFG_ECUDA;
  if (fuse_mode == kForceBodyKick) std::swap(h->v, h->v2);
  return MCFG_OK;
}

}  // namespace mcfg
