// sweep32.cu -- FP32-mixed density and force sweeps over the candidate list.
//
// With neighbour-list reuse, a rebuild lists for every particle the
// candidates within rc + skin (k_verlet_build, pair_kernels.cu), partitioned
// by species: the fluid partners of a fluid particle first, from row 0 up;
// every other pair (wall, colloid, or a boundary particle's own pairs) from
// the last row down.  vcount packs both counts (fluid-fluid | other << 16).
//
// Each step the density sweep re-tests every candidate exactly (the FP32
// test of the per-step scan, same operation order) and writes the step's
// pairs as a compact list in the same two segments (nl rows from 0 up and
// from the last row down, ncount = fluid-fluid | other << 16): coalesced
// rows and no holes, so the force sweep walks every list row with all lanes
// busy.  The force sweep takes the fluid-fluid segment with a body that has
// no species tests (no wall or colloid terms), gathering the next pair's
// records while it computes the current one, and the other segment with the
// general body (Morris no-slip walls, colloid no-slip, boundary pressure).
// Every pair is evaluated from both sides (gather, no scatter, no atomics),
// sums run in list order: deterministic.
//
// Reference: particles_compute_density.F90:578-867, particles_compute_
// interaction.F90:609-900, pp_interaction*.inc, rhs_force_ff_Newtonian*.F90.
#include "mcfg_internal.cuh"
#include "pair_common.cuh"
#include "sph.cuh"
#include "sweep_common.cuh"

namespace mcfg {

namespace {

// physical row of logical candidate p (front segment up, back segment down)
__device__ __forceinline__ int cand_row(int p, int nff, int vcap) {
  return p < nff ? p : vcap - 1 - (p - nff);
}

// Density over the candidate list, S lanes per particle (S = 4 below
// kSplitBelow particles, as the force sweep).  Candidate p of particle i is
// a pair when its FP32 test passes; kept pairs go to the compact list, the
// fluid-fluid ones from row 0 up, the others from row cap-1 down.
template <int D, int S>
__global__ void __launch_bounds__(kReuseTPB)
    k_density_list(Consts k, const int* __restrict__ cell_start, const int* __restrict__ cell_of,
                   const float4* __restrict__ off, const double4_32a* __restrict__ x,
                   const double4_32a* __restrict__ v, const double* __restrict__ m,
                   const int* __restrict__ pid, const uint16_t* __restrict__ vl,
                   const int* __restrict__ vcount, int vcap, uint16_t* __restrict__ nl,
                   int* __restrict__ ncount, int cap, double* __restrict__ rho,
                   double* __restrict__ pr, float4* __restrict__ pcf, float4* __restrict__ vf,
                   int with_pressure, unsigned* __restrict__ err, int* __restrict__ stats,
                   unsigned long long* __restrict__ pairs, NN nn, CollArgs ca) {
  __shared__ int s_start[kMaxStencil * kReuseTPB];
  __shared__ float4 s_slot[kSlotTable];
  const int n = k.n, tid = threadIdx.x;
  const int gt = blockIdx.x * kReuseTPB + tid;
  const int i = gt / S, lane_s = gt % S;
  fill_slot_offsets<D>(k, s_slot);
  __syncthreads();
  int kff = 0, ko = 0, si = 0;
  bool acc_i = false;
  float sum = 0.0f, comp = 0.0f;
  if (i < n) {
    const int celli = cell_of[i];
    build_lane_table<D, kReuseTPB, false>(k, celli, cell_start, s_start, nullptr);
    const float4* slot_tab = slot_table(k, s_slot, celli);
    const float4 oi = off[i];
    si = __float_as_int(oi.w);
    acc_i = dyn_rho(k, si);
    const bool mass = k.rhs_density_type == 1;
    const int vc = vcount[i];
    const int nff = vc & 0xffff, ntot = nff + (vc >> 16);
    if (S == 1) {
      // candidates in groups of four: their entries, then their offsets,
      // are loaded before any is used (the sweep waits on these gathers)
      constexpr int kGather = 4;
      for (int p0 = 0; p0 < ntot; p0 += kGather) {
        int entg[kGather], jg[kGather];
        float4 og[kGather];
#pragma unroll
        for (int u = 0; u < kGather; ++u)
          entg[u] = (p0 + u < ntot) ? (int)vl[(size_t)cand_row(p0 + u, nff, vcap) * n + i] : 0;
#pragma unroll
        for (int u = 0; u < kGather; ++u) {
          jg[u] = s_start[(entg[u] >> kLocalBits) * kReuseTPB + tid] +
                  (entg[u] & (kMaxCellCount - 1));
          og[u] = (p0 + u < ntot) ? off[jg[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kGather; ++u) {
          const int p = p0 + u;
          if (p >= ntot) break;
          const float4 oj = og[u];
          const float4 so = slot_tab[entg[u] >> kLocalBits];
          // the pair test as k_density's scan rounds it: (o_i - slot) - o_j
          const float tx = (oi.x - so.x) - oj.x, ty = (oi.y - so.y) - oj.y;
          float t2 = tx * tx + ty * ty;
          if (D == 3) {
            const float tz = (oi.z - so.z) - oj.z;
            t2 += tz * tz;
          }
          if (!(t2 < k.rc2f)) continue;
          if (kff + ko < cap) {
            const int row = (p < nff) ? kff : cap - 1 - ko;
            nl[(size_t)row * n + i] = (uint16_t)entg[u];
          }
          if (p < nff)
            ++kff;
          else
            ++ko;
          if (!acc_i) continue;
          // W as k_density's second phase rounds it: (o_i - o_j) - slot
          const float rx = (oi.x - oj.x) - so.x, ry = (oi.y - oj.y) - so.y;
          float d2 = rx * rx + ry * ry;
          if (D == 3) {
            const float rz = (oi.z - oj.z) - so.z;
            d2 += rz * rz;
          }
          float w = kernel_w<float>(k, sqrtf(d2));
          if (mass) w *= (float)m[jg[u]];
          const float y = w - comp;
          const float tt = sum + y;
          comp = (tt - sum) - y;
          sum = tt;
        }
      }
    } else {
      // lane l tests candidates l, l + S, ...; the group's ballots place the
      // kept pairs in candidate order in their segment
      const int base = (tid & 31) & ~(S - 1);
      const unsigned gmask = ((1u << S) - 1u) << base;
      const unsigned below = (1u << lane_s) - 1u;
      for (int p0 = 0; p0 < ntot; p0 += S) {
        const int p = p0 + lane_s;
        bool in = false;
        int ent = 0, j = 0;
        float4 oj = make_float4(0.f, 0.f, 0.f, 0.f), so = oj;
        if (p < ntot) {
          ent = vl[(size_t)cand_row(p, nff, vcap) * n + i];
          const int sl = ent >> kLocalBits;
          j = s_start[sl * kReuseTPB + tid] + (ent & (kMaxCellCount - 1));
          oj = off[j];
          so = slot_tab[sl];
          const float tx = (oi.x - so.x) - oj.x, ty = (oi.y - so.y) - oj.y;
          float t2 = tx * tx + ty * ty;
          if (D == 3) {
            const float tz = (oi.z - so.z) - oj.z;
            t2 += tz * tz;
          }
          in = t2 < k.rc2f;
        }
        const unsigned bf = (__ballot_sync(gmask, in && p < nff) >> base) & ((1u << S) - 1u);
        const unsigned bo = (__ballot_sync(gmask, in && p >= nff) >> base) & ((1u << S) - 1u);
        if (in) {
          const bool front = p < nff;
          const int pos = front ? kff + __popc(bf & below) : ko + __popc(bo & below);
          if (kff + ko + __popc(bf | bo) <= cap) {
            const int row = front ? pos : cap - 1 - pos;
            nl[(size_t)row * n + i] = (uint16_t)ent;
          }
          if (acc_i) {
            const float rx = (oi.x - oj.x) - so.x, ry = (oi.y - oj.y) - so.y;
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
        }
        kff += __popc(bf);
        ko += __popc(bo);
      }
      // the lanes' sums, added in lane order
      const float part = sum - comp;
      float tot = part;
      for (int q = 1; q < S; ++q) tot += __shfl_sync(gmask, part, base + q);
      sum = tot;
      comp = 0.0f;
    }
  }
  int my_max = 0;
  unsigned long long my_pairs = 0;
  if (i < n && lane_s == 0) {
    const int kept = kff + ko;
    if (kept > cap) {
      atomicOr(err, kErrNeighOverflow);
      kff = min(kff, cap);
      ko = min(ko, cap - kff);
    }
    ncount[i] = kff | (ko << 16);
    my_max = kept;
    my_pairs = (unsigned long long)(kff + ko);
    const double mi = m[i];
    const double rho_i = (double)(sum - comp);
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
      write_particle_records<false>(k, i, rho_out, mi, pid[i], vi4, pr, nullptr, pcf, vf, nn);
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

// State of particle i for the pair bodies of the force sweep.
template <int D, bool NNW, bool STRESS>
struct ForceAcc {
  float4 oi, v4i, ci;
  float2 wdi;
  int si, pidi, i;
  float qi[1 + D * D];
  float L[D * D];
  float acc[3], comp[3];
  float sacc[STRESS ? 9 : 1];
};

// Kahan-compensated add of one pair's acceleration (and its stress share)
template <int D, bool NNW, bool STRESS>
__device__ __forceinline__ void acc_add(ForceAcc<D, NNW, STRESS>& A, const float* pa,
                                        const float* r) {
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const float y = pa[a] - A.comp[a];
    const float tt = A.acc[a] + y;
    A.comp[a] = (tt - A.acc[a]) - y;
    A.acc[a] = tt;
  }
  if (STRESS) {
#pragma unroll
    for (int b = 0; b < D; ++b)
#pragma unroll
      for (int a = 0; a < D; ++a) A.sacc[b * D + a] += r[a] * pa[b] * 0.5f;
  }
}

// Polymer pressure-tensor force and velocity gradient of one pair (FP32).
template <int D, bool NNW, bool STRESS>
__device__ __forceinline__ void nn_pair(ForceAcc<D, NNW, STRESS>& A, const float* qie,
                                        const float* qj, const float* r, const float* vi,
                                        const float* vj, float gw, float inv_d, float* pa) {
#pragma unroll
  for (int b = 0; b < D; ++b) {
    float s_ = 0.f;
#pragma unroll
    for (int a = 0; a < D; ++a) s_ += (qie[1 + a + D * b] + qj[1 + a + D * b]) * r[a];
    pa[b] += gw * inv_d * s_;
  }
  const float fac = gw * qie[0] * inv_d;
#pragma unroll
  for (int b = 0; b < D; ++b)
#pragma unroll
    for (int a = 0; a < D; ++a) A.L[a + D * b] += (vj[a] - vi[a]) * r[b] * fac;
}

// A partner's records, gathered one pair ahead of their use.
struct PairData {
  float4 o, v, c;
  int sl, j;
};

__device__ __forceinline__ PairData load_pair(int ent, const int* s_start,
                                              const float4* __restrict__ off,
                                              const float4* __restrict__ vf,
                                              const float4* __restrict__ pcf) {
  PairData d;
  d.sl = ent >> kLocalBits;
  d.j = s_start[d.sl * kReuseTPB + threadIdx.x] + (ent & (kMaxCellCount - 1));
  d.o = off[d.j];
  d.v = vf[d.j];
  d.c = pcf[d.j];
  return d;
}

// Fluid-fluid pair: no species tests, no boundary terms.
template <int D, bool NNW, bool STRESS>
__device__ __forceinline__ void pair_fluid(const Consts& k, ForceAcc<D, NNW, STRESS>& A,
                                           const PairData& P, const float4* slot_tab,
                                           const float* qq, uint32_t step, float inv_sqdt,
                                           bool noise) {
  const float4 so = slot_tab[P.sl];
  float r[3];
  r[0] = (A.oi.x - P.o.x) - so.x;
  r[1] = (A.oi.y - P.o.y) - so.y;
  r[2] = (D == 3) ? (A.oi.z - P.o.z) - so.z : 0.f;
  float d2 = r[0] * r[0] + r[1] * r[1];
  if (D == 3) d2 += r[2] * r[2];
  const float inv_d = rsqrtf(d2);
  const float d = d2 * inv_d;
  const float vi[3] = {A.v4i.x, A.v4i.y, A.v4i.z};
  const float vj[3] = {P.v.x + so.w, P.v.y, P.v.z};
  const float gw = kernel_gradw<float>(k, d);
  float vij[3];
#pragma unroll
  for (int a = 0; a < D; ++a) vij[a] = vi[a] - vj[a];
  float z[6];
  if (noise) pair_draw<D>(k.rhs_force_type, k.rk, step, A.pidi, __float_as_int(P.v.w), z);
  float pa[3];
  pair_force<float, D>(k, r, inv_d, vij, A.ci.x, A.ci.y, P.c.x, P.c.y, gw, noise, z, inv_sqdt,
                       pa);
  if (NNW) {
    float qj[1 + D * D];
#pragma unroll
    for (int cc = 0; cc <= D * D; ++cc) qj[cc] = qq[(size_t)cc * k.n + P.j];
    nn_pair<D, NNW, STRESS>(A, A.qi, qj, r, vi, vj, gw, inv_d, pa);
  }
  float si_s, sj_s;
  pair_scales<float>(k.rhs_force_type, A.ci.z, P.c.z, si_s, sj_s);
#pragma unroll
  for (int a = 0; a < D; ++a) pa[a] *= si_s;
  acc_add<D, NNW, STRESS>(A, pa, r);
}

// Any pair with a wall or colloid particle (pp_interaction_fw/_wf/_fc/_cf/
// _cc.inc): the boundary particle takes its no-slip velocity and the fluid
// partner's pressure (Oldroyd-B: density and pressure tensor).
template <int D, bool NNW, bool STRESS>
__device__ __forceinline__ void pair_general(const Consts& k, ForceAcc<D, NNW, STRESS>& A,
                                             int ent, const int* s_start, const float4* slot_tab,
                                             const float4* __restrict__ off,
                                             const float4* __restrict__ vf,
                                             const float4* __restrict__ pcf,
                                             const float2* __restrict__ wd,
                                             const double4_32a* __restrict__ x, const float* qq,
                                             const CollArgs& ca, uint32_t step, float inv_sqdt,
                                             bool noise) {
  constexpr int D2 = D * D;
  const int sl = ent >> kLocalBits;
  const int j = s_start[sl * kReuseTPB + threadIdx.x] + (ent & (kMaxCellCount - 1));
  const float4 oj = off[j];
  const int si = A.si, sj = __float_as_int(oj.w);
  if (si != 0 && sj != 0 && !(si > 0 && sj > 0 && si != sj && k.pp_cc)) return;
  const float4 vj4 = vf[j], cj = pcf[j];
  const float4 so = slot_tab[sl];
  float r[3];
  r[0] = (A.oi.x - oj.x) - so.x;
  r[1] = (A.oi.y - oj.y) - so.y;
  r[2] = (D == 3) ? (A.oi.z - oj.z) - so.z : 0.f;
  float d2 = r[0] * r[0] + r[1] * r[1];
  if (D == 3) d2 += r[2] * r[2];
  const float inv_d = rsqrtf(d2);
  const float d = d2 * inv_d;
  float vi[3] = {A.v4i.x, A.v4i.y, A.v4i.z};
  float vj[3] = {vj4.x + so.w, vj4.y, vj4.z};
  float Ai = A.ci.x, Aj = cj.x, Bi = A.ci.y, Bj = cj.y;
  float qj[1 + D2], qie[1 + D2];
  if (NNW) {
#pragma unroll
    for (int cc = 0; cc <= D2; ++cc) {
      qj[cc] = qq[(size_t)cc * k.n + j];
      qie[cc] = A.qi[cc];
    }
  }
  if (si < 0 || sj < 0) {
    // fluid-wall pair: face distances from the FP64-rounded per-particle
    // values (one wall axis) or from the FP64 positions (several)
    const int sw = (sj < 0) ? sj : si;
    const int face = -sw;
    const bool lower = (face & 1) != 0;
    float df, dw;
    if (k.wall_axis >= 0) {
      const float2 wj = wd[j];
      const float di = lower ? A.wdi.x : A.wdi.y, dj = lower ? wj.x : wj.y;
      df = (sj < 0) ? di : dj;
      dw = (sj < 0) ? dj : di;
    } else {
      const int axis = (face - 1) >> 1;
      const double x_sur = axis == 0 ? (lower ? k.min_phys[0] : k.max_phys[0])
                           : axis == 1 ? (lower ? k.min_phys[1] : k.max_phys[1])
                                       : (lower ? k.min_phys[2] : k.max_phys[2]);
      const double4_32a a4 = x[A.i], b4 = x[j];
      const double xa = axis == 0 ? a4.x : axis == 1 ? a4.y : a4.z;
      const double xb = axis == 0 ? b4.x : axis == 1 ? b4.y : b4.z;
      df = (float)(((sj < 0) ? xa : xb) - x_sur);
      dw = (float)(((sj < 0) ? xb : xa) - x_sur);
    }
    float vw[3];
    if (sj < 0) {
      wall_noslip_dist<float, D>(k, df, dw, vi, sj, vw);
#pragma unroll
      for (int a = 0; a < D; ++a) vj[a] = vw[a];
      if (NNW) {
        Aj = Ai;
        Bj = Bi;
#pragma unroll
        for (int cc = 0; cc <= D2; ++cc) qj[cc] = A.qi[cc];
      } else {
        Aj = boundary_A<float>(k.rhs_force_type, A.ci.w, cj.y);
      }
    } else {
      wall_noslip_dist<float, D>(k, df, dw, vj, si, vw);
#pragma unroll
      for (int a = 0; a < D; ++a) vi[a] = vw[a];
      if (NNW) {
        Ai = Aj;
        Bi = Bj;
#pragma unroll
        for (int cc = 0; cc <= D2; ++cc) qie[cc] = qj[cc];
      } else {
        Ai = boundary_A<float>(k.rhs_force_type, cj.w, A.ci.y);
      }
    }
  } else if ((si > 0) != (sj > 0)) {
    // fluid-colloid pair (pp_interaction_fc.inc / _cf.inc)
    if (sj > 0) {
      if (k.coll_noslip == 2) {
        const float4 rc4 = ca.rxcf[j];
        const float rxc_[3] = {rc4.x, rc4.y, rc4.z};
        float vw[3];
        colloid_noslip<float, D>(k, sj - 1, rxc_, r, vi, vw);
#pragma unroll
        for (int a = 0; a < D; ++a) vj[a] = vw[a];
      }
      if (NNW) {
        Aj = Ai;
        Bj = Bi;
#pragma unroll
        for (int cc = 0; cc <= D2; ++cc) qj[cc] = A.qi[cc];
      } else {
        Aj = boundary_A<float>(k.rhs_force_type, A.ci.w, cj.y);
      }
    } else {
      if (k.coll_noslip == 2) {
        const float4 rc4 = ca.rxcf[A.i];
        const float rxc_[3] = {rc4.x, rc4.y, rc4.z};
        const float rfc[3] = {-r[0], -r[1], -r[2]};
        float vw[3];
        colloid_noslip<float, D>(k, si - 1, rxc_, rfc, vj, vw);
#pragma unroll
        for (int a = 0; a < D; ++a) vi[a] = vw[a];
      }
      if (NNW) {
        Ai = Aj;
        Bi = Bj;
#pragma unroll
        for (int cc = 0; cc <= D2; ++cc) qie[cc] = qj[cc];
      } else {
        Ai = boundary_A<float>(k.rhs_force_type, cj.w, A.ci.y);
      }
    }
  }
  const float gw = kernel_gradw<float>(k, d);
  float vij[3];
#pragma unroll
  for (int a = 0; a < D; ++a) vij[a] = vi[a] - vj[a];
  float z[6];
  if (noise) pair_draw<D>(k.rhs_force_type, k.rk, step, A.pidi, __float_as_int(vj4.w), z);
  float pa[3];
  pair_force<float, D>(k, r, inv_d, vij, Ai, Bi, Aj, Bj, gw, noise, z, inv_sqdt, pa);
  if (NNW) nn_pair<D, NNW, STRESS>(A, qie, qj, r, vi, vj, gw, inv_d, pa);
  float si_s, sj_s;
  pair_scales<float>(k.rhs_force_type, A.ci.z, cj.z, si_s, sj_s);
#pragma unroll
  for (int a = 0; a < D; ++a) pa[a] *= si_s;
  acc_add<D, NNW, STRESS>(A, pa, r);
}

// FP32-mixed force sweep over the density sweep's compact pair list,
// S lanes per particle (lane l takes the list entries q = l mod S); the
// lanes' sums are added in lane order by the first lane, which runs the
// epilogue.
template <int D, bool NNW, bool STRESS, int S>
__global__ void __launch_bounds__(kReuseTPB)
    k_force_list(Consts k, const int* __restrict__ cell_start, const int* __restrict__ cell_of,
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
  const uint32_t step = step_ptr ? (uint32_t)*step_ptr : step_arg;
  __shared__ int s_start[kMaxStencil * kReuseTPB];
  __shared__ float4 s_slot[kSlotTable];
  const int n = k.n;
  const bool noise = k.noise != 0;
  fill_slot_offsets<D>(k, s_slot);
  __syncthreads();
  const int gt = blockIdx.x * kReuseTPB + threadIdx.x;
  const int i = gt / S, lane_s = gt % S;
  if (i >= n) return;  // the S lanes of a particle leave together
  const int celli = cell_of[i];
  build_lane_table<D, kReuseTPB, false>(k, celli, cell_start, s_start, nullptr);
  const float4* slot_tab = slot_table(k, s_slot, celli);
  const float* qq = (const float*)nn.qq;
  ForceAcc<D, NNW, STRESS> A;
  A.i = i;
  A.oi = off[i];
  A.si = __float_as_int(A.oi.w);
  A.v4i = vf[i];
  A.pidi = __float_as_int(A.v4i.w);
  A.ci = pcf[i];
  A.wdi = (k.wall_axis >= 0) ? wd[i] : make_float2(0.f, 0.f);
#pragma unroll
  for (int cc = 0; cc < D2; ++cc) A.L[cc] = 0.f;
  if (NNW) {
#pragma unroll
    for (int cc = 0; cc <= D2; ++cc) A.qi[cc] = qq[(size_t)cc * n + i];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) A.acc[a] = A.comp[a] = 0.f;
  if (STRESS) {
#pragma unroll
    for (int a = 0; a < 9; ++a) A.sacc[a] = 0.f;
  }
  const int nc = ncount[i];
  const int kff = nc & 0xffff, ntot = kff + (nc >> 16);
  if (S == 1) {
    // fluid-fluid segment: the next pair's records are gathered while the
    // current pair is computed, the entry after it one step earlier still
    PairData nxt;
    int ent_n = 0;
    if (kff > 0) nxt = load_pair(nl[i], s_start, off, vf, pcf);
    if (kff > 1) ent_n = nl[(size_t)n + i];
    for (int e = 0; e < kff; ++e) {
      const PairData cur = nxt;
      if (e + 1 < kff) {
        nxt = load_pair(ent_n, s_start, off, vf, pcf);
        if (e + 2 < kff) ent_n = nl[(size_t)(e + 2) * n + i];
      }
      pair_fluid<D, NNW, STRESS>(k, A, cur, slot_tab, qq, step, inv_sqdt, noise);
    }
    // wall / colloid segment, from the last row down
    for (int e = kff; e < ntot; ++e) {
      const int ent = nl[(size_t)(cap - 1 - (e - kff)) * n + i];
      pair_general<D, NNW, STRESS>(k, A, ent, s_start, slot_tab, off, vf, pcf, wd, x, qq, ca,
                                   step, inv_sqdt, noise);
    }
  } else {
    for (int e = lane_s; e < ntot; e += S) {
      const int ent = nl[(size_t)cand_row(e, kff, cap) * n + i];
      if (e < kff)
        pair_fluid<D, NNW, STRESS>(k, A, load_pair(ent, s_start, off, vf, pcf), slot_tab, qq,
                                   step, inv_sqdt, noise);
      else
        pair_general<D, NNW, STRESS>(k, A, ent, s_start, slot_tab, off, vf, pcf, wd, x, qq, ca,
                                     step, inv_sqdt, noise);
    }
    // the lanes' sums, added in lane order by lane 0 of the group
    const int base = (threadIdx.x & 31) & ~(S - 1);
    const unsigned gmask = ((1u << S) - 1u) << base;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float part = A.acc[a] - A.comp[a];
      float tot = part;
      for (int q = 1; q < S; ++q) tot += __shfl_sync(gmask, part, base + q);
      A.acc[a] = tot;
      A.comp[a] = 0.f;
    }
    if (NNW) {
#pragma unroll
      for (int cc = 0; cc < D2; ++cc) {
        float tot = A.L[cc];
        for (int q = 1; q < S; ++q) tot += __shfl_sync(gmask, A.L[cc], base + q);
        A.L[cc] = tot;
      }
    }
    if (STRESS) {
#pragma unroll
      for (int a = 0; a < 9; ++a) {
        float tot = A.sacc[a];
        for (int q = 1; q < S; ++q) tot += __shfl_sync(gmask, A.sacc[a], base + q);
        A.sacc[a] = tot;
      }
    }
    if (lane_s != 0) return;
  }
  if (STRESS) {
#pragma unroll
    for (int a = 0; a < D2; ++a) st[(size_t)a * n + i] = (double)A.sacc[a];
  }
  const double4_32a xi4 = x[i];
  const double xi[3] = {xi4.x, xi4.y, xi4.z};
  if (NNW) {
    double Ld[D2];
#pragma unroll
    for (int cc = 0; cc < D2; ++cc) Ld[cc] = (double)A.L[cc];
    nn_epilogue<D>(k, nn, i, Ld, fuse_mode, dt);
  }
  force_epilogue<D>(k, i, A.si, xi, (double)A.acc[0], (double)A.acc[1],
                    D == 3 ? (double)A.acc[2] : 0.0, fuse_mode, dt, v, f, v_out, err);
}

}  // namespace

int density_list(Handle* h, bool with_pressure) {
  Consts& k = h->k;
  cudaStream_t s = h->stream;
  const int n = (int)h->n;
  if (cuda_check(h, cudaMemsetAsync(h->d_stats, 0, sizeof(int) * 4, s), "memset stats") ||
      cuda_check(h, cudaMemsetAsync(h->d_pairs, 0, sizeof(unsigned long long), s), "memset pairs"))
    return MCFG_ECUDA;
  if (n == 0) return MCFG_OK;
  const bool split = n < kSplitBelow;
  const int S = split ? 4 : 1;
  const int g = (int)(((int64_t)n * S + kReuseTPB - 1) / kReuseTPB);
#define LAUNCH(DD, SS)                                                                          \
  k_density_list<DD, SS><<<g, kReuseTPB, 0, s>>>(                                              \
      k, h->cell_start, h->cell_of, h->off, h->x, h->v, h->m, h->pid, h->vl, h->vcount, h->vcap, \
      h->nl, h->ncount, h->neigh_cap, h->rho, h->pr, h->pcf, h->vf, with_pressure ? 1 : 0,      \
      h->d_err, h->d_stats, h->d_pairs, NN{h->ct, h->act, h->vgt, h->qq},                       \
      CollArgs{h->v, h->rxc, h->rxcf})
  if (k.d == 3) {
    if (split) LAUNCH(3, 4); else LAUNCH(3, 1);
  } else {
    if (split) LAUNCH(2, 4); else LAUNCH(2, 1);
  }
#undef LAUNCH
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "density launch") ? MCFG_ECUDA : MCFG_OK;
}

int force_list(Handle* h, int64_t step, int fuse_mode, double dt) {
  Consts& k = h->k;
  cudaStream_t s = h->stream;
  const int n = (int)h->n;
  if (k.noise && !(dt > 0.0)) return set_error(h, MCFG_EINVAL, "random force needs dt > 0");
  const float inv_sqdt = (k.noise && dt > 0.0) ? (float)(1.0 / sqrt(dt)) : 0.0f;
  const int64_t* step_ptr = h->graph_capturing ? h->d_step : nullptr;
  const NN nn{h->ct, h->act, h->vgt, h->qq};
  const CollArgs ca{h->v, h->rxc, h->rxcf};
  if (n > 0) {
    const bool split = n < kSplitBelow;
    const int S = split ? 4 : 1;
    const int g = (int)(((int64_t)n * S + kReuseTPB - 1) / kReuseTPB);
#define LAUNCH(DD, NW, ST, SS)                                                                  \
  k_force_list<DD, NW, ST, SS><<<g, kReuseTPB, 0, s>>>(                                        \
      k, h->cell_start, h->cell_of, h->nl, h->ncount, h->neigh_cap, h->off, h->x, h->v,         \
      h->pcf, h->vf, h->wd, h->f, h->st, fuse_mode, dt, h->v2, (uint32_t)step, step_ptr,        \
      inv_sqdt, h->d_err, nn, ca)
#define PICK_S(DD, NW, ST)         \
  do {                             \
    if (split) LAUNCH(DD, NW, ST, 4); \
    else LAUNCH(DD, NW, ST, 1);    \
  } while (0)
#define PICK_ST(DD, NW)                  \
  do {                                   \
    if (k.stress) PICK_S(DD, NW, true);  \
    else PICK_S(DD, NW, false);          \
  } while (0)
    if (k.d == 3) {
      if (k.newtonian) PICK_ST(3, false); else PICK_ST(3, true);
    } else {
      if (k.newtonian) PICK_ST(2, false); else PICK_ST(2, true);
    }
#undef PICK_ST
#undef PICK_S
#undef LAUNCH
    h->launches++;
    if (cuda_check(h, cudaGetLastError(), "force launch")) return MCFG_ECUDA;
  }
  if (fuse_mode == kForceBodyKick) std::swap(h->v, h->v2);
  return MCFG_OK;
}

}  // namespace mcfg
