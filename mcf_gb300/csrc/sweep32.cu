// sweep32.cu -- FP32-mixed density sweep over the candidate list.
//
// With neighbour-list reuse, a rebuild lists for every particle the
// candidates within rc + skin (k_verlet_build, pair_kernels.cu), partitioned
// by species: the fluid partners of a fluid particle first, from row 0 up;
// every other pair (wall, colloid, or a boundary particle's own pairs) from
// the last row down.  vcount packs both counts (fluid-fluid | other << 16).
//
// Each step the density sweep re-tests every candidate exactly (the FP32
// test of the per-step scan, same operation order), sums the number
// density, and writes the step's pairs as a compact list in the same two
// segments (nl rows from 0 up and from the last row down, ncount =
// fluid-fluid | other << 16): coalesced rows and no holes.  The force sweep
// (k_force32, pair_kernels.cu) walks that list, the fluid-fluid pairs first.
//
// Reference: particles_compute_density.F90:578-867.
#include "mcfg_internal.cuh"
#include "pair_common.cuh"
#include "sph.cuh"
#include "sweep_common.cuh"

namespace mcfg {

namespace {

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

}  // namespace mcfg
