// pair_common.cuh -- cell-neighbour table and exact FP64 pair separation
// shared by the pair sweeps of the right-hand side and of its adjoint.
#pragma once
#include "mcfg_internal.cuh"

namespace mcfg {

constexpr int kWarpsPerBlock = 4;

struct NbTable {
  int start[kMaxStencil];
  int count[kMaxStencil];
  int shift[kMaxStencil];  // 2 bits per axis: 0 none, 1 image at x+L, 2 at x-L
  float4 o[kMaxStencil];   // stencil offset x cell side (FP32), per slot
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
      t.o[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
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
    t.o[lane] = make_float4((float)o[0] * k.csf[0], (float)o[1] * k.csf[1],
                            D == 3 ? (float)o[2] * k.csf[2] : 0.0f, 0.0f);
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

}  // namespace mcfg

namespace mcfg {

// Per-thread neighbour-cell table for thread-per-particle sweeps: slot s of
// thread t lives at s * TPB + t (conflict-free).  Same slots, starts and
// periodic image bits as build_table, so the neighbour-list entries
// slot<<11 | local index decode the same way.
template <int D, int TPB>
__device__ __forceinline__ void build_lane_table(const Consts& k, int cell,
                                                 const int* __restrict__ cell_start,
                                                 int* __restrict__ s_start,
                                                 int* __restrict__ s_shift) {
  constexpr int NS = (D == 3) ? 27 : 9;
  constexpr int CENTER = (D == 3) ? 13 : 4;
  const int t = threadIdx.x;
  if (cell == k.ncell) {
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      s_start[s * TPB + t] = (s == CENTER) ? cell_start[cell] : 0;
      s_shift[s * TPB + t] = 0;
    }
    return;
  }
  int c[3] = {0, 0, 0};
  int rem = cell;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    c[a] = rem % k.nm[a];
    rem /= k.nm[a];
  }
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const int o[3] = {s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1};
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
    s_start[s * TPB + t] = ok ? cell_start[nc] : 0;
    s_shift[s * TPB + t] = sh;
  }
}

}  // namespace mcfg
