// pair_common.cuh -- cell-neighbour table and exact FP64 pair separation
// shared by the pair sweeps of the right-hand side and of its adjoint.
#pragma once
#include "mcfg_internal.cuh"

namespace mcfg {

constexpr int kWarpsPerBlock = 4;

struct NbTable {
  int start[kMaxStencil];
  int count[kMaxStencil];
  int shift[kMaxStencil];  // shift word of the slot (kLeUp / kLeDown, 2 bits per axis)
  float4 o[kMaxStencil];   // FP32 slot offset (neighbour cell origin - home cell
                           // origin, Lees-Edwards shift included), w = the
                           // neighbour's x-velocity jump across a Lees-Edwards face
};

// Lees-Edwards state of a home cell row: 1 top row (its y+ neighbours are
// bottom-row particles imaged above the y+ face, ppm_bcdef_le_y.inc), 2
// bottom row (its y- neighbours are top-row particles; the pair is MCF's
// top particle with this particle's image above), 0 otherwise.
__device__ __forceinline__ int le_state(const Consts& k, int cy) {
  if (!k.le) return 0;
  return (cy == k.nm[1] - 1) ? 1 : (cy == 0 ? 2 : 0);
}

// Cell offsets of stencil slot s: the 27 (9) cells -1..1 per axis, then,
// in a Lees-Edwards crossing row, the fourth x cell (offset 2) of the row
// across the face, z -1..1.
template <int D>
__device__ __forceinline__ void slot_dirs(int s, int st, int* o) {
  constexpr int NS0 = (D == 3) ? 27 : 9;
  if (s < NS0) {
    o[0] = s % 3 - 1;
    o[1] = (s / 3) % 3 - 1;
    o[2] = s / 9 - 1;
  } else {
    o[0] = 2;
    o[1] = (st == 1) ? 1 : -1;
    o[2] = (D == 3) ? s - NS0 - 1 : 0;
  }
}

// Neighbour cell of home cell c (coordinates) in slot s, -1 if none, and
// the slot's shift word.  Periodic axes wrap with an image bit; across a
// Lees-Edwards face the x cells of the row are those of the images' x
// range: le_cu + 1 cells to the left (top row) or le_cl - 1 to the right
// (bottom row) of the home cell, four of them, wrapped along x.
template <int D>
__device__ __forceinline__ int slot_cell(const Consts& k, const int* c, int s, int st, int& sh) {
  constexpr int NS0 = (D == 3) ? 27 : 9;
  sh = 0;
  if (s >= NS0 && st == 0) return -1;
  int o[3];
  slot_dirs<D>(s, st, o);
  const bool cross = st != 0 && o[1] == ((st == 1) ? 1 : -1);
  int nc = 0, stride = 1;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    int t2;
    if (a == 0 && cross) {
      t2 = (st == 1) ? c[0] - k.le_cu + o[0] : c[0] + k.le_cl + o[0];
      t2 %= k.nm[0];
      if (t2 < 0) t2 += k.nm[0];
    } else {
      t2 = c[a] + o[a];
      const bool wraps = k.periodic[a] || (a == 1 && cross);
      if (t2 < 0) {
        if (!wraps) return -1;
        t2 += k.nm[a];
        sh |= 2 << (2 * a);
      } else if (t2 >= k.nm[a]) {
        if (!wraps) return -1;
        t2 -= k.nm[a];
        sh |= 1 << (2 * a);
      }
    }
    nc += t2 * stride;
    stride *= k.nm[a];
  }
  if (cross) sh |= (st == 1) ? kLeUp : kLeDown;
  return nc;
}

// FP32 offset of slot s for a home cell in Lees-Edwards state st: the
// neighbour cell's origin (its image's, across a Lees-Edwards face) minus
// the home cell's; w = the x-velocity jump added to the neighbour (+dv for
// an image above, -dv when the home particle is the one imaged above).
// Between list rebuilds the images have moved by le_dS since the cells of
// the row were chosen: + le_dS for the neighbour's image above, - le_dS
// when it is the home particle's (0 without list reuse, leaving the
// offset unchanged).
template <int D>
__device__ __forceinline__ float4 slot_offset(const Consts& k, int s, int st) {
  int o[3];
  slot_dirs<D>(s, st, o);
  float ox = (float)o[0] * k.csf[0], w = 0.0f;
  if (st != 0 && o[1] == ((st == 1) ? 1 : -1)) {
    const double base = __dmul_rn((double)o[0] - ((st == 1) ? k.le_pu : k.le_pl), k.cs[0]);
    ox = (float)__dadd_rn(base, (st == 1) ? k.le_dS : -k.le_dS);
    w = (float)((st == 1) ? k.le_dv : -k.le_dv);
  }
  return make_float4(ox, (float)o[1] * k.csf[1], D == 3 ? (float)o[2] * k.csf[2] : 0.0f, w);
}

template <int D>
__device__ __forceinline__ void cell_coords(const Consts& k, int cell, int* c) {
  c[0] = c[1] = c[2] = 0;
  int rem = cell;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    c[a] = rem % k.nm[a];
    rem /= k.nm[a];
  }
}

// cell == k.ncell is the bin of particles without a real cell: it has no
// neighbours (PPM gives such particles no box, ppm_util_rank3d.F90:463-473).
template <int D>
__device__ __forceinline__ void build_table(const Consts& k, int cell,
                                            const int* __restrict__ cell_start, NbTable& t) {
  constexpr int CENTER = (D == 3) ? 13 : 4;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if (cell == k.ncell) {
    if (lane < k.ns) {
      const int s0 = cell_start[cell];
      t.start[lane] = s0;
      t.count[lane] = (lane == CENTER) ? cell_start[cell + 1] - s0 : 0;
      t.shift[lane] = 0;
      t.o[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncwarp();
    return;
  }
  if (lane < k.ns) {
    int c[3];
    cell_coords<D>(k, cell, c);
    const int st = le_state(k, c[1]);
    int sh;
    const int nc = slot_cell<D>(k, c, lane, st, sh);
    if (nc >= 0) {
      const int s0 = cell_start[nc];
      t.start[lane] = s0;
      t.count[lane] = cell_start[nc + 1] - s0;
    } else {
      t.start[lane] = 0;
      t.count[lane] = 0;
    }
    t.shift[lane] = sh;
    t.o[lane] = slot_offset<D>(k, lane, st);
  }
  __syncwarp();
}

// gfortran's MODULO for reals (p > 0): fmod, exact, plus p when the
// remainder is negative
__device__ __forceinline__ double f_modulo(double a, double p) {
  double r = fmod(a, p);
  if (r < 0.0) r = __dadd_rn(r, p);
  return r;
}

// a - b along a periodic axis of period L, the image taken like PPM's
// ghosts: the smaller coordinate at + L when they are more than L/2 apart
__device__ __forceinline__ double wrap_sep(double a, double b, double L) {
  const double d = __dsub_rn(a, b);
  if (d > 0.5 * L) return __dsub_rn(a, __dadd_rn(b, L));
  if (d < -0.5 * L) return __dsub_rn(__dadd_rn(a, L), b);
  return d;
}

// FP64 separation of MCF's pair (ip, jp) where jp may be a periodic image:
// PPM creates images only at x+L (symmetry=T), so a pair across a boundary
// is evaluated as (x_upper) - (x_lower + L) per axis.  Rounded exactly like
// rij = x(ip) - x(jp) with the ghost coordinate x + len_phys
// (ppm_bcdef_periodic_x.inc), and d2 = ((r0*r0 + r1*r1) + r2*r2) without
// fused multiply-add (pp_interaction.inc:37-50).  Across a Lees-Edwards
// face the bottom particle's image above has x = MODULO(x + shear_length,
// L_x) (ppm_bcdef_le_y.inc), then an x image as PPM's periodic ghosts give
// it (ppm_map_part_ghost_get.F90:776-910 makes them after the Lees-Edwards
// ones).
template <int D>
__device__ __forceinline__ double exact_sep(const Consts& k, const double* xi, const double* xj,
                                            int sh, double* r) {
  double d2 = 0.0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int s = (sh >> (2 * a)) & 3;
    double ra;
    if (a == 0 && (sh & (kLeUp | kLeDown))) {
      if (sh & kLeUp)
        ra = wrap_sep(xi[0], f_modulo(__dadd_rn(xj[0], k.le_S), k.len[0]), k.len[0]);
      else
        ra = wrap_sep(f_modulo(__dadd_rn(xi[0], k.le_S), k.len[0]), xj[0], k.len[0]);
    } else if (s == 1) {
      ra = __dsub_rn(xi[a], __dadd_rn(xj[a], k.len[a]));
    } else if (s == 2) {
      ra = __dsub_rn(__dadd_rn(xi[a], k.len[a]), xj[a]);
    } else {
      ra = __dsub_rn(xi[a], xj[a]);
    }
    r[a] = ra;
    d2 = (a == 0) ? __dmul_rn(ra, ra) : __dadd_rn(d2, __dmul_rn(ra, ra));
  }
  return d2;
}

// face velocity of a wall particle (sid = -face) after the step,
// particles_set_boundary_velocity.F90, selected with constant indices
template <int D>
__device__ __forceinline__ void wall_end_velocity(const Consts& k, int sid, double* vs) {
  const int fi = -sid - 1;
#pragma unroll
  for (int f = 0; f < 6; ++f)
    if (f == fi) {
#pragma unroll
      for (int a = 0; a < D; ++a) vs[a] = k.wall_v_end[f][a];
    }
}

// FP64 velocities of a pair across a Lees-Edwards face: the image above
// the y+ face moves with + le_dv along x (particles_set_boundary_ghost_
// velocity.F90), added before the difference as MCF's ghost velocity is
template <typename T>
__device__ __forceinline__ void le_velocity(const Consts& k, int sh, T* vi, T* vj) {
  if (sh & kLeUp) vj[0] = vj[0] + (T)k.le_dv;
  if (sh & kLeDown) vi[0] = vi[0] + (T)k.le_dv;
}

}  // namespace mcfg

namespace mcfg {

// Per-thread neighbour-cell table for thread-per-particle sweeps: slot s of
// thread t lives at s * TPB + t (conflict-free).  Same slots, starts and
// periodic image bits as build_table, so the neighbour-list entries
// slot<<11 | local index decode the same way.
template <int D, int TPB, bool SHIFT = true>
__device__ __forceinline__ void build_lane_table(const Consts& k, int cell,
                                                 const int* __restrict__ cell_start,
                                                 int* __restrict__ s_start,
                                                 int* __restrict__ s_shift) {
  constexpr int NS0 = (D == 3) ? 27 : 9;
  constexpr int CENTER = (D == 3) ? 13 : 4;
  const int t = threadIdx.x;
  if (cell == k.ncell) {
    for (int s = 0; s < k.ns; ++s) {
      s_start[s * TPB + t] = (s == CENTER) ? cell_start[cell] : 0;
      if (SHIFT) s_shift[s * TPB + t] = 0;
    }
    return;
  }
  int c[3];
  cell_coords<D>(k, cell, c);
  const int st = le_state(k, c[1]);
#pragma unroll
  for (int s = 0; s < NS0; ++s) {
    int sh;
    const int nc = slot_cell<D>(k, c, s, st, sh);
    s_start[s * TPB + t] = (nc >= 0) ? cell_start[nc] : 0;
    if (SHIFT) s_shift[s * TPB + t] = sh;
  }
  for (int s = NS0; s < k.ns; ++s) {
    int sh;
    const int nc = slot_cell<D>(k, c, s, st, sh);
    s_start[s * TPB + t] = (nc >= 0) ? cell_start[nc] : 0;
    if (SHIFT) s_shift[s * TPB + t] = sh;
  }
}

}  // namespace mcfg
