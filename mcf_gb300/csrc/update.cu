// update.cu -- per-particle O(N) kernels of the velocity-Verlet step and the
// FP64 global reductions.
//
// Reference: particles_integrate_velocity.F90:84-94, particles_integrate_
// position.F90:82-111, particles_adjust_particles.F90:137-389,
// particles_apply_body_force.F90:96-353, marching_integrate_VV.F90:303-322,
// statistic_compute_statistic.F90:230-303.
#include "mcfg_internal.cuh"
#include "pair_common.cuh"
#include "sph.cuh"

namespace mcfg {

// Periodic wrap of one coordinate, particles_adjust_particles.F90:150-161,
// 268-279: x < min -> x + length; then x >= max -> x - length.  Solid-wall
// faces only clamp wall particles to the total domain.
__device__ __forceinline__ void wrap_axis(const Consts& k, int a,
                                          int sid, double& x, double& v) {
  if (x < k.min_phys[a]) {
    if (k.bc_lo[a] == MCFG_BC_PERIODIC) {
      x = __dadd_rn(x, k.len[a]);
    } else if (k.bc_lo[a] == MCFG_BC_WALL_SOLID) {
      if (sid < 0 && x < k.xmin[a]) {
        x = k.xmin[a];
        v = 0.0;
      }
    }
  }
  if (x >= k.max_phys[a]) {
    if (k.bc_hi[a] == MCFG_BC_PERIODIC) {
      x = __dsub_rn(x, k.len[a]);
    } else if (k.bc_hi[a] == MCFG_BC_WALL_SOLID) {
      if (sid < 0 && x > k.xmax[a]) {
        x = k.xmax[a] - k.machine_zero;
        v = 0.0;
      }
    }
  }
}

// particles_adjust_particles.F90:228-257, 352-381: a particle leaving
// through a Lees-Edwards y face re-enters through the other one with the
// other coordinates MODULO(x - shear_length, L) (x: shear_length(x, y-) =
// -S, (x, y+) = S; z: 0) and the x velocity jump shear_v(y+/-) -
// shear_v(y-/+).  MCF then checks no further axis for it (EXIT).
template <int D>
__device__ __forceinline__ bool le_wrap(const Consts& k, double* xs, double* vs) {
  double sl;
  if (xs[1] < k.min_phys[1]) {
    xs[1] = __dadd_rn(xs[1], k.len[1]);
    sl = -k.le_S;
    vs[0] = __dadd_rn(vs[0], k.le_dv);
  } else if (xs[1] >= k.max_phys[1]) {
    xs[1] = __dsub_rn(xs[1], k.len[1]);
    sl = k.le_S;
    vs[0] = __dadd_rn(vs[0], -k.le_dv);
  } else {
    return false;
  }
  xs[0] = f_modulo(__dsub_rn(xs[0], sl), k.len[0]);
  if (D == 3) xs[2] = f_modulo(xs[2], k.len[2]);
  return true;
}

// flags: 1 half kick, 2 drift, 4 wrap, 8 conformation-tensor half step,
// 16 end of a VV step (wall particles take their face's velocity).
// The arithmetic is rounded exactly like MCF's: v + (lambda*f)*dt,
// x + v*dt, ct + act*dt*lambda (no fused multiply-add).  With solid walls
// the drift also moves wall particles with their velocity
// (particles_integrate_boundary_position.F90, marching_integrate_VV.F90:797).
template <int D>
__global__ void k_integrate(Consts k, int flags, double dt, double lambda,
                            double4_32a* __restrict__ x, double4_32a* __restrict__ v,
                            const double4_32a* __restrict__ f, const int* __restrict__ sid,
                            double* __restrict__ ct, const double* __restrict__ act) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  if ((flags & 8) && ct != nullptr) {
    // particles_integrate_ct.F90:66-68 (all real particles)
#pragma unroll
    for (int cc = 0; cc < D * D; ++cc) {
      const size_t q = (size_t)cc * k.n + i;
      ct[q] = __dadd_rn(ct[q], __dmul_rn(__dmul_rn(act[q], dt), 0.5));
    }
  }
  const int s = sid[i];
  double4_32a xv = x[i], vv = v[i];
  double xs[3] = {xv.x, xv.y, xv.z}, vs[3] = {vv.x, vv.y, vv.z};
  if (s == 0) {
    if (flags & 1) {
      const double4_32a fv = f[i];
      const double fs[3] = {fv.x, fv.y, fv.z};
#pragma unroll
      for (int a = 0; a < D; ++a) vs[a] = __dadd_rn(vs[a], __dmul_rn(__dmul_rn(lambda, fs[a]), dt));
    }
    if (flags & 2) {
#pragma unroll
      for (int a = 0; a < D; ++a) xs[a] = __dadd_rn(xs[a], __dmul_rn(vs[a], dt));
    }
  } else if (s < 0 && k.walls) {
    if (flags & 2) {
#pragma unroll
      for (int a = 0; a < D; ++a) xs[a] = __dadd_rn(xs[a], __dmul_rn(vs[a], dt));
    }
    if (flags & 16) wall_end_velocity<D>(k, s, vs);
  }
  if (flags & 4) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      if (a == 1 && k.le) {
        if (s >= 0 && le_wrap<D>(k, xs, vs)) break;
      } else {
        wrap_axis(k, a, s, xs[a], vs[a]);
      }
    }
  }
  x[i] = make_double4_32a(xs[0], xs[1], D == 3 ? xs[2] : 0.0, 0.0);
  v[i] = make_double4_32a(vs[0], vs[1], D == 3 ? vs[2] : 0.0, 0.0);
}

template <int D>
__global__ void k_body_force(Consts k, const double4_32a* __restrict__ x, double4_32a* __restrict__ f,
                             const int* __restrict__ sid) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n || sid[i] != 0) return;
  double4_32a fv = f[i];
  const double4_32a xv = x[i];
  const double* g = k.body_force;
  if (k.body_force_type == 1) {
    if (fabs(g[0]) > k.machine_zero) fv.x = fv.x + g[0];
    if (fabs(g[1]) > k.machine_zero) fv.y = fv.y + g[1];
    if (D == 3 && fabs(g[2]) > k.machine_zero) fv.z = fv.z + g[2];
  } else if (k.body_force_type == 2) {
    if (fabs(g[0]) > k.machine_zero) {
      const double half = k.max_phys[D - 1] * 0.5;
      const double xl = (D == 3) ? xv.z : xv.y;
      if (xl < half)
        fv.x = fv.x + g[0];
      else if (xl > half)
        fv.x = fv.x - g[0];
    }
  } else if (k.body_force_type == 3) {
    if (fabs(g[0]) > k.machine_zero) {
      const double kw = 2.0 * kPi / (k.max_phys[1] - k.min_phys[1]);
      fv.x = fv.x + g[0] * sin(kw * xv.y);
    }
  }
  f[i] = fv;
}

// ---- FP64 reductions: fixed-order two-pass block sums (deterministic) ----
constexpr int kRedThreads = 256;
constexpr int kRedVals = 13;  // ke, mom[3], stress[9]

template <int D>
__global__ void k_stats_partial(Consts k, const double4_32a* __restrict__ v,
                                const double* __restrict__ m, const int* __restrict__ sid,
                                const double* __restrict__ st, const int* __restrict__ hidx,
                                int64_t owned, double* __restrict__ part) {
  __shared__ double sm[kRedVals][kRedThreads];
  double acc[kRedVals];
#pragma unroll
  for (int q = 0; q < kRedVals; ++q) acc[q] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.n; i += gridDim.x * blockDim.x) {
    if (hidx[i] >= owned) continue;  // a subdomain's ghost copy
    const int s = sid[i];
    if (s == 0) {
      const double4_32a vv = v[i];
      const double mi = m[i];
      double v2 = vv.x * vv.x + vv.y * vv.y;
      if (D == 3) v2 += vv.z * vv.z;
      acc[0] += 0.5 * mi * v2;
      acc[1] += mi * vv.x;
      acc[2] += mi * vv.y;
      if (D == 3) acc[3] += mi * vv.z;
    }
    if (k.stress && s >= 0) {
#pragma unroll
      for (int a = 0; a < D * D; ++a) acc[4 + a] += st[(size_t)a * k.n + i];
    }
  }
#pragma unroll
  for (int q = 0; q < kRedVals; ++q) sm[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int q = 0; q < kRedVals; ++q) sm[q][threadIdx.x] += sm[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < kRedVals; ++q) part[(size_t)blockIdx.x * kRedVals + q] = sm[q][0];
}

__global__ void k_stats_final(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  const int q = threadIdx.x;
  if (q >= kRedVals) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[(size_t)b * kRedVals + q];
  out[q] = s;
}

// particles_collect_colloid_interaction.F90:93-136: one warp per colloid
// sums m f and r x (m f) over its boundary particles in a fixed order.
template <int D>
__global__ void k_colloid_drag(Consts k, const int* __restrict__ cstart,
                               const int* __restrict__ cmem, const int* __restrict__ slot_of,
                               const double4_32a* __restrict__ x,
                               const double4_32a* __restrict__ f, const double* __restrict__ m,
                               double* __restrict__ out) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= k.ncoll) return;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int q = cstart[c] + lane; q < cstart[c + 1]; q += 32) {
    const int s = slot_of[cmem[q]];
    const double4_32a fv = f[s], xv = x[s];
    const double mi = m[s];
    const double F[3] = {fv.x * mi, fv.y * mi, D == 3 ? fv.z * mi : 0.0};
    const double xs[3] = {xv.x, xv.y, xv.z};
    double rx[3] = {0.0, 0.0, 0.0};
    colloid_rx<D>(k, xs, c, rx);
    double T[3];
    cross3t<double>(rx, F, T);
    for (int a = 0; a < 3; ++a) {
      acc[a] += F[a];
      acc[3 + a] += T[a];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int a = 0; a < 6; ++a) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], o);
  if (lane == 0)
    for (int a = 0; a < 6; ++a) out[(size_t)c * 6 + a] = acc[a];
}

// Boundary particles follow their colloid (particles_compute_colloid_
// relative_position.F90 then _absolute_position.F90): relative to the
// nearest image of the old centre, turned by the step's rotation matrix
// (rot[9c + i + 3j] = R(i,j)), put at the new centre in the same periodic
// image as before (so list reuse sees a small displacement).  One warp per
// colloid; coll still holds the old centres.
template <int D>
__global__ void k_colloid_move(Consts k, const int* __restrict__ cstart,
                               const int* __restrict__ cmem, const int* __restrict__ slot_of,
                               const double* __restrict__ xnew, const double* __restrict__ rot,
                               double4_32a* __restrict__ x) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= k.ncoll) return;
  const double* cd = k.coll + (size_t)c * 12;
  for (int q = cstart[c] + lane; q < cstart[c + 1]; q += 32) {
    const int s = slot_of[cmem[q]];
    const double4_32a xv = x[s];
    const double xs[3] = {xv.x, xv.y, xv.z};
    double rx[3] = {0.0, 0.0, 0.0};
    colloid_rx<D>(k, xs, c, rx);
    double rb[3] = {rx[0], rx[1], rx[2]};
    if (k.coll_rotate && rot != nullptr) {
#pragma unroll
      for (int a = 0; a < D; ++a) {
        double t = 0.0;
#pragma unroll
        for (int b = 0; b < D; ++b)
          t = __dadd_rn(t, __dmul_rn(rot[(size_t)c * 9 + a + 3 * b], rx[b]));
        rb[a] = t;
      }
    }
    double xo[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int a = 0; a < D; ++a) {
      // the old centre image the particle was taken against: xs - rx
      const double img = (xs[a] - rx[a]) - cd[a];
      double xn = __dadd_rn(rb[a], xnew[(size_t)c * D + a]);
      if (k.periodic[a] && fabs(img) > 0.5 * k.len[a])
        xn = __dadd_rn(xn, img > 0.0 ? k.len[a] : -k.len[a]);
      xo[a] = xn;
    }
    x[s] = make_double4_32a(xo[0], xo[1], D == 3 ? xo[2] : 0.0, 0.0);
  }
}

int colloid_move(Handle* h, const double* d_xnew, const double* d_rot) {
  const int nc = h->k.ncoll;
  if (nc == 0 || !(h->k.coll_translate || h->k.coll_rotate)) return MCFG_OK;
  const int warps_per_block = 4;
  const int g = (nc + warps_per_block - 1) / warps_per_block;
  if (h->k.d == 3)
    k_colloid_move<3><<<g, 32 * warps_per_block, 0, h->stream>>>(
        h->k, h->coll_start, h->coll_mem, h->slot_of, d_xnew, d_rot, h->x);
  else
    k_colloid_move<2><<<g, 32 * warps_per_block, 0, h->stream>>>(
        h->k, h->coll_start, h->coll_mem, h->slot_of, d_xnew, d_rot, h->x);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "colloid move launch") ? MCFG_ECUDA : MCFG_OK;
}

// the drag and torque sums of every colloid into coll_out [nc][6]
int colloid_drag_launch(Handle* h) {
  const int nc = h->k.ncoll, d = h->k.d;
  if (nc == 0) return MCFG_OK;
  const int warps_per_block = 4;
  const int g = (nc + warps_per_block - 1) / warps_per_block;
  if (d == 3)
    k_colloid_drag<3><<<g, 32 * warps_per_block, 0, h->stream>>>(
        h->k, h->coll_start, h->coll_mem, h->slot_of, h->x, h->f, h->m, h->coll_out);
  else
    k_colloid_drag<2><<<g, 32 * warps_per_block, 0, h->stream>>>(
        h->k, h->coll_start, h->coll_mem, h->slot_of, h->x, h->f, h->m, h->coll_out);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "colloid drag launch") ? MCFG_ECUDA : MCFG_OK;
}

int colloid_drag(Handle* h, double* drag, double* torque) {
  const int nc = h->k.ncoll, d = h->k.d;
  if (nc == 0) return MCFG_OK;
  int rc = colloid_drag_launch(h);
  if (rc) return rc;
  std::vector<double> buf((size_t)nc * 6);
  if (cuda_check(h, cudaMemcpyAsync(buf.data(), h->coll_out, sizeof(double) * buf.size(),
                                    cudaMemcpyDeviceToHost, h->stream),
                 "drag copy") ||
      cuda_check(h, cudaStreamSynchronize(h->stream), "drag sync"))
    return MCFG_ECUDA;
  for (int c = 0; c < nc; ++c) {
    for (int a = 0; a < d; ++a)
      if (drag) drag[(size_t)c * d + a] = buf[(size_t)c * 6 + a];
    for (int a = 0; a < 3; ++a)
      if (torque) torque[(size_t)c * 3 + a] = buf[(size_t)c * 6 + 3 + a];
  }
  return MCFG_OK;
}

// List-reuse form of the first half of a VV step: ct half step, kick and
// drift as k_integrate, positions left unwrapped (the candidate list and its
// periodic images stay valid until the next rebuild, which wraps), the FP32
// cell offsets and wall distances refreshed against the rebuild cell, and the
// rebuild flag raised when a particle has moved more than skin/2 (with
// Lees-Edwards faces: from the imposed shear, by more than the bound the
// host derives) or leaves through a Lees-Edwards face.
template <int D>
__global__ void k_kdw_reuse(Consts k, double dt, double4_32a* __restrict__ x,
                            double4_32a* __restrict__ v, const double4_32a* __restrict__ f,
                            const int* __restrict__ sid, double* __restrict__ ct,
                            const double* __restrict__ act, const double4_32a* __restrict__ x_ref,
                            const int* __restrict__ cell_of, float4* __restrict__ off,
                            float2* __restrict__ wd, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool far = false;
  if (i < k.n) {
    if (ct != nullptr) {
#pragma unroll
      for (int cc = 0; cc < D * D; ++cc) {
        const size_t q = (size_t)cc * k.n + i;
        ct[q] = __dadd_rn(ct[q], __dmul_rn(__dmul_rn(act[q], dt), 0.5));
      }
    }
    const int s = sid[i];
    double4_32a xv = x[i];
    if (s == 0) {
      double4_32a vv = v[i];
      const double4_32a fv = f[i];
      double xs[3] = {xv.x, xv.y, xv.z}, vs[3] = {vv.x, vv.y, vv.z};
      const double fs[3] = {fv.x, fv.y, fv.z};
#pragma unroll
      for (int a = 0; a < D; ++a) {
        vs[a] = __dadd_rn(vs[a], __dmul_rn(__dmul_rn(0.5, fs[a]), dt));
        xs[a] = __dadd_rn(xs[a], __dmul_rn(vs[a], dt));
      }
      xv = make_double4_32a(xs[0], xs[1], D == 3 ? xs[2] : 0.0, 0.0);
      x[i] = xv;
      v[i] = make_double4_32a(vs[0], vs[1], D == 3 ? vs[2] : 0.0, 0.0);
    } else if (s < 0 && k.walls) {
      // wall particles drift with their velocity
      const double4_32a vv = v[i];
      xv.x = __dadd_rn(xv.x, __dmul_rn(vv.x, dt));
      xv.y = __dadd_rn(xv.y, __dmul_rn(vv.y, dt));
      if (D == 3) xv.z = __dadd_rn(xv.z, __dmul_rn(vv.z, dt));
      x[i] = xv;
    }
    const double4_32a xr = x_ref[i];
    const double dx = xv.x - xr.x, dy = xv.y - xr.y, dz = (D == 3) ? xv.z - xr.z : 0.0;
    // offsets to the rebuild cell's origin (k_cell_finalize's formula)
    const int cell = cell_of[i];
    double org[3] = {0.0, 0.0, 0.0};
    if (cell < k.ncell) {
      int cq = cell;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const int ca = cq % k.nm[a];
        cq /= k.nm[a];
        org[a] = k.xmin[a] + (double)ca * k.cs[a];
      }
    }
    if (k.le) {
      // Lees-Edwards: the displacement from the shear the faces impose
      // (which moves the images across the faces with their particles); a
      // fluid particle leaving through a y face re-enters at the rebuild
      // (its shift and velocity jump are applied there, in this step, as
      // MCF does)
      const double px = dx - k.le_aff * (xr.y - k.le_y0);
      far = px * px + dy * dy + dz * dz > k.half_skin_le2;
      if (s >= 0 && (xv.y < k.min_phys[1] || xv.y >= k.max_phys[1])) far = true;
    } else {
      far = dx * dx + dy * dy + dz * dz > k.half_skin2;
    }
    float4 of = off[i];
    of.x = (float)(xv.x - org[0]);
    of.y = (float)(xv.y - org[1]);
    of.z = (D == 3) ? (float)(xv.z - org[2]) : 0.0f;
    off[i] = of;
    if (wd != nullptr && k.wall_axis >= 0) {
      const double xa = k.wall_axis == 0 ? xv.x : (k.wall_axis == 1 ? xv.y : xv.z);
      wd[i] = make_float2((float)(xa - k.min_phys[k.wall_axis]),
                          (float)(xa - k.max_phys[k.wall_axis]));
    }
  }
  if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// periodic wrap of every particle before a rebuild (Lees-Edwards re-entry
// through the y faces as k_integrate's); returns at once when no rebuild is
// due
template <int D>
__global__ void k_wrap_gated(Consts k, const int* __restrict__ flag, double4_32a* __restrict__ x,
                             double4_32a* __restrict__ v, const int* __restrict__ sid) {
  if (*flag == 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  double4_32a xv = x[i], vv = v[i];
  double xs[3] = {xv.x, xv.y, xv.z}, vs[3] = {vv.x, vv.y, vv.z};
  const int s = sid[i];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    if (a == 1 && k.le) {
      if (s >= 0 && le_wrap<D>(k, xs, vs)) break;
    } else {
      wrap_axis(k, a, s, xs[a], vs[a]);
    }
  }
  x[i] = make_double4_32a(xs[0], xs[1], D == 3 ? xs[2] : 0.0, 0.0);
  v[i] = make_double4_32a(vs[0], vs[1], D == 3 ? vs[2] : 0.0, 0.0);
}

int wrap_gated(Handle* h) {
  const int n = (int)h->n;
  if (n == 0) return MCFG_OK;
  const int tb = 256, gb = (n + tb - 1) / tb;
  if (h->k.d == 3)
    k_wrap_gated<3><<<gb, tb, 0, h->stream>>>(h->k, h->d_rebuild, h->x, h->v, h->sid);
  else
    k_wrap_gated<2><<<gb, tb, 0, h->stream>>>(h->k, h->d_rebuild, h->x, h->v, h->sid);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "wrap launch") ? MCFG_ECUDA : MCFG_OK;
}

int kick_drift_reuse(Handle* h, double dt) {
  const int n = (int)h->n;
  if (n == 0) return MCFG_OK;
  const int tb = 256, gb = (n + tb - 1) / tb;
  double* ct = h->p.Newtonian ? nullptr : h->ct;
  if (h->k.d == 3)
    k_kdw_reuse<3><<<gb, tb, 0, h->stream>>>(h->k, dt, h->x, h->v, h->f, h->sid, ct, h->act,
                                             h->x_ref, h->cell_of, h->off, h->wd, h->d_rebuild);
  else
    k_kdw_reuse<2><<<gb, tb, 0, h->stream>>>(h->k, dt, h->x, h->v, h->f, h->sid, ct, h->act,
                                             h->x_ref, h->cell_of, h->off, h->wd, h->d_rebuild);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "kick-drift launch") ? MCFG_ECUDA : MCFG_OK;
}

static int launch_integrate(Handle* h, int flags, double dt, double lambda) {
  const int n = (int)h->n;
  if (n == 0) return MCFG_OK;
  const int tb = 256, gb = (n + tb - 1) / tb;
  if (h->k.d == 3)
    k_integrate<3><<<gb, tb, 0, h->stream>>>(h->k, flags, dt, lambda, h->x, h->v, h->f,
                                             h->sid, h->ct, h->act);
  else
    k_integrate<2><<<gb, tb, 0, h->stream>>>(h->k, flags, dt, lambda, h->x, h->v, h->f,
                                             h->sid, h->ct, h->act);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "integrate launch") ? MCFG_ECUDA : MCFG_OK;
}

int integrate_velocity(Handle* h, double dt, double lambda) {
  return launch_integrate(h, 1, dt, lambda);
}
int integrate_position(Handle* h, double dt) { return launch_integrate(h, 2, dt, 0.0); }
int adjust_particles(Handle* h) {
  // a wrap moves particles by a period: the candidate list's images no longer hold
  h->reuse_valid = false;
  h->unwrapped = false;
  return launch_integrate(h, 4, 0.0, 0.0);
}
int kick_ct_half(Handle* h, double dt) {
  return launch_integrate(h, (h->p.Newtonian ? 1 : 9) | 16, dt, 0.5);
}
int kick_drift_wrap(Handle* h, double dt) {
  return launch_integrate(h, h->p.Newtonian ? 7 : 15, dt, 0.5);
}

int apply_body_force(Handle* h) {
  const int n = (int)h->n;
  if (n == 0 || h->k.body_force_type == 0) return MCFG_OK;
  const int tb = 256, gb = (n + tb - 1) / tb;
  if (h->k.d == 3)
    k_body_force<3><<<gb, tb, 0, h->stream>>>(h->k, h->x, h->f, h->sid);
  else
    k_body_force<2><<<gb, tb, 0, h->stream>>>(h->k, h->x, h->f, h->sid);
  h->launches++;
  return cuda_check(h, cudaGetLastError(), "body force launch") ? MCFG_ECUDA : MCFG_OK;
}

int statistics(Handle* h, double* ke, double* mom, double* stress, int64_t owned) {
  const int n = (int)h->n;
  int nb = (n + kRedThreads - 1) / kRedThreads;
  if (nb > 1024) nb = 1024;
  if (nb < 1) nb = 1;
  double* part = h->red;
  double* out = h->red + (size_t)1024 * kRedVals;
  if (h->k.d == 3)
    k_stats_partial<3><<<nb, kRedThreads, 0, h->stream>>>(h->k, h->v, h->m, h->sid, h->st,
                                                          h->hidx, owned, part);
  else
    k_stats_partial<2><<<nb, kRedThreads, 0, h->stream>>>(h->k, h->v, h->m, h->sid, h->st,
                                                          h->hidx, owned, part);
  k_stats_final<<<1, 32, 0, h->stream>>>(part, nb, out);
  h->launches += 2;
  double res[kRedVals];
  if (cuda_check(h, cudaMemcpyAsync(res, out, sizeof res, cudaMemcpyDeviceToHost, h->stream),
                 "stats copy"))
    return MCFG_ECUDA;
  if (cuda_check(h, cudaStreamSynchronize(h->stream), "stats sync")) return MCFG_ECUDA;
  if (ke) *ke = res[0];
  if (mom)
    for (int a = 0; a < 3; ++a) mom[a] = res[1 + a];
  if (stress) {
    const int d = h->k.d;
    for (int a = 0; a < 9; ++a) stress[a] = (a < d * d && h->k.stress) ? res[4 + a] : 0.0;
  }
  return MCFG_OK;
}

}  // namespace mcfg
