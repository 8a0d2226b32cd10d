// cell_list.cu -- per-step cell list: PPM's box index (bit-exact), a stable
// counting sort by (cell, host index), CSR cell starts and the permutation
// of the particle state into cell order.
//
// Reference: ppm:src/ppm_neighlist_clist.F90:318-438 -> ppm_util_rank3d.F90
// :308-531 (rank2d alike), called each step from technique_build_list
// (mcf/src/technique_build_list.F90:94-109, marching_integrate_VV.F90:968).
#include "mcfg_internal.cuh"

namespace mcfg {

// Real-cell coordinate of position xa along one axis, or -1 if the particle
// has no real cell.  Same operations as ppm_util_rank3d.F90:422-459: the
// subtraction comes before the multiplication, FLOOR, then the two
// corrections at the upper boundary.  No contraction is possible here.
__device__ __forceinline__ int ppm_axis_cell(double xa, double xmin, double xmax,
                                             double rdx, int nm) {
  int ia = (int)floor(__dmul_rn(__dsub_rn(xa, xmin), rdx));
  if (xa >= xmax && ia < nm) ia = nm;       // outside above: ghost layer
  if (xa < xmax && ia >= nm) ia = nm - 1;   // inside: last real cell
  return (ia >= 0 && ia < nm) ? ia : -1;
}

template <int D>
__global__ void k_cell_key(Consts k, const double4_32a* __restrict__ x, int* __restrict__ key,
                           int* __restrict__ rank, int* __restrict__ cnt,
                           const int* __restrict__ gate) {
  if (gate && *gate == 0) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= k.n) return;
  const double4_32a xp = x[p];
  const double xs[3] = {xp.x, xp.y, xp.z};
  int cell = 0, stride = 1;
  bool inside = true;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int ia = ppm_axis_cell(xs[a], k.xmin[a], k.xmax[a], k.rdx[a], k.nm[a]);
    if (ia < 0) inside = false;
    cell += ia * stride;
    stride *= k.nm[a];
  }
  if (!inside) cell = k.ncell;  // extra bin: no box, no interactions
  key[p] = cell;
  rank[p] = atomicAdd(&cnt[cell], 1);
}

// Exclusive scan in three launches over tiles of kScanTile counts.
constexpr int kScanThreads = 512;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanThreads * kScanPer;

__device__ __forceinline__ int block_exclusive_scan(int v, int* smem, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) smem[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    int w = (lane < nw) ? smem[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < nw) smem[lane] = w;
  }
  __syncthreads();
  const int warp_off = (wid > 0) ? smem[wid - 1] : 0;
  total = smem[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + inc - v;
}

__global__ void k_scan_tiles(const int* __restrict__ in, int n, int* __restrict__ part,
                             const int* __restrict__ gate) {
  if (gate && *gate == 0) return;
  __shared__ int smem[32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  int s = 0;
#pragma unroll
  for (int e = 0; e < kScanPer; ++e)
    if (base + e < n) s += in[base + e];
  int total;
  block_exclusive_scan(s, smem, total);
  if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void k_scan_partials(int* part, int nparts, const int* __restrict__ gate) {
  if (gate && *gate == 0) return;
  __shared__ int smem[32];
  int carry = 0;
  for (int b0 = 0; b0 < nparts; b0 += blockDim.x) {
    const int i = b0 + threadIdx.x;
    const int v = (i < nparts) ? part[i] : 0;
    int total;
    const int ex = block_exclusive_scan(v, smem, total);
    if (i < nparts) part[i] = carry + ex;
    carry += total;
  }
}

__global__ void k_scan_final(const int* __restrict__ in, int n, const int* __restrict__ part,
                             int* __restrict__ out, const int* __restrict__ gate) {
  if (gate && *gate == 0) return;
  __shared__ int smem[32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  int vals[kScanPer];
  int s = 0;
#pragma unroll
  for (int e = 0; e < kScanPer; ++e) {
    vals[e] = (base + e < n) ? in[base + e] : 0;
    s += vals[e];
  }
  int total;
  int run = block_exclusive_scan(s, smem, total) + part[blockIdx.x];
#pragma unroll
  for (int e = 0; e < kScanPer; ++e) {
    if (base + e < n) out[base + e] = run;
    run += vals[e];
  }
  // out[n] = grand total
  if (base + kScanPer >= n && base < n) out[n] = run;
}

__global__ void k_scatter(int n, const int* __restrict__ key, const int* __restrict__ rank,
                          const int* __restrict__ start, int* __restrict__ order,
                          const int* __restrict__ gate) {
  if (gate && *gate == 0) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  order[start[key[p]] + rank[p]] = p;
}

// One warp per bin: rank the bin's particles by host index (the stable order
// of PPM's counting sort, rank3d.F90:504-531, whose input order is MCF's
// array order), gather the state into the new slots and write the FP32
// offsets to the cell origin (w = species id).
template <int D>
__global__ void k_cell_finalize(Consts k, const int* __restrict__ start,
                                const int* __restrict__ order, const int* __restrict__ hidx_in,
                                const double4_32a* __restrict__ x_in, const double4_32a* __restrict__ v_in,
                                const double4_32a* __restrict__ f_in, const double* __restrict__ m_in,
                                const int* __restrict__ pid_in, const int* __restrict__ sid_in,
                                double4_32a* __restrict__ x_out, double4_32a* __restrict__ v_out,
                                double4_32a* __restrict__ f_out, double* __restrict__ m_out,
                                int* __restrict__ pid_out, int* __restrict__ sid_out,
                                int* __restrict__ hidx_out, float4* __restrict__ off,
                                int* __restrict__ cell_of, float2* __restrict__ wd,
                                const double* __restrict__ ct_in, const double* __restrict__ act_in,
                                double* __restrict__ ct_out, double* __restrict__ act_out,
                                int* __restrict__ slot_of, unsigned* __restrict__ err,
                                const int* __restrict__ gate) {
  if (gate && *gate == 0) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp > k.ncell) return;
  const int s0 = start[warp], s1 = start[warp + 1];
  const int cnt = s1 - s0;
  if (cnt == 0) return;
  if (warp < k.ncell && cnt > kMaxCellCount && lane == 0) atomicOr(err, kErrCellOverflow);
  double org[3] = {0.0, 0.0, 0.0};
  if (warp < k.ncell) {
    int c = warp;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const int ca = c % k.nm[a];
      c /= k.nm[a];
      org[a] = k.xmin[a] + (double)ca * k.cs[a];
    }
  }
  for (int e = lane; e < cnt; e += 32) {
    const int o = order[s0 + e];
    const int hm = hidx_in[o];
    int r = 0;
    for (int q = 0; q < cnt; ++q) r += (hidx_in[order[s0 + q]] < hm) ? 1 : 0;
    const int dst = s0 + r;
    const double4_32a xp = x_in[o];
    x_out[dst] = xp;
    v_out[dst] = v_in[o];
    f_out[dst] = f_in[o];
    m_out[dst] = m_in[o];
    pid_out[dst] = pid_in[o];
    sid_out[dst] = sid_in[o];
    hidx_out[dst] = hm;
    slot_of[hm] = dst;
    cell_of[dst] = warp;
    float4 of;
    of.x = (float)(xp.x - org[0]);
    of.y = (float)(xp.y - org[1]);
    of.z = (D == 3) ? (float)(xp.z - org[2]) : 0.0f;
    of.w = __int_as_float(sid_in[o]);  // species id rides in the w lane
    off[dst] = of;
    if (ct_in != nullptr) {
      const int n = k.n;
      for (int cc = 0; cc < D * D; ++cc) {
        ct_out[(size_t)cc * n + dst] = ct_in[(size_t)cc * n + o];
        act_out[(size_t)cc * n + dst] = act_in[(size_t)cc * n + o];
      }
    }
    if (wd != nullptr && k.wall_axis >= 0) {
      // distances to the two faces of the wall axis, formed in FP64 and
      // rounded once (boundary_noslip_solid.F90:200-206 uses x - x_sur)
      const double xa = k.wall_axis == 0 ? xp.x : (k.wall_axis == 1 ? xp.y : xp.z);
      wd[dst] = make_float2((float)(xa - k.min_phys[k.wall_axis]),
                            (float)(xa - k.max_phys[k.wall_axis]));
    }
  }
}

// zero the per-bin counts (a kernel, so that it can be gated)
__global__ void k_zero_counts(int* __restrict__ cnt, int nbins, const int* __restrict__ gate) {
  if (gate && *gate == 0) return;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nbins) cnt[b] = 0;
}

// after a gated rebuild: the permuted state back into the primary buffers
// (a host-side pointer swap cannot depend on the device flag) and the
// reference positions of the new candidate list
template <int D>
__global__ void k_copy_back(int n, const int* __restrict__ gate, const double4_32a* __restrict__ x2,
                            const double4_32a* __restrict__ v2, const double4_32a* __restrict__ f2,
                            const double* __restrict__ m2, const int* __restrict__ pid2,
                            const int* __restrict__ sid2, const int* __restrict__ hidx2,
                            const double* __restrict__ ct2, const double* __restrict__ act2,
                            double4_32a* __restrict__ x, double4_32a* __restrict__ v,
                            double4_32a* __restrict__ f, double* __restrict__ m,
                            int* __restrict__ pid, int* __restrict__ sid, int* __restrict__ hidx,
                            double* __restrict__ ct, double* __restrict__ act,
                            double4_32a* __restrict__ x_ref) {
  if (*gate == 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a xp = x2[i];
  x[i] = xp;
  x_ref[i] = xp;
  v[i] = v2[i];
  f[i] = f2[i];
  m[i] = m2[i];
  pid[i] = pid2[i];
  sid[i] = sid2[i];
  hidx[i] = hidx2[i];
  if (ct != nullptr)
    for (int cc = 0; cc < D * D; ++cc) {
      ct[(size_t)cc * n + i] = ct2[(size_t)cc * n + i];
      act[(size_t)cc * n + i] = act2[(size_t)cc * n + i];
    }
}

// the cell list proper; with a gate every kernel returns at once when the
// device flag is zero, and the permuted state is copied back instead of
// swapping the buffers
static int cell_list_launches(Handle* h, const int* gate) {
  Consts& k = h->k;
  const int n = (int)h->n;
  cudaStream_t s = h->stream;
  const int nbins = k.ncell + 1;
  if (gate == nullptr) {
    if (cuda_check(h, cudaMemsetAsync(h->cnt, 0, sizeof(int) * (size_t)nbins, s), "memset cnt"))
      return MCFG_ECUDA;
  } else {
    k_zero_counts<<<(nbins + 255) / 256, 256, 0, s>>>(h->cnt, nbins, gate);
    h->launches++;
  }
  const int tb = 256;
  const int gb = (n + tb - 1) / tb;
  if (n > 0) {
    if (k.d == 3)
      k_cell_key<3><<<gb, tb, 0, s>>>(k, h->x, h->key, h->rank, h->cnt, gate);
    else
      k_cell_key<2><<<gb, tb, 0, s>>>(k, h->x, h->key, h->rank, h->cnt, gate);
    h->launches++;
  }
  const int ntiles = (nbins + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<ntiles, kScanThreads, 0, s>>>(h->cnt, nbins, h->scan_part, gate);
  k_scan_partials<<<1, 1024, 0, s>>>(h->scan_part, ntiles, gate);
  k_scan_final<<<ntiles, kScanThreads, 0, s>>>(h->cnt, nbins, h->scan_part, h->cell_start, gate);
  h->launches += 3;
  if (n > 0) {
    k_scatter<<<gb, tb, 0, s>>>(n, h->key, h->rank, h->cell_start, h->order, gate);
    const int warps_per_block = 8;
    const int gw = (nbins + warps_per_block - 1) / warps_per_block;
    if (k.d == 3)
      k_cell_finalize<3><<<gw, warps_per_block * 32, 0, s>>>(
          k, h->cell_start, h->order, h->hidx, h->x, h->v, h->f, h->m, h->pid, h->sid, h->x2,
          h->v2, h->f2, h->m2, h->pid2, h->sid2, h->hidx2, h->off, h->cell_of, h->wd, h->ct, h->act,
          h->ct2, h->act2, h->slot_of, h->d_err, gate);
    else
      k_cell_finalize<2><<<gw, warps_per_block * 32, 0, s>>>(
          k, h->cell_start, h->order, h->hidx, h->x, h->v, h->f, h->m, h->pid, h->sid, h->x2,
          h->v2, h->f2, h->m2, h->pid2, h->sid2, h->hidx2, h->off, h->cell_of, h->wd, h->ct, h->act,
          h->ct2, h->act2, h->slot_of, h->d_err, gate);
    h->launches += 2;
    if (gate == nullptr) {
      std::swap(h->x, h->x2);
      std::swap(h->v, h->v2);
      std::swap(h->f, h->f2);
      std::swap(h->m, h->m2);
      std::swap(h->pid, h->pid2);
      std::swap(h->sid, h->sid2);
      std::swap(h->hidx, h->hidx2);
      if (h->ct) {
        std::swap(h->ct, h->ct2);
        std::swap(h->act, h->act2);
      }
    } else {
#define COPY_BACK(DD)                                                                            \
  k_copy_back<DD><<<gb, tb, 0, s>>>(n, gate, h->x2, h->v2, h->f2, h->m2, h->pid2, h->sid2,       \
                                    h->hidx2, h->ct2, h->act2, h->x, h->v, h->f, h->m, h->pid,   \
                                    h->sid, h->hidx, h->ct, h->act, h->x_ref)
      if (k.d == 3) COPY_BACK(3); else COPY_BACK(2);
#undef COPY_BACK
      h->launches++;
    }
  }
  if (cuda_check(h, cudaGetLastError(), "cell list launch")) return MCFG_ECUDA;
  return MCFG_OK;
}

int build_cell_list(Handle* h) {
  h->reuse_valid = false;  // the particle order changes under any candidate list
  if (h->k.le) le_map(h);  // the crossing rows' cells of the current shift
  if (h->unwrapped) {      // after list-reuse steps: MCF's wrap first
    const int rc = adjust_particles(h);
    if (rc) return rc;
    h->unwrapped = false;
  }
  return cell_list_launches(h, nullptr);
}

int gated_cell_list(Handle* h) { return cell_list_launches(h, h->d_rebuild); }

}  // namespace mcfg
