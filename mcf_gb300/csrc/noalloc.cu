// noalloc.cu -- number-density summation that allocates no device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs while a
// caching allocator holds its lock, hosts that hand the library only buffers
// they registered themselves, or a process that has to stay inside a fixed
// device-memory budget decided up front.  mcfg_density_noalloc serves them:
// the caller passes device inputs and a device output, and the cell list the
// sweep needs lives in one file-scope __device__ array of fixed size that
// every GPU loading this library holds until the process exits.
//
// Limits: at most kNoAllocMaxParticles particles and kNoAllocMaxCells real
// cells per call.  Every call uses the same array and it keeps the previous
// call's contents, so the per-cell counters and the status word are cleared
// at the start of each call, and calls whose GPU work overlaps (different
// streams, or different host threads on one device) race on it: serialise
// them.
//
// The sweep is the density of particles_compute_density.F90:369-867 (same
// PPM box index, same FP64 pair separation and cut-off test, same species
// rules: fluid always sums, walls with wall_rho_type 1 and colloid boundary
// particles with a dynamic colloid density) computed with a plain cell-list
// gather.  Each cell's particles are visited in host index order, as in
// PPM's stable cell list, so the sums have a fixed order and repeated calls
// give identical bits; the result agrees with mcfg_compute_density to
// rounding.
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "mcfg_internal.cuh"
#include "sph.cuh"

namespace {

using namespace mcfg;

constexpr int kNoAllocMaxParticles = 1 << 16;  // 65,536
constexpr int kNoAllocMaxCells = 1 << 16;      // 65,536 real cells
// layout in int32 words:
//   key[P] | rank[P] | order[P] | cnt[C+1] | status | start[C+2]
// rank[] is reused for the host-index order of each cell after the scatter;
// status (cleared with the counters) collects kNaZeroDensity
constexpr size_t kScratchWords =
    3 * (size_t)kNoAllocMaxParticles + 2 * (size_t)kNoAllocMaxCells + 4;
constexpr int kNaZeroDensity = 1;  // a density came out <= 0 (or NaN)

static __device__ __align__(256) int g_noalloc_scratch[kScratchWords];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
int* g_scratch_dev[kMaxDevices] = {};  // device address per device ordinal
std::string g_err = "no error";

// A failed CUDA call also leaves the error as the thread's last error; take
// it off so that a later, unrelated launch check does not report it again.
int cuda_fail(const char* what, cudaError_t e) {
  (void)cudaGetLastError();
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return MCFG_ECUDA;
}

// Puts the caller's current device back when the call returns.
struct DeviceRestore {
  int prev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      (void)cudaGetLastError();
      prev = -1;
    }
  }
  ~DeviceRestore() {
    if (prev >= 0 && cudaSetDevice(prev) != cudaSuccess) (void)cudaGetLastError();
  }
};

// The array's name is a host-side stand-in in host code: its device address
// is looked up once per device, with that device current.
int scratch_address(int dev, int** out) {
  if (dev < 0 || dev >= kMaxDevices) {
    g_err = "device ordinal out of range";
    return MCFG_EINVAL;
  }
  if (!g_scratch_dev[dev]) {
    int* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress", e);
    if (ptr == nullptr) {
      g_err = "cudaGetSymbolAddress returned no address";
      return MCFG_ECUDA;
    }
    g_scratch_dev[dev] = ptr;
  }
  *out = g_scratch_dev[dev];
  return MCFG_OK;
}

__device__ __forceinline__ int na_axis_cell(double xa, double xmin, double xmax, double rdx,
                                            int nm) {
  int ia = (int)floor(__dmul_rn(__dsub_rn(xa, xmin), rdx));
  if (xa >= xmax && ia < nm) ia = nm;
  if (xa < xmax && ia >= nm) ia = nm - 1;
  return (ia >= 0 && ia < nm) ? ia : -1;
}

template <int D>
__global__ void k_na_count(Consts k, int n, const double* __restrict__ x, int* __restrict__ key,
                           int* __restrict__ rank, int* __restrict__ cnt) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int cell = 0, stride = 1;
  bool inside = true;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int ia = na_axis_cell(x[(size_t)p * D + a], k.xmin[a], k.xmax[a], k.rdx[a], k.nm[a]);
    if (ia < 0) inside = false;
    cell += ia * stride;
    stride *= k.nm[a];
  }
  if (!inside) cell = k.ncell;
  key[p] = cell;
  rank[p] = atomicAdd(&cnt[cell], 1);
}

// one block: exclusive scan of nb counts into start[0..nb]
__global__ void k_na_scan(const int* __restrict__ cnt, int nb, int* __restrict__ start) {
  __shared__ int warp_tot[32];
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int b0 = threadIdx.x * per;
  int s = 0;
  for (int b = b0; b < b0 + per && b < nb; ++b) s += cnt[b];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    int w = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < nw) warp_tot[lane] = w;
  }
  __syncthreads();
  int run = inc - s + (wid > 0 ? warp_tot[wid - 1] : 0);
  for (int b = b0; b < b0 + per && b < nb; ++b) {
    start[b] = run;
    run += cnt[b];
  }
  if (threadIdx.x == blockDim.x - 1) start[nb] = warp_tot[(blockDim.x >> 5) - 1];
}

__global__ void k_na_scatter(int n, const int* __restrict__ key, const int* __restrict__ rank,
                             const int* __restrict__ start, int* __restrict__ order) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  order[start[key[p]] + rank[p]] = p;
}

// The scatter's slot order inside a cell follows the atomics of k_na_count
// and changes from call to call.  One warp per cell writes the cell's
// particles to sorted[] in host index order (PPM's stable order): an entry's
// place is the number of the cell's entries with a smaller index (indices
// are distinct).
__global__ void k_na_order(int ncell, const int* __restrict__ start,
                           const int* __restrict__ order, int* __restrict__ sorted) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncell) return;
  const int s0 = start[warp], len = start[warp + 1] - s0;
  for (int t = lane; t < len; t += 32) {
    const int me = order[s0 + t];
    int below = 0;
    for (int u = 0; u < len; ++u) below += order[s0 + u] < me;
    sorted[s0 + below] = me;
  }
}

template <int D>
__global__ void k_na_density(Consts k, int n, const double* __restrict__ x,
                             const double* __restrict__ m, const int* __restrict__ id,
                             const int* __restrict__ key, const int* __restrict__ start,
                             const int* __restrict__ order, double* __restrict__ rho,
                             int* __restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int si = id[2 * i + 1];
  const bool acc_i = dyn_rho(k, si);
  const double mi = m[i];
  if (!acc_i) {
    const double r0 = (k.rhs_density_type == 1) ? k.init_density : k.init_density / mi;
    rho[i] = r0;
    if (!(r0 > 0.0)) atomicOr(status, kNaZeroDensity);
    return;
  }
  double xi[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int a = 0; a < D; ++a) xi[a] = x[(size_t)i * D + a];
  double sum = 0.0;
  const int ci = key[i];
  if (ci < k.ncell) {
    int c[3] = {0, 0, 0};
    int rem = ci;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      c[a] = rem % k.nm[a];
      rem /= k.nm[a];
    }
    constexpr int NS = (D == 3) ? 27 : 9;
    for (int sl = 0; sl < NS; ++sl) {
      const int o[3] = {sl % 3 - 1, (sl / 3) % 3 - 1, sl / 9 - 1};
      int nc = 0, stride = 1;
      int sh[3] = {0, 0, 0};
      bool ok = true;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        int t = c[a] + o[a];
        if (t < 0) {
          if (k.periodic[a]) {
            t += k.nm[a];
            sh[a] = 2;
          } else {
            ok = false;
          }
        } else if (t >= k.nm[a]) {
          if (k.periodic[a]) {
            t -= k.nm[a];
            sh[a] = 1;
          } else {
            ok = false;
          }
        }
        nc += t * stride;
        stride *= k.nm[a];
      }
      if (!ok) continue;
      for (int q = start[nc]; q < start[nc + 1]; ++q) {
        const int j = order[q];
        if (j == i) continue;
        // separation rounded like MCF's pair with a ghost image at x + L
        double d2 = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          const double xj = x[(size_t)j * D + a];
          double ra;
          if (sh[a] == 1)
            ra = __dsub_rn(xi[a], __dadd_rn(xj, k.len[a]));
          else if (sh[a] == 2)
            ra = __dsub_rn(__dadd_rn(xi[a], k.len[a]), xj);
          else
            ra = __dsub_rn(xi[a], xj);
          d2 = (a == 0) ? __dmul_rn(ra, ra) : __dadd_rn(d2, __dmul_rn(ra, ra));
        }
        if (d2 >= k.rc2) continue;
        const double w = kernel_w<double>(k, sqrt(d2));
        sum += (k.rhs_density_type == 1) ? w * m[j] : w;
      }
    }
  }
  const double r = ((k.rhs_density_type == 1) ? k.w0 * mi : k.w0) + sum;
  rho[i] = r;
  if (!(r > 0.0)) atomicOr(status, kNaZeroDensity);
}

// the scratch words of one call
struct NaScratch {
  int *key, *rank, *order, *cnt, *status, *start;
};

NaScratch na_layout(int* base) {
  NaScratch t;
  t.key = base;
  t.rank = t.key + kNoAllocMaxParticles;
  t.order = t.rank + kNoAllocMaxParticles;
  t.cnt = t.order + kNoAllocMaxParticles;
  t.status = t.cnt + (kNoAllocMaxCells + 1);
  t.start = t.status + 1;
  return t;
}

}  // namespace

extern "C" {

int mcfg_density_noalloc(const mcfg_params* params, int32_t coll_rho_type, int32_t n,
                         const double* x, const double* m, const int32_t* id, double* rho,
                         void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  const char* msg = validate_params(params);
  if (msg) {
    g_err = msg;
    return MCFG_EINVAL;
  }
  if (n < 0 || n > kNoAllocMaxParticles) {
    char buf[160];
    snprintf(buf, sizeof buf,
             "mcfg_density_noalloc: %d particles, the fixed scratch holds at most %d", n,
             kNoAllocMaxParticles);
    g_err = buf;
    return MCFG_EINVAL;
  }
  if (coll_rho_type != 0 && coll_rho_type != 1) {
    g_err = "mcfg_density_noalloc: coll_rho_type must be 0 (constant) or 1 (dynamic)";
    return MCFG_EINVAL;
  }
  if (n > 0 && (!x || !m || !id || !rho)) {
    g_err = "mcfg_density_noalloc: NULL array";
    return MCFG_EINVAL;
  }
  Consts k;
  make_consts(*params, k);
  k.n = n;
  k.coll_rho_type = coll_rho_type;
  if (k.le) {
    g_err = "mcfg_density_noalloc: Lees-Edwards faces are not supported here";
    return MCFG_ENOTSUP;
  }
  if (k.ncell > kNoAllocMaxCells) {
    char buf[160];
    snprintf(buf, sizeof buf,
             "mcfg_density_noalloc: %d cells, the fixed scratch holds at most %d", k.ncell,
             kNoAllocMaxCells);
    g_err = buf;
    return MCFG_EINVAL;
  }
  for (int a = 0; a < k.d; ++a)
    if (k.periodic[a] && k.nm[a] < 3) {
      g_err = "a periodic axis needs at least 3 cells (box >= 3*1.0001*cut_off)";
      return MCFG_EINVAL;
    }
  DeviceRestore restore;
  cudaError_t e = cudaSetDevice(params->device);
  if (e != cudaSuccess) {
    cuda_fail("cudaSetDevice", e);
    return MCFG_ENODEV;
  }
  int* base = nullptr;
  int rc = scratch_address(params->device, &base);
  if (rc) return rc;
  const NaScratch t = na_layout(base);
  cudaStream_t s = (cudaStream_t)stream;
  const int nbins = k.ncell + 1;
  // the counters and the status word after them keep the previous call's
  // values: clear both
  e = cudaMemsetAsync(t.cnt, 0, sizeof(int) * ((size_t)kNoAllocMaxCells + 2), s);
  if (e != cudaSuccess) return cuda_fail("cudaMemsetAsync", e);
  if (n == 0) return MCFG_OK;
  const int tb = 256, gb = (n + tb - 1) / tb;
  if (k.d == 3)
    k_na_count<3><<<gb, tb, 0, s>>>(k, n, x, t.key, t.rank, t.cnt);
  else
    k_na_count<2><<<gb, tb, 0, s>>>(k, n, x, t.key, t.rank, t.cnt);
  k_na_scan<<<1, 1024, 0, s>>>(t.cnt, nbins, t.start);
  k_na_scatter<<<gb, tb, 0, s>>>(n, t.key, t.rank, t.start, t.order);
  // host-index order inside each real cell, into rank[] (free after the
  // scatter); particles outside the mesh take no part in any sum
  const int gcell = (int)(((int64_t)k.ncell * 32 + tb - 1) / tb);
  k_na_order<<<gcell, tb, 0, s>>>(k.ncell, t.start, t.order, t.rank);
  if (k.d == 3)
    k_na_density<3><<<gb, tb, 0, s>>>(k, n, x, m, id, t.key, t.start, t.rank, rho, t.status);
  else
    k_na_density<2><<<gb, tb, 0, s>>>(k, n, x, m, id, t.key, t.start, t.rank, rho, t.status);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail("mcfg_density_noalloc launch", e);
  return MCFG_OK;
}

int mcfg_noalloc_status(int32_t device, void* stream, int32_t* flags) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!flags) {
    g_err = "mcfg_noalloc_status: NULL flags";
    return MCFG_EINVAL;
  }
  *flags = 0;
  DeviceRestore restore;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    cuda_fail("cudaSetDevice", e);
    return MCFG_ENODEV;
  }
  int* base = nullptr;
  int rc = scratch_address(device, &base);
  if (rc) return rc;
  const NaScratch t = na_layout(base);
  cudaStream_t s = (cudaStream_t)stream;
  int32_t word = 0;
  e = cudaMemcpyAsync(&word, t.status, sizeof word, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync", e);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail("cudaStreamSynchronize", e);
  *flags = word;
  return MCFG_OK;
}

const char* mcfg_noalloc_error(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_err.c_str();
}

}  // extern "C"
