// adjoint.cu -- reverse-mode derivative of the time-averaged stress of a VV
// trajectory (differentiation form of the SDPD step).
//
// Forward map of one step t (marching_integrate_VV.F90:303-1620 as this
// library computes it; all particles fluid):
//   v' = v + dt/2 a,  x' = wrap(x + dt v'),  c' = ct + dt/2 act,
//   (n, p, a_new, L, S_t) = RHS(x', v', c'),  act_new = c' L^T + L c' - (c' - I)/tau,
//   ct_new = c' + dt/2 act_new,  v_new = v' + dt/2 a_new,
// and J = (1/T) sum_t w : S_t.  The reverse sweep carries the adjoints of
// (x, v, ct) in host particle order; the adjoints of the carried a and act
// are dt/2 times those of v and ct, so one step backwards is
//   lam = phi vbar, Abar = phi cbar  (phi = dt, or dt/2 at the last step and
//                                     for the initial right-hand side),
//   act VJP:  cbar += Abar L + L^T Abar - Abar/tau,  Lbar = Abar^T c + Abar c^T,
//   pair VJP (k_adj_force), density VJP (k_adj_density),
//   xbar(prev) = xbar', vbar(prev) = vbar' + dt xbar', cbar(prev) = cbar'.
// Each step's right-hand-side inputs (cell order, neighbour list included)
// come from a tape filled while the segment since the last checkpoint is
// recomputed (the last segment is taped during the first pass, which also
// takes the checkpoints, every K steps).  The
// random term is replayed from the same Philox keys (seed, step, pid pair).
//
// Pair VJP of the Hu-Adams force (rhs_force_ff_Newtonian_HuAdams.F90:124-237,
// non-Newtonian form rhs_force_ff_non_Newtonian_HuAdams.F90:95-201) with
// g = f_d v_ij - f_c e + W' u P^T r + f_r We, f_c = (A_i + A_j) W',
// f_d = eta (B_i + B_j) W' u, f_r = sqrt(-4 kT f_d)/sqrt(dt),
// A = (p + G)/n^2, B = 1/n^2, P = G (c_i B_i + c_j B_j), u = 1/|r|, and the
// velocity gradient L_i += (v_j - v_i) (x) r W' u / n_i (pp_vgt_ip.inc).
// Every pair is differentiated from both sides (gather, no atomics), as
// the forward sweep evaluates it.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mcfg_internal.cuh"
#include "pair_common.cuh"
#include "sph.cuh"

namespace mcfg {

// One step's right-hand-side inputs, in that step's cell order.
struct Tape {
  double4_32a* x;    // positions x'
  double4_32a* v;    // half-step velocities v'
  double4_32a* pc;   // (A, B, 1/m, p)
  double* rho;       // number density
  int* pid;
  int* hidx;
  int* ncount;
  int* cell_of;      // cell of each particle (ncell: outside the mesh)
  int* cell_start;
  uint16_t* nl;      // [neigh][n]
  double* ct;        // [d*d][n] conformation tensor c' (Oldroyd-B)
  double* vgt;       // [d*d][n] velocity gradient L (Oldroyd-B)
};

// Carried VV state in host particle order.
struct Ckpt {
  double4_32a *x, *v, *f;
  double *ct, *act, *rho, *pr, *st;
};

struct AdjBuffers {
  int n = 0, d = 0, nnw = 0, K = 0, T = 0, ncell = 0, neigh = 0, nb = 0;
  std::vector<Tape> tape;  // K slots + 1 for the initial right-hand side
  // a second set of tapes when memory allows: segment s - 1 is recomputed
  // into one set while the reverse sweep of segment s reads the other, on
  // its own stream (rs); ev_fill / ev_read order the two sets' reuse
  std::vector<Tape> tape2;
  cudaStream_t rs = nullptr;
  cudaEvent_t ev_fill[2] = {nullptr, nullptr}, ev_read[2] = {nullptr, nullptr};
  std::vector<Ckpt> ck;    // segment starts 0, K, 2K, ...
  Ckpt last{};             // state after the last step
  double* m_h = nullptr;
  int *pid_h = nullptr, *sid_h = nullptr;
  double4_32a *xb_h = nullptr, *vb_h = nullptr;  // carried adjoints (host order)
  double* cb_h = nullptr;
  double4_32a *lam = nullptr, *xbs = nullptr, *vbs = nullptr;  // per step, cell order
  double *Lb = nullptr, *qb = nullptr, *cbs = nullptr, *nbar = nullptr;
  double* gp = nullptr;     // [3][n] parameter partials (host order)
  double* jpart = nullptr;  // [T][nb] block partials of w : S_t
  double* red = nullptr;    // [3][nb]
  double* w = nullptr;      // [9]
  std::vector<void*> allocs;
};

void free_adjoint(Handle* h) {
  if (!h->adj) return;
  AdjBuffers* b = h->adj;
  if (b->rs) cudaStreamSynchronize(b->rs);
  for (int q = 0; q < 2; ++q) {
    if (b->ev_fill[q]) cudaEventDestroy(b->ev_fill[q]);
    if (b->ev_read[q]) cudaEventDestroy(b->ev_read[q]);
  }
  if (b->rs) cudaStreamDestroy(b->rs);
  for (void* p : h->adj->allocs) cudaFree(p);
  delete h->adj;
  h->adj = nullptr;
}

namespace {

constexpr int kAdjRedThreads = 256;
constexpr int kAdjTPB = 128;  // threads per block of the thread-per-particle sweeps

template <typename T>
int aalloc(Handle* h, AdjBuffers* b, T** p, size_t count) {
  if (count == 0) count = 1;
  const size_t bytes = sizeof(T) * count;
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    char buf[160];
    snprintf(buf, sizeof buf, "adjoint cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    return set_error(h, MCFG_ENOMEM, buf);
  }
  b->allocs.push_back(*p);
  h->device_bytes += (int64_t)bytes;
  return MCFG_OK;
}

#define ATRY(expr)         \
  do {                     \
    int _rc = (expr);      \
    if (_rc) return _rc;   \
  } while (0)

int alloc_ckpt(Handle* h, AdjBuffers* b, Ckpt& c, bool full) {
  const size_t n = (size_t)b->n, d2 = (size_t)b->d * b->d;
  c = Ckpt{};
  ATRY(aalloc(h, b, &c.x, n));
  ATRY(aalloc(h, b, &c.v, n));
  if (b->nnw) ATRY(aalloc(h, b, &c.ct, n * d2));
  if (!full) return MCFG_OK;
  ATRY(aalloc(h, b, &c.f, n));
  if (b->nnw) ATRY(aalloc(h, b, &c.act, n * d2));
  return MCFG_OK;
}

int ensure_buffers(Handle* h, int K, int T) {
  const int n = (int)h->n, d = h->k.d, nnw = h->k.newtonian ? 0 : 1;
  const int ncell = h->k.ncell, neigh = h->neigh_cap;
  AdjBuffers* b = h->adj;
  if (b && b->n == n && b->d == d && b->nnw == nnw && b->K == K && b->T == T &&
      b->ncell == ncell && b->neigh == neigh)
    return MCFG_OK;
  free_adjoint(h);
  b = h->adj = new AdjBuffers();
  b->n = n;
  b->d = d;
  b->nnw = nnw;
  b->K = K;
  b->T = T;
  b->ncell = ncell;
  b->neigh = neigh;
  int nb = (n + kAdjRedThreads - 1) / kAdjRedThreads;
  b->nb = std::max(1, std::min(nb, 1024));
  const size_t N = (size_t)n, d2 = (size_t)d * d;
  auto alloc_tapes = [&](std::vector<Tape>& set) -> int {
    set.resize((size_t)K + 1);
    for (Tape& t : set) {
      t = Tape{};
      ATRY(aalloc(h, b, &t.x, N));
      ATRY(aalloc(h, b, &t.v, N));
      ATRY(aalloc(h, b, &t.pc, N));
      ATRY(aalloc(h, b, &t.rho, N));
      ATRY(aalloc(h, b, &t.pid, N));
      ATRY(aalloc(h, b, &t.hidx, N));
      ATRY(aalloc(h, b, &t.ncount, N));
      ATRY(aalloc(h, b, &t.cell_of, N));
      ATRY(aalloc(h, b, &t.cell_start, (size_t)ncell + 2));
      ATRY(aalloc(h, b, &t.nl, (size_t)neigh * N));
      if (nnw) {
        ATRY(aalloc(h, b, &t.ct, d2 * N));
        ATRY(aalloc(h, b, &t.vgt, d2 * N));
      }
    }
    return MCFG_OK;
  };
  ATRY(alloc_tapes(b->tape));
  const int nseg = (T + K - 1) / K;
  if (nseg > 1) {
    // the second tape set, if it leaves a quarter of the device free
    const size_t set_bytes =
        (size_t)(K + 1) * (N * (3 * sizeof(double4_32a) + sizeof(double) + 4 * sizeof(int) +
                                neigh * sizeof(uint16_t) + (nnw ? 2 * d2 * sizeof(double) : 0)) +
                           sizeof(int) * ((size_t)ncell + 2));
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && free_b > set_bytes + total_b / 4 &&
        cudaStreamCreateWithFlags(&b->rs, cudaStreamNonBlocking) == cudaSuccess) {
      bool ok = true;
      for (int q = 0; q < 2 && ok; ++q)
        ok = cudaEventCreateWithFlags(&b->ev_fill[q], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->ev_read[q], cudaEventDisableTiming) == cudaSuccess;
      if (!ok) return set_error(h, MCFG_ECUDA, "adjoint stream events");
      ATRY(alloc_tapes(b->tape2));
    }
    cudaGetLastError();
  }
  b->ck.resize((size_t)nseg);
  for (int s = 0; s < nseg; ++s) ATRY(alloc_ckpt(h, b, b->ck[(size_t)s], s > 0));
  ATRY(alloc_ckpt(h, b, b->last, true));
  ATRY(aalloc(h, b, &b->last.rho, N));
  ATRY(aalloc(h, b, &b->last.pr, N));
  ATRY(aalloc(h, b, &b->last.st, d2 * N));
  ATRY(aalloc(h, b, &b->m_h, N));
  ATRY(aalloc(h, b, &b->pid_h, N));
  ATRY(aalloc(h, b, &b->sid_h, N));
  ATRY(aalloc(h, b, &b->xb_h, N));
  ATRY(aalloc(h, b, &b->vb_h, N));
  ATRY(aalloc(h, b, &b->lam, N));
  ATRY(aalloc(h, b, &b->xbs, N));
  ATRY(aalloc(h, b, &b->vbs, N));
  ATRY(aalloc(h, b, &b->nbar, N));
  if (nnw) {
    ATRY(aalloc(h, b, &b->cb_h, d2 * N));
    ATRY(aalloc(h, b, &b->Lb, d2 * N));
    ATRY(aalloc(h, b, &b->qb, d2 * N));
    ATRY(aalloc(h, b, &b->cbs, d2 * N));
  }
  ATRY(aalloc(h, b, &b->gp, 3 * N));
  ATRY(aalloc(h, b, &b->jpart, (size_t)T * b->nb));
  ATRY(aalloc(h, b, &b->red, (size_t)3 * b->nb));
  ATRY(aalloc(h, b, &b->w, 9));
  return MCFG_OK;
}

// ---------------------------------------------------------------------------
// checkpoints, tape, reductions
// ---------------------------------------------------------------------------

// cell order -> host order; null destinations are skipped
__global__ void k_ck_save(int n, int d2, const int* __restrict__ hidx, const double4_32a* x,
                          const double4_32a* v, const double4_32a* f, const double* ct,
                          const double* act, const double* rho, const double* pr,
                          const double* st, Ckpt out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int hi = hidx[i];
  out.x[hi] = x[i];
  out.v[hi] = v[i];
  if (out.f) out.f[hi] = f[i];
  if (out.rho) out.rho[hi] = rho[i];
  if (out.pr) out.pr[hi] = pr[i];
  for (int c = 0; c < d2; ++c) {
    if (out.ct) out.ct[(size_t)c * n + hi] = ct[(size_t)c * n + i];
    if (out.act) out.act[(size_t)c * n + hi] = act[(size_t)c * n + i];
    if (out.st) out.st[(size_t)c * n + hi] = st[(size_t)c * n + i];
  }
}

__global__ void k_consts_save(int n, const int* __restrict__ hidx, const double* m,
                              const int* pid, const int* sid, double* m_h, int* pid_h,
                              int* sid_h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int hi = hidx[i];
  m_h[hi] = m[i];
  pid_h[hi] = pid[i];
  sid_h[hi] = sid[i];
}

// host order -> handle arrays in host order (the next cell-list build sorts
// them; its in-cell rank is by host index, so the result does not depend on
// the order the state arrives in)
__global__ void k_ck_restore(int n, int d2, Ckpt in, const double* __restrict__ m_h,
                             const int* __restrict__ pid_h, const int* __restrict__ sid_h,
                             double4_32a* x, double4_32a* v, double4_32a* f, double* ct,
                             double* act, double* rho, double* pr, double* st, double* m,
                             int* pid, int* sid, int* hidx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = in.x[i];
  v[i] = in.v[i];
  if (in.f) f[i] = in.f[i];
  if (in.rho) rho[i] = in.rho[i];
  if (in.pr) pr[i] = in.pr[i];
  for (int c = 0; c < d2; ++c) {
    if (in.ct) ct[(size_t)c * n + i] = in.ct[(size_t)c * n + i];
    if (in.act) act[(size_t)c * n + i] = in.act[(size_t)c * n + i];
    if (in.st) st[(size_t)c * n + i] = in.st[(size_t)c * n + i];
  }
  m[i] = m_h[i];
  pid[i] = pid_h[i];
  sid[i] = sid_h[i];
  hidx[i] = i;
}

__global__ void k_tape_record(int n, int ncell2, int d2, Tape out, const double4_32a* x,
                              const double4_32a* v, const double4_32a* pc, const double* rho,
                              const int* pid, const int* hidx, const int* ncount,
                              const int* cell_of, const int* cell_start, const uint16_t* nl,
                              const double* ct, const double* vgt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ncell2) out.cell_start[i] = cell_start[i];
  if (i >= n) return;
  out.x[i] = x[i];
  out.v[i] = v[i];
  out.pc[i] = pc[i];
  out.rho[i] = rho[i];
  out.pid[i] = pid[i];
  out.hidx[i] = hidx[i];
  out.cell_of[i] = cell_of[i];
  const int c = ncount[i];
  out.ncount[i] = c;
  for (int e = 0; e < c; ++e) out.nl[(size_t)e * n + i] = nl[(size_t)e * n + i];
  if (out.ct)
    for (int q = 0; q < d2; ++q) {
      out.ct[(size_t)q * n + i] = ct[(size_t)q * n + i];
      out.vgt[(size_t)q * n + i] = vgt[(size_t)q * n + i];
    }
}

// block partial sums of w : s_i over fluid and colloid particles (the stress
// statistic_compute_statistic.F90:230-303 sums), fixed order
__global__ void k_stress_dot(int n, int d2, const double* __restrict__ w,
                             const double* __restrict__ st, const int* __restrict__ sid,
                             double* __restrict__ out) {
  __shared__ double sm[kAdjRedThreads];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (sid[i] < 0) continue;
    for (int q = 0; q < d2; ++q) acc += w[q] * st[(size_t)q * n + i];
  }
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kAdjRedThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sm[0];
}

// block partial sums of the rows of a [rows][n] array, fixed order
__global__ void k_row_sums(int n, int rows, const double* __restrict__ a,
                           double* __restrict__ out) {
  __shared__ double sm[kAdjRedThreads];
  for (int r = 0; r < rows; ++r) {
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
      acc += a[(size_t)r * n + i];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kAdjRedThreads / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)r * gridDim.x + blockIdx.x] = sm[0];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// adjoint kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ double d4(const double4_32a& a, int c) {
  return c == 0 ? a.x : (c == 1 ? a.y : a.z);
}

// per particle, before the pair sweeps: seeds of a and act, the act VJP,
// the body-force VJP (type 3, particles_apply_body_force.F90:276-353)
template <int D, bool NNW>
__global__ void k_adj_pre(Consts k, Tape tp, double phi, const double4_32a* __restrict__ xb_h,
                          const double4_32a* __restrict__ vb_h, const double* __restrict__ cb_h,
                          double4_32a* __restrict__ lam, double4_32a* __restrict__ xbs,
                          double4_32a* __restrict__ vbs, double* __restrict__ cbs,
                          double* __restrict__ Lb, double* __restrict__ qb,
                          double* __restrict__ gp) {
  constexpr int D2 = D * D;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = k.n;
  if (i >= n) return;
  const int hi = tp.hidx[i];
  const double4_32a vb = vb_h[hi];
  double4_32a xb = xb_h[hi];
  const double4_32a l = make_double4_32a(phi * vb.x, phi * vb.y, phi * vb.z, 0.0);
  lam[i] = l;
  if (k.body_force_type == 3 && fabs(k.body_force[0]) > k.machine_zero) {
    const double kw = 2.0 * kPi / (k.max_phys[1] - k.min_phys[1]);
    xb.y += l.x * k.body_force[0] * kw * cos(kw * tp.x[i].y);
  }
  xbs[i] = xb;
  vbs[i] = vb;
  if (NNW) {
    const double qn = 1.0 / tp.rho[i], Bn = tp.pc[i].y;
    double cb[D2], A[D2], c[D2], L[D2];
#pragma unroll
    for (int q = 0; q < D2; ++q) {
      cb[q] = cb_h[(size_t)q * n + hi];
      A[q] = phi * cb[q];
      c[q] = tp.ct[(size_t)q * n + i];
      L[q] = tp.vgt[(size_t)q * n + i];
    }
    double taub = 0.0;
#pragma unroll
    for (int b = 0; b < D; ++b)
#pragma unroll
      for (int a = 0; a < D; ++a) {
        double s1 = 0.0, s2 = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) {
          // (A L)(a,b) + (L^T A)(a,b)
          s1 += A[a + D * j] * L[j + D * b] + L[j + D * a] * A[j + D * b];
          // (A^T c)(a,b) + (A c^T)(a,b)
          s2 += A[j + D * a] * c[j + D * b] + A[a + D * j] * c[b + D * j];
        }
        cbs[(size_t)(a + D * b) * n + i] = cb[a + D * b] + s1 - A[a + D * b] * k.inv_tau;
        // for the pair sweep: Lbar / n and Q = G c B, so that a pair needs
        // only sums of its two particles' values
        Lb[(size_t)(a + D * b) * n + i] = s2 * qn;
        qb[(size_t)(a + D * b) * n + i] = k.G * c[a + D * b] * Bn;
        taub += A[a + D * b] * (c[a + D * b] - (a == b ? 1.0 : 0.0));
      }
    gp[(size_t)n + hi] += taub * k.inv_tau * k.inv_tau;
  }
}

// pair VJP of the force, the velocity gradient and the stress functional;
// writes nbar (adjoint of the number density) for the density VJP
template <int D, bool NNW>
__global__ void __launch_bounds__(kAdjTPB)
    k_adj_force(Consts k, Tape tp, const double4_32a* __restrict__ lam,
                const double* __restrict__ Lb, const double* __restrict__ qb,
                const double* __restrict__ w, double wscale,
                uint32_t step, double inv_sqdt, double4_32a* __restrict__ xbs,
                double4_32a* __restrict__ vbs, double* __restrict__ cbs,
                double* __restrict__ nbar, double* __restrict__ gp, int split) {
  constexpr int D2 = D * D;
  __shared__ int s_start[kMaxStencil * kAdjTPB];
  __shared__ int s_shift[kMaxStencil * kAdjTPB];
  const int n = k.n;
  const bool noise = k.noise != 0;
  const double eta = k.eta, kt = k.kt;
  const double G = NNW ? k.G : 0.0;
  double wt[D2];
#pragma unroll
  for (int q = 0; q < D2; ++q) wt[q] = w[q] * wscale;
  const int tid = threadIdx.x;
  // `split` adjacent lanes share one particle and take every split-th
  // neighbour entry (small systems: more threads in flight); their partial
  // sums are combined by a fixed butterfly, so the result is deterministic
  const int g_ = blockIdx.x * kAdjTPB + tid;
  const int i = g_ / split, part = g_ - i * split;
  const bool live = i < n;
  const int il = live ? i : n - 1;
  build_lane_table<D, kAdjTPB>(k, tp.cell_of[il], tp.cell_start, s_start, s_shift);
  const double4_32a xi4 = tp.x[il];
  const double xi[3] = {xi4.x, xi4.y, xi4.z};
  const double4_32a vi4 = tp.v[il];
  const double4_32a pci = tp.pc[il];
  const double ni = tp.rho[il];
  const double4_32a li4 = lam[il];
  const int pidi = tp.pid[il];
  double ci[D2], Lbi[D2], Qi[D2];
  if (NNW) {
#pragma unroll
    for (int q = 0; q < D2; ++q) {
      ci[q] = tp.ct[(size_t)q * n + il];
      Lbi[q] = Lb[(size_t)q * n + il];  // Lbar_i / n_i
      Qi[q] = qb[(size_t)q * n + il];   // G c_i / n_i^2
    }
  }
  const double qi = 1.0 / ni;
  double xb[3] = {0, 0, 0}, vb[3] = {0, 0, 0}, Pbar[D2];
#pragma unroll
  for (int q = 0; q < D2; ++q) Pbar[q] = 0.0;
  double Bbar = 0.0, Abar = 0.0, nbL = 0.0, etab = 0.0;
  const int cnt = live ? tp.ncount[il] : 0;
  for (int e = part; e < cnt; e += split) {
    const int ent = tp.nl[(size_t)e * n + il];
    const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
    const int j = s_start[sl * kAdjTPB + tid] + q;
    const double4_32a xj4 = tp.x[j];
    const double xj[3] = {xj4.x, xj4.y, xj4.z};
    double r[3];
    const double dd2 = exact_sep<D>(k, xi, xj, s_shift[sl * kAdjTPB + tid], r);
    const double u = rsqrt(dd2);
    const double dist = dd2 * u;
    double ev[3];
#pragma unroll
    for (int a = 0; a < D; ++a) ev[a] = r[a] * u;
    double gw, g2;
    kernel_gradw2<double>(k, dist, gw, g2);
    const double4_32a vj4 = tp.v[j];
    const double4_32a pcj = tp.pc[j];
    const double4_32a lj4 = lam[j];
    double vij[3], gb[3], g[3];
#pragma unroll
    for (int a = 0; a < D; ++a) vij[a] = d4(vi4, a) - d4(vj4, a);
    const double SB = pci.y + pcj.y, SA = pci.x + pcj.x;
    const double f_c = SA * gw;
    const double f_d = eta * SB * gw * u;
    // random term We = s (ca (e.g) e + cb (g - (e.g) e)), replayed from
    // the pair's keys exactly as pair_force draws it
    // f_r = sqrt(-4 kT f_d)/sqrt(dt) and df_r/df_d = f_r/(2 f_d) =
    // -2 kT/sqrt(dt) / sqrt(-4 kT f_d), from one reciprocal square root
    double gz[3] = {0, 0, 0}, sg = 0.0, f_r = 0.0, dfr = 0.0;
    if (noise && f_d < 0.0) {
      float z[6];
      pair_draw<D>(3, k.rk, step, pidi, tp.pid[j], z);
#pragma unroll
      for (int a = 0; a < D; ++a) gz[a] = (double)z[a];
      sg = (double)z[5];
      const double arg = -4.0 * kt * f_d;
      const double rs = rsqrt(arg);
      f_r = arg * rs * inv_sqdt;
      dfr = -2.0 * kt * rs * inv_sqdt;
    }
    const double cbn = 0.70710678118654752440;
    const double cdn = ((D == 3) ? 0.81649658092772603273 : cbn) - cbn;  // ca - cb
    double eg = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) eg += ev[a] * gz[a];
    double P[D2], Phi[D2];
    if (NNW) {
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        P[c] = Qi[c] + qb[(size_t)c * n + j];
        Phi[c] = Lbi[c] + Lb[(size_t)c * n + j];
      }
    }
    const double hm = 0.5 * (pci.z + pcj.z);
    // forward pair value and its seed gbar = lam_i/m_i - lam_j/m_j + h w~ r
    double We[3], Pr[3];
#pragma unroll
    for (int b = 0; b < D; ++b) {
      We[b] = sg * (cdn * eg * ev[b] + cbn * gz[b]);
      Pr[b] = 0.0;
      if (NNW) {
#pragma unroll
        for (int a = 0; a < D; ++a) Pr[b] += P[a + D * b] * r[a];
      }
      g[b] = f_d * vij[b] - f_c * ev[b] + gw * u * Pr[b] + f_r * We[b];
      double sw = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) sw += wt[b * D + a] * r[a];
      gb[b] = d4(li4, b) * pci.z - d4(lj4, b) * pcj.z + hm * sw;
    }
    double gbv = 0.0, gbe = 0.0, gbWe = 0.0, gbPr = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      gbv += gb[a] * vij[a];
      gbe += gb[a] * ev[a];
      gbWe += gb[a] * We[a];
      gbPr += gb[a] * Pr[a];
    }
    const double fdb = gbv + gbWe * dfr;
    const double fcb = -gbe;
    double Wb = fdb * eta * SB * u + fcb * SA + u * gbPr;
    double ub = fdb * eta * SB * gw + gw * gbPr;
    double rb[3], eb[3];
    const double fre = f_r * sg * cdn;  // d(We)/de = s (ca - cb) ((e.g) I + e g^T)
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double s1 = 0.0, s3 = 0.0;
#pragma unroll
      for (int b = 0; b < D; ++b) {
        s1 += wt[b * D + a] * g[b];
        if (NNW) s3 += P[a + D * b] * gb[b];
      }
      rb[a] = hm * s1 + gw * u * s3;
      eb[a] = -f_c * gb[a] + fre * (gz[a] * gbe + gb[a] * eg);
    }
    if (NNW) {
      // L term: W' u sum_ab Phi_ab (v_j - v_i)_a r_b
      double phv = 0.0, phi_i = 0.0;
#pragma unroll
      for (int b = 0; b < D; ++b)
#pragma unroll
        for (int a = 0; a < D; ++a) {
          phv += Phi[a + D * b] * (-vij[a]) * r[b];
          phi_i += Lbi[a + D * b] * (-vij[a]) * r[b];
        }
      Wb += u * phv;
      ub += gw * phv;
#pragma unroll
      for (int b = 0; b < D; ++b) {
        double s = 0.0, sv = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          s += Phi[a + D * b] * (-vij[a]);
          sv += Phi[b + D * a] * r[a];
        }
        rb[b] += gw * u * s;
        vb[b] -= gw * u * sv;  // d/dv_i of (v_j - v_i)
      }
      nbL -= gw * u * phi_i * qi;  // Lbi holds Lbar_i / n_i already
#pragma unroll
      for (int b = 0; b < D; ++b)
#pragma unroll
        for (int a = 0; a < D; ++a) Pbar[a + D * b] += gw * u * r[a] * gb[b];
    }
    double ee = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) ee += eb[a] * ev[a];
    const double radial = Wb * g2 - ub * u * u;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      xb[a] += rb[a] + u * (eb[a] - ee * ev[a]) + radial * ev[a];
      vb[a] += f_d * gb[a];
    }
    Bbar += fdb * eta * gw * u;
    Abar += fcb * gw;
    etab += 0.5 * fdb * SB * gw * u;
  }
  for (int o = 1; o < split; o <<= 1) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      xb[a] += __shfl_xor_sync(0xffffffffu, xb[a], o);
      vb[a] += __shfl_xor_sync(0xffffffffu, vb[a], o);
    }
    if (NNW) {
#pragma unroll
      for (int q = 0; q < D2; ++q) Pbar[q] += __shfl_xor_sync(0xffffffffu, Pbar[q], o);
    }
    Bbar += __shfl_xor_sync(0xffffffffu, Bbar, o);
    Abar += __shfl_xor_sync(0xffffffffu, Abar, o);
    nbL += __shfl_xor_sync(0xffffffffu, nbL, o);
    etab += __shfl_xor_sync(0xffffffffu, etab, o);
  }
  if (!live || part != 0) return;
  // per-particle chain: A = (p + G) B, B = 1/n^2, Q = G c B, p = EOS(n m)
  const double Bi = pci.y, p = pci.w, mi = 1.0 / pci.z;
  const double pbar = Abar * Bi;
  double Bt = Bbar + Abar * (p + G);
  if (NNW) {
#pragma unroll
    for (int q = 0; q < D2; ++q) {
      Bt += G * ci[q] * Pbar[q];
      cbs[(size_t)q * n + i] += G * Bi * Pbar[q];
    }
  }
  const double r_eos = ni * mi;
  double dpdn;
  if (k.eos_type == 1)
    dpdn = k.c2 * ((k.gamma == 1.0) ? 1.0 : k.gamma * pow(r_eos, k.gamma - 1.0)) * mi;
  else
    dpdn = k.p0 * ((k.gamma == 1.0) ? 1.0 : k.gamma * pow(r_eos / k.rho_ref, k.gamma - 1.0)) *
           mi / k.rho_ref;
  nbar[i] = Bt * (-2.0 * Bi * qi) + nbL + pbar * dpdn;
  double4_32a xo = xbs[i], vo = vbs[i];
  xo.x += xb[0];
  xo.y += xb[1];
  vo.x += vb[0];
  vo.y += vb[1];
  if (D == 3) {
    xo.z += xb[2];
    vo.z += vb[2];
  }
  xbs[i] = xo;
  vbs[i] = vo;
  const int hi = tp.hidx[i];
  const double csound = sqrt(k.c2);
  gp[hi] += etab;
  gp[(size_t)2 * n + hi] += (csound > 0.0) ? pbar * 2.0 * p / csound : 0.0;
}

// density VJP, x_i gets sum_j (nbar_i + nbar_j) W'(r_ij) e_ij, then the
// drift: the carried adjoints of the previous step, in host order
template <int D, bool NNW>
__global__ void __launch_bounds__(kAdjTPB)
    k_adj_density(Consts k, Tape tp, const double* __restrict__ nbar,
                  const double4_32a* __restrict__ xbs, const double4_32a* __restrict__ vbs,
                  const double* __restrict__ cbs, int drift, double dt,
                  double4_32a* __restrict__ xb_h, double4_32a* __restrict__ vb_h,
                  double* __restrict__ cb_h, int split) {
  __shared__ int s_start[kMaxStencil * kAdjTPB];
  __shared__ int s_shift[kMaxStencil * kAdjTPB];
  const int n = k.n;
  const int tid = threadIdx.x;
  const int g_ = blockIdx.x * kAdjTPB + tid;
  const int i0 = g_ / split, part = g_ - i0 * split;
  const bool live = i0 < n;
  const int i = live ? i0 : n - 1;
  build_lane_table<D, kAdjTPB>(k, tp.cell_of[i], tp.cell_start, s_start, s_shift);
  const double4_32a xi4 = tp.x[i];
  const double xi[3] = {xi4.x, xi4.y, xi4.z};
  const double nbi = nbar[i];
  double acc[3] = {0, 0, 0};
  const int cnt = live ? tp.ncount[i] : 0;
  for (int e = part; e < cnt; e += split) {
    const int ent = tp.nl[(size_t)e * n + i];
    const int sl = ent >> kLocalBits, q = ent & (kMaxCellCount - 1);
    const int j = s_start[sl * kAdjTPB + tid] + q;
    const double4_32a xj4 = tp.x[j];
    const double xj[3] = {xj4.x, xj4.y, xj4.z};
    double r[3];
    const double dd2 = exact_sep<D>(k, xi, xj, s_shift[sl * kAdjTPB + tid], r);
    const double dist = sqrt(dd2);
    const double f = (nbi + nbar[j]) * kernel_gradw<double>(k, dist) / dist;
#pragma unroll
    for (int a = 0; a < D; ++a) acc[a] += f * r[a];
  }
  for (int o = 1; o < split; o <<= 1) {
#pragma unroll
    for (int a = 0; a < 3; ++a) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], o);
  }
  if (!live || part != 0) return;
  const int hi = tp.hidx[i];
  double4_32a xo = xbs[i], vo = vbs[i];
  xo.x += acc[0];
  xo.y += acc[1];
  if (D == 3) xo.z += acc[2];
  if (drift) {
    vo.x += dt * xo.x;
    vo.y += dt * xo.y;
    if (D == 3) vo.z += dt * xo.z;
  }
  xb_h[hi] = xo;
  vb_h[hi] = vo;
  if (NNW) {
#pragma unroll
    for (int q = 0; q < D * D; ++q) cb_h[(size_t)q * n + hi] = cbs[(size_t)q * n + i];
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

int grid1(int n) { return std::max(1, (n + 255) / 256); }

int launched(Handle* h, const char* what, int count = 1) {
  h->launches += count;
  return cuda_check(h, cudaGetLastError(), what) ? MCFG_ECUDA : MCFG_OK;
}

int save_ckpt(Handle* h, Ckpt& c) {
  const int n = (int)h->n, d2 = h->k.d * h->k.d;
  k_ck_save<<<grid1(n), 256, 0, h->stream>>>(n, d2, h->hidx, h->x, h->v, h->f, h->ct, h->act,
                                             h->rho, h->pr, h->st, c);
  return launched(h, "checkpoint save");
}

int restore_ckpt(Handle* h, const Ckpt& c) {
  const int n = (int)h->n, d2 = h->k.d * h->k.d;
  AdjBuffers* b = h->adj;
  k_ck_restore<<<grid1(n), 256, 0, h->stream>>>(n, d2, c, b->m_h, b->pid_h, b->sid_h, h->x,
                                                h->v, h->f, h->ct, h->act, h->rho, h->pr,
                                                h->st, h->m, h->pid, h->sid, h->hidx);
  return launched(h, "checkpoint restore");
}

int record_tape(Handle* h, const Tape& t) {
  PhaseScope ps(h, kPhaseOther);
  const int n = (int)h->n, d2 = h->k.d * h->k.d, nc2 = h->k.ncell + 2;
  k_tape_record<<<grid1(std::max(n, nc2)), 256, 0, h->stream>>>(
      n, nc2, d2, t, h->x, h->v, h->pc, h->rho, h->pid, h->hidx, h->ncount, h->cell_of,
      h->cell_start, h->nl, h->ct, h->vgt);
  return launched(h, "tape record");
}

// one forward VV step with the unfused tail, so that v' and c' survive the
// right-hand side for the tape (bit-identical to mcfg_step_vv)
int forward_step(Handle* h, int64_t step, double dt, const Tape* tape, double* jrow) {
  ATRY(kdw(h, dt));
  // the recomputation needs no stress (J is summed in the first pass)
  const int stress = h->k.stress;
  if (jrow == nullptr) h->k.stress = 0;
  const int rc = rhs(h, step, kForceBody, dt);
  h->k.stress = stress;
  ATRY(rc);
  if (tape) ATRY(record_tape(h, *tape));
  if (jrow) {
    AdjBuffers* b = h->adj;
    k_stress_dot<<<b->nb, kAdjRedThreads, 0, h->stream>>>((int)h->n, h->k.d * h->k.d, b->w,
                                                          h->st, h->sid, jrow);
    ATRY(launched(h, "stress dot"));
  }
  return kick_ct_half(h, dt);
}

int adjoint_step(Handle* h, const Tape& tp, int64_t step, double dt, double phi, int drift,
                 double wscale, cudaStream_t s) {
  AdjBuffers* b = h->adj;
  const Consts& k = h->k;
  const int n = (int)h->n;
  const double inv_sqdt = k.noise ? 1.0 / sqrt(dt) : 0.0;
  const int gp_ = std::max(1, (n + kAdjTPB - 1) / kAdjTPB);
  // lanes per particle in the pair sweeps: small systems fill the GPU with
  // more threads (the neighbour entries are dealt round-robin)
  const int split = n < 150000 ? 4 : (n < 600000 ? 2 : 1);
  const int gs_ = std::max(1, (int)(((int64_t)n * split + kAdjTPB - 1) / kAdjTPB));
#define ADJ_LAUNCH(DD, NW)                                                                     \
  do {                                                                                         \
    k_adj_pre<DD, NW><<<grid1(n), 256, 0, s>>>(k, tp, phi, b->xb_h, b->vb_h, b->cb_h, b->lam,  \
                                               b->xbs, b->vbs, b->cbs, b->Lb, b->qb, b->gp);   \
    k_adj_force<DD, NW><<<gs_, kAdjTPB, 0, s>>>(k, tp, b->lam, b->Lb, b->qb, b->w, wscale,        \
                                             (uint32_t)step, inv_sqdt, b->xbs, b->vbs, b->cbs, \
                                             b->nbar, b->gp, split);                           \
    k_adj_density<DD, NW><<<gs_, kAdjTPB, 0, s>>>(k, tp, b->nbar, b->xbs, b->vbs, b->cbs, drift,  \
                                               dt, b->xb_h, b->vb_h, b->cb_h, split);          \
  } while (0)
  if (k.d == 3) {
    if (k.newtonian) ADJ_LAUNCH(3, false); else ADJ_LAUNCH(3, true);
  } else {
    if (k.newtonian) ADJ_LAUNCH(2, false); else ADJ_LAUNCH(2, true);
  }
#undef ADJ_LAUNCH
  return launched(h, "adjoint step", 3);
}

const char* adjoint_unsupported(const Handle* h) {
  const mcfg_params& p = h->p;
  if (p.precision != MCFG_PRECISION_FP64) return "the adjoint needs precision FP64";
  if (p.rhs_density_type != 2) return "the adjoint needs rhs_density_type 2 (number density)";
  if (p.rhs_force_type != 3) return "the adjoint needs rhs_force_type 3 (Hu-Adams)";
  if (!p.stress_tensor) return "the adjoint needs stress_tensor on (J is built from the stress)";
  for (int f = 0; f < 2 * p.num_dim; ++f)
    if (p.bcdef[f] != MCFG_BC_PERIODIC) return "the adjoint needs a fully periodic box";
  if (h->n_boundary != 0 || h->k.ncoll != 0)
    return "the adjoint needs an all-fluid system (no wall or colloid particles)";
  return nullptr;
}

int download_vec(Handle* h, const double4_32a* src, double* host, int d) {
  const int n = (int)h->n;
  std::vector<double4_32a> buf((size_t)n);
  if (cuda_check(h, cudaMemcpyAsync(buf.data(), src, sizeof(double4_32a) * (size_t)n,
                                    cudaMemcpyDeviceToHost, h->stream),
                 "adjoint download") ||
      cuda_check(h, cudaStreamSynchronize(h->stream), "adjoint download sync"))
    return MCFG_ECUDA;
  for (int i = 0; i < n; ++i) {
    host[(size_t)i * d] = buf[(size_t)i].x;
    host[(size_t)i * d + 1] = buf[(size_t)i].y;
    if (d == 3) host[(size_t)i * d + 2] = buf[(size_t)i].z;
  }
  return MCFG_OK;
}

}  // namespace

}  // namespace mcfg

using namespace mcfg;

extern "C" int mcfg_adjoint_run(mcfg_handle* h, int64_t step0, int32_t nsteps, double dt,
                                int32_t checkpoint_every, const double* w, double* J,
                                double* dJ_dparams, double* dJ_dx0, double* dJ_dv0,
                                double* dJ_dct0) {
  if (h) h->graph_gen++;
  if (!h) return MCFG_EINVAL;
  if (cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice")) return MCFG_ECUDA;
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  if (nsteps < 1) return set_error(h, MCFG_EINVAL, "nsteps must be >= 1");
  if (!(dt > 0.0)) return set_error(h, MCFG_EINVAL, "dt must be positive");
  if (!w) return set_error(h, MCFG_EINVAL, "stress weights w are required");
  if (dJ_dct0 && h->p.Newtonian)
    return set_error(h, MCFG_EINVAL, "no conformation tensor (Newtonian)");
  if (const char* why = adjoint_unsupported(h)) return set_error(h, MCFG_ENOTSUP, why);
  const int n = (int)h->n, d = h->k.d, d2 = d * d;
  if (n == 0) return set_error(h, MCFG_EINVAL, "no particles");
  int K = checkpoint_every > 0 ? checkpoint_every : 20;
  if (K > nsteps) K = nsteps;
  const int T = nsteps, nseg = (T + K - 1) / K;
  ATRY(ensure_buffers(h, K, T));
  AdjBuffers* b = h->adj;
  cudaStream_t s = h->stream;
  {
    double wv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < d2; ++q) wv[q] = w[q];
    if (cuda_check(h, cudaMemcpyAsync(b->w, wv, sizeof wv, cudaMemcpyHostToDevice, s),
                   "weights") ||
        cuda_check(h, cudaStreamSynchronize(s), "weights sync"))
      return MCFG_ECUDA;
  }
  h->dt = dt;
  // ---- first pass: J and the checkpoints ----
  ATRY(adjust_particles(h));
  k_consts_save<<<grid1(n), 256, 0, s>>>(n, h->hidx, h->m, h->pid, h->sid, b->m_h, b->pid_h,
                                         b->sid_h);
  ATRY(launched(h, "save constants"));
  ATRY(save_ckpt(h, b->ck[0]));
  ATRY(rhs(h, step0, kForceBody, dt));
  // the last segment is taped on the way (it is walked back first, with no
  // recomputation)
  const int klast = (nseg - 1) * K;
  if (nseg == 1) ATRY(record_tape(h, b->tape[(size_t)K]));
  for (int t = 1; t <= T; ++t) {
    if (t > 1 && (t - 1) % K == 0) ATRY(save_ckpt(h, b->ck[(size_t)((t - 1) / K)]));
    const Tape* tp = (t > klast) ? &b->tape[(size_t)(t - klast - 1)] : nullptr;
    ATRY(forward_step(h, step0 + t, dt, tp, b->jpart + (size_t)(t - 1) * b->nb));
  }
  ATRY(save_ckpt(h, b->last));
  ATRY(check_device_errors(h));
  // ---- reverse sweep ----
  if (cuda_check(h, cudaMemsetAsync(b->xb_h, 0, sizeof(double4_32a) * (size_t)n, s), "zero") ||
      cuda_check(h, cudaMemsetAsync(b->vb_h, 0, sizeof(double4_32a) * (size_t)n, s), "zero") ||
      cuda_check(h, cudaMemsetAsync(b->gp, 0, sizeof(double) * 3 * (size_t)n, s), "zero"))
    return MCFG_ECUDA;
  if (b->cb_h &&
      cuda_check(h, cudaMemsetAsync(b->cb_h, 0, sizeof(double) * (size_t)d2 * n, s), "zero"))
    return MCFG_ECUDA;
  const double wscale = 1.0 / (double)T;
  // segment sg recomputed from its checkpoint into a tape set
  auto recompute = [&](int sg, std::vector<Tape>& set) -> int {
    const int k0 = sg * K, k1 = std::min(k0 + K, T);
    ATRY(restore_ckpt(h, b->ck[(size_t)sg]));
    if (sg == 0) {
      ATRY(rhs(h, step0, kForceBody, dt));
      ATRY(record_tape(h, set[(size_t)K]));
    }
    for (int t = k0 + 1; t <= k1; ++t)
      ATRY(forward_step(h, step0 + t, dt, &set[(size_t)(t - k0 - 1)], nullptr));
    return MCFG_OK;
  };
  // segment sg walked backwards from a tape set
  auto reverse = [&](int sg, std::vector<Tape>& set, cudaStream_t st) -> int {
    const int k0 = sg * K, k1 = std::min(k0 + K, T);
    for (int t = k1; t > k0; --t)
      ATRY(adjoint_step(h, set[(size_t)(t - k0 - 1)], step0 + t, dt, t == T ? 0.5 * dt : dt, 1,
                        wscale, st));
    if (sg == 0) ATRY(adjoint_step(h, set[(size_t)K], step0, dt, 0.5 * dt, 0, 0.0, st));
    return MCFG_OK;
  };
  if (b->tape2.empty()) {
    for (int sg = nseg - 1; sg >= 0; --sg) {
      if (sg < nseg - 1) ATRY(recompute(sg, b->tape));
      ATRY(reverse(sg, b->tape, s));
    }
  } else {
    // two tape sets: while segment sg is walked back on rs from one set,
    // segment sg - 1 is recomputed on the handle's stream into the other
    // (the reverse sweep reads only tapes and adjoint buffers, so the two
    // streams share no data but the tape sets; the arithmetic and its order
    // are those of the sequential sweep)
    std::vector<Tape>* sets[2] = {&b->tape, &b->tape2};
    int cur = 0;  // the first pass taped the last segment into set 0
    if (cuda_check(h, cudaEventRecord(b->ev_fill[0], s), "tape event")) return MCFG_ECUDA;
    for (int sg = nseg - 1; sg >= 0; --sg) {
      if (sg > 0) {
        // set cur ^ 1 was last read by the reverse of segment sg + 1
        if (cuda_check(h, cudaStreamWaitEvent(s, b->ev_read[cur ^ 1], 0), "tape wait"))
          return MCFG_ECUDA;
        ATRY(recompute(sg - 1, *sets[cur ^ 1]));
        if (cuda_check(h, cudaEventRecord(b->ev_fill[cur ^ 1], s), "tape event"))
          return MCFG_ECUDA;
      }
      if (cuda_check(h, cudaStreamWaitEvent(b->rs, b->ev_fill[cur], 0), "tape wait"))
        return MCFG_ECUDA;
      ATRY(reverse(sg, *sets[cur], b->rs));
      if (cuda_check(h, cudaEventRecord(b->ev_read[cur], b->rs), "tape event"))
        return MCFG_ECUDA;
      cur ^= 1;
    }
    // the outputs below read the adjoint buffers on the handle's stream
    if (cuda_check(h, cudaStreamWaitEvent(s, b->ev_read[cur ^ 1], 0), "reverse wait"))
      return MCFG_ECUDA;
  }
  ATRY(restore_ckpt(h, b->last));
  h->have_list = false;
  h->have_density = h->have_pressure = h->have_force = true;
  ATRY(check_device_errors(h));
  // ---- outputs ----
  if (J) {
    std::vector<double> jp((size_t)T * b->nb);
    if (cuda_check(h, cudaMemcpy(jp.data(), b->jpart, sizeof(double) * jp.size(),
                                 cudaMemcpyDeviceToHost),
                   "J copy"))
      return MCFG_ECUDA;
    double acc = 0.0;
    for (int t = 0; t < T; ++t) {
      double st = 0.0;
      for (int q = 0; q < b->nb; ++q) st += jp[(size_t)t * b->nb + q];
      acc += st;
    }
    *J = acc / (double)T;
  }
  if (dJ_dparams) {
    k_row_sums<<<b->nb, kAdjRedThreads, 0, s>>>(n, 3, b->gp, b->red);
    ATRY(launched(h, "parameter sums"));
    std::vector<double> r((size_t)3 * b->nb);
    if (cuda_check(h, cudaMemcpyAsync(r.data(), b->red, sizeof(double) * r.size(),
                                      cudaMemcpyDeviceToHost, s),
                   "parameter copy") ||
        cuda_check(h, cudaStreamSynchronize(s), "parameter sync"))
      return MCFG_ECUDA;
    for (int q = 0; q < 3; ++q) {
      double acc = 0.0;
      for (int c = 0; c < b->nb; ++c) acc += r[(size_t)q * b->nb + c];
      dJ_dparams[q] = acc;
    }
  }
  if (dJ_dx0) ATRY(download_vec(h, b->xb_h, dJ_dx0, d));
  if (dJ_dv0) ATRY(download_vec(h, b->vb_h, dJ_dv0, d));
  if (dJ_dct0) {
    std::vector<double> c((size_t)d2 * n);
    if (cuda_check(h, cudaMemcpy(c.data(), b->cb_h, sizeof(double) * c.size(),
                                 cudaMemcpyDeviceToHost),
                   "ct adjoint copy"))
      return MCFG_ECUDA;
    for (int i = 0; i < n; ++i)
      for (int q = 0; q < d2; ++q) dJ_dct0[(size_t)i * d2 + q] = c[(size_t)q * n + i];
  }
  return MCFG_OK;
}
