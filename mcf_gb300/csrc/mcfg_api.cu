// mcfg_api.cu -- the extern "C" boundary (include/mcfg.h): parameter checks,
// device memory, host<->device layout conversion and the orchestration of
// the per-step kernels.  Every entry point returns a status; none aborts.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <string>

#include "mcfg_internal.cuh"
#include "sph.cuh"

using namespace mcfg;

namespace mcfg {

int set_error(Handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_check(Handle* h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  h->err = buf;
  // consume the thread's last-error state: a failed call that leaves the
  // context usable (a bad argument, an unregistered pointer) must not fail
  // the next launch check of this or another handle
  cudaGetLastError();
  return MCFG_ECUDA;
}

void resolve_phases(Handle* h) {
  for (int ph = 0; ph < 5; ++ph) {
    for (auto& ev : h->ev_pending[ph]) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, ev.first, ev.second) == cudaSuccess) {
        h->phase_ms[ph] += ms;
        h->phase_cnt[ph] += 1;
      }
      h->ev_pool.push_back(ev);
    }
    h->ev_pending[ph].clear();
  }
}

#define TRY_STATUS(expr) \
  do {                    \
    int _rc = (expr);     \
    if (_rc) return _rc;  \
  } while (0)

// the device status words into h->h_status (pinned), on the handle's stream
static int status_copy_async(Handle* h) {
  if (!h->h_status &&
      cuda_check(h, cudaHostAlloc((void**)&h->h_status, sizeof(Handle::HostStatus),
                                  cudaHostAllocDefault),
                 "status buffer"))
    return MCFG_ECUDA;
  Handle::HostStatus* hs = h->h_status;
  if (cuda_check(h, cudaMemcpyAsync(&hs->err, h->d_err, sizeof hs->err, cudaMemcpyDeviceToHost,
                                    h->stream),
                 "error flag copy") ||
      cuda_check(h, cudaMemcpyAsync(hs->stats, h->d_stats, sizeof hs->stats,
                                    cudaMemcpyDeviceToHost, h->stream),
                 "stats copy") ||
      cuda_check(h, cudaMemcpyAsync(&hs->pairs, h->d_pairs, sizeof hs->pairs,
                                    cudaMemcpyDeviceToHost, h->stream),
                 "pairs copy"))
    return MCFG_ECUDA;
  return MCFG_OK;
}

// the status words copied by status_copy_async, after the stream's sync
static int status_evaluate(Handle* h) {
  const unsigned e = h->h_status->err;
  int st[4];
  for (int q = 0; q < 4; ++q) st[q] = h->h_status->stats[q];
  const unsigned long long pairs = h->h_status->pairs;
  resolve_phases(h);
  h->max_neigh = st[1];
  h->num_pairs = (int64_t)pairs;
  if (e) {
    cudaMemsetAsync(h->d_err, 0, sizeof(unsigned), h->stream);
    if (e & kErrNeighOverflow) {
      char buf[200];
      snprintf(buf, sizeof buf,
               "neighbour list overflow: a particle has %d candidates, capacity %d "
               "(raise mcfg_params.reserved[0])",
               st[1], h->neigh_cap);
      return set_error(h, MCFG_EOVERFLOW, buf);
    }
    if (e & kErrCellOverflow)
      return set_error(h, MCFG_EOVERFLOW, "a cell holds more than 2048 particles");
    if (e & kErrZeroDensity) return set_error(h, MCFG_EPHYS, "non-positive density");
    if (e & kErrNonFinite) return set_error(h, MCFG_EPHYS, "non-finite acceleration");
  }
  return MCFG_OK;
}

int check_device_errors(Handle* h) {
  TRY_STATUS(status_copy_async(h));
  if (cuda_check(h, cudaStreamSynchronize(h->stream), "synchronize")) return MCFG_ECUDA;
  return status_evaluate(h);
}

}  // namespace mcfg

namespace {

std::mutex g_create_mu;
std::string g_create_err = "no error";

template <typename T>
int dalloc(Handle* h, T** p, size_t count) {
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
  }
  if (count == 0) count = 1;
  const size_t bytes = sizeof(T) * count;
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    char buf[160];
    snprintf(buf, sizeof buf, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    h->err = buf;
    return MCFG_ENOMEM;
  }
  h->device_bytes += (int64_t)bytes;
  return MCFG_OK;
}

void free_all(Handle* h) {
  free_adjoint(h);
  destroy_graphs(h);
  h->graph_gen++;
  if (h->d_step) cudaFree(h->d_step);
  h->d_step = nullptr;
  if (h->out_dev) cudaFree(h->out_dev);
  if (h->out_host) cudaFreeHost(h->out_host);
  h->out_dev = nullptr;
  h->out_host = nullptr;
  h->out_cap = 0;
  for (void* p : {(void*)h->x_ref, (void*)h->vl, (void*)h->vcount, (void*)h->d_rebuild})
    if (p) cudaFree(p);
  h->x_ref = nullptr;
  h->vl = nullptr;
  h->vcount = h->d_rebuild = nullptr;
  h->vcap = 0;
  h->reuse_valid = false;
  void* ptrs[] = {h->x, h->v, h->f, h->m, h->pid, h->sid, h->hidx, h->rho, h->pr, h->st,
                  h->x2, h->v2, h->f2, h->m2, h->pid2, h->sid2, h->hidx2, h->key, h->rank,
                  h->cnt, h->cell_start, h->scan_part, h->order, h->off, h->cell_of, h->nl,
                  h->ncount, h->nhs, h->jp, h->pc, h->pcf, h->vf, h->wd, h->red, h->d_err, h->d_stats, h->d_pairs,
                  h->up_x, h->up_v, h->up_m, h->up_id, h->ct, h->act, h->vgt, h->ct2,
                  h->act2, h->qq, h->coll, h->coll_start, h->coll_mem, h->slot_of, h->rxc,
                  h->rxcf, h->coll_out, h->crec, h->cxnew};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  h->x = h->v = h->f = h->x2 = h->v2 = h->f2 = nullptr;
  h->m = h->m2 = h->rho = h->pr = h->st = h->red = h->up_x = h->up_v = h->up_m = nullptr;
  h->pid = h->sid = h->hidx = h->pid2 = h->sid2 = h->hidx2 = nullptr;
  h->key = h->rank = h->cnt = h->cell_start = h->scan_part = h->order = h->cell_of = nullptr;
  h->ncount = h->d_stats = h->up_id = h->nhs = nullptr;
  h->jp = nullptr;
  h->ct = h->act = h->vgt = h->ct2 = h->act2 = nullptr;
  h->qq = nullptr;
  h->coll = h->coll_out = nullptr;
  h->crec = h->cxnew = nullptr;
  h->cdyn = false;
  h->coll_host_stale = false;
  h->coll_start = h->coll_mem = h->slot_of = nullptr;
  h->rxc = nullptr;
  h->rxcf = nullptr;
  h->k.coll = nullptr;
  h->k.ncoll = 0;
  h->off = h->pcf = h->vf = nullptr;
  h->wd = nullptr;
  h->pc = nullptr;
  h->nl = nullptr;
  h->d_err = nullptr;
  h->d_pairs = nullptr;
  h->device_bytes = 0;
}

}  // namespace

namespace mcfg {

const char* validate_params(const mcfg_params* p) {
  if (!p) return "params is NULL";
  if (p->num_dim != 2 && p->num_dim != 3) return "num_dim must be 2 or 3";
  if (!(p->cut_off > 0.0)) return "cut_off must be positive";
  if (p->kernel_type != 1 && p->kernel_type != 2) return "kernel_type must be 1 or 2";
  if (p->rhs_density_type != 1 && p->rhs_density_type != 2)
    return "rhs_density_type must be 1 or 2";
  if (p->rhs_force_type < 1 || p->rhs_force_type > 4) return "rhs_force_type must be 1..4";
  if (p->stateEquation_type != 1 && p->stateEquation_type != 2)
    return "stateEquation_type must be 1 or 2";
  if (p->body_force_type < 0 || p->body_force_type > 3) return "body_force_type must be 0..3";
  if (p->precision != MCFG_PRECISION_FP64 && p->precision != MCFG_PRECISION_FP32_MIXED)
    return "precision must be MCFG_PRECISION_FP64 or MCFG_PRECISION_FP32_MIXED";
  if (!p->Newtonian && p->rhs_force_type != 3)
    return "the Oldroyd-B model needs rhs_force_type 3 (Hu-Adams)";
  if (!p->Newtonian && !(std::fabs(p->tau) > 1e-14)) return "tau should not be zero";
  const bool le = p->bcdef[2] == MCFG_BC_LE || p->bcdef[3] == MCFG_BC_LE;
  for (int a = 0; a < p->num_dim; ++a) {
    const int lo = p->bcdef[2 * a], hi = p->bcdef[2 * a + 1];
    const bool le_ok = (a == 1 && lo == MCFG_BC_LE && hi == MCFG_BC_LE);
    auto plain = [](int b) {
      return b == MCFG_BC_PERIODIC || b == MCFG_BC_FREESPACE || b == MCFG_BC_WALL_SOLID;
    };
    if (!le_ok && (!plain(lo) || !plain(hi)))
      return "bcdef: periodic (1), freespace (2) and solid wall (9) faces, Lees-Edwards (10) "
             "on both y faces";
    if ((lo == MCFG_BC_PERIODIC) != (hi == MCFG_BC_PERIODIC))
      return "bcdef: a periodic face needs a periodic opposite face";
    if (le && a != 1) {
      // the images' x (and z) are MODULO(x + shear_length, L): the box
      // starts at 0 on the other axes, which are periodic
      if (lo != MCFG_BC_PERIODIC)
        return "Lees-Edwards y faces need periodic x (and z) faces, no solid walls";
      if (p->min_phys_t[a] != 0.0 || p->min_phys[a] != 0.0)
        return "Lees-Edwards: the box must start at 0 along x (and z)";
    }
    if (!(p->max_phys_t[a] > p->min_phys_t[a])) return "max_phys_t must exceed min_phys_t";
    if (!(p->max_phys[a] > p->min_phys[a])) return "max_phys must exceed min_phys";
  }
  if (le && p->num_dim == 3 && p->wall_v[2][2] != p->wall_v[3][2])
    return "Lees-Edwards: the y faces may slide only along x (wall_v[2][2] == wall_v[3][2])";
  if (p->rhs_force_type == 1 && p->rhs_density_type != 1)
    return "rhs_force_type 1 (Morris) needs rhs_density_type 1 (mass density)";
  if (p->stateEquation_type == 2 && (p->rho_ref == 0.0 || p->gamma == 0.0))
    return "Batchelor EOS needs non-zero rho_ref and gamma";
  return nullptr;
}

}  // namespace mcfg

namespace {

}  // namespace

namespace mcfg {

void make_consts(const mcfg_params& p, Consts& k) {
  memset(&k, 0, sizeof k);
  k.d = p.num_dim;
  const double cf = p.cell_factor > 0.0 ? p.cell_factor : 1.0001;
  const double gs = p.cut_off * cf;  // mcf.F90:617
  k.ncell = 1;
  for (int a = 0; a < 3; ++a) {
    k.nm[a] = 1;
    k.csf[a] = 0.0f;
  }
  for (int a = 0; a < k.d; ++a) {
    k.xmin[a] = p.min_phys_t[a];
    k.xmax[a] = p.max_phys_t[a];
    int nm = (int)((k.xmax[a] - k.xmin[a]) / gs);  // ppm_neighlist_clist.F90:370-376
    if (nm < 1) nm = 1;
    k.nm[a] = nm;
    k.ncell *= nm;
    k.rdx[a] = (double)nm / (k.xmax[a] - k.xmin[a]);
    k.cs[a] = (k.xmax[a] - k.xmin[a]) / (double)nm;
    k.csf[a] = (float)k.cs[a];
    k.len[a] = p.max_phys_t[a] - p.min_phys_t[a];
    k.bc_lo[a] = p.bcdef[2 * a];
    k.bc_hi[a] = p.bcdef[2 * a + 1];
    k.periodic[a] = (p.bcdef[2 * a] == MCFG_BC_PERIODIC) ? 1 : 0;
    k.min_phys[a] = p.min_phys[a];
    k.max_phys[a] = p.max_phys[a];
  }
  k.rc2 = p.cut_off * p.cut_off;
  k.rc2f = (float)k.rc2;
  // Lees-Edwards y faces: 3 (2D: 1) more stencil slots for the fourth x
  // cell of the row across the face; the offsets follow the time
  // (boundary_update)
  k.le = (k.d >= 2 && p.bcdef[2] == MCFG_BC_LE) ? 1 : 0;
  k.ns = (k.d == 3 ? 27 : 9) + (k.le ? (k.d == 3 ? 3 : 1) : 0);
  k.walls = 0;
  for (int f = 0; f < 2 * k.d; ++f)
    if (p.bcdef[f] == MCFG_BC_WALL_SOLID) k.walls = 1;
  k.reuse = 0;
  k.le_dS = 0.0;
  if (p.reserved[1] != 0) {
    double csmin = 1e300;
    for (int a = 0; a < k.d; ++a) csmin = std::min(csmin, k.cs[a]);
    const double skin = 0.99 * (csmin - p.cut_off);
    if (skin > 0.0) {
      k.reuse = 1;
      k.half_skin2 = 0.25 * skin * skin;
      k.half_skin_le2 = k.half_skin2;
      const double rv = p.cut_off + skin;
      k.rv2f = (float)(rv * rv * (1.0 + 1e-4));
    }
  }
  // FP32 prefilter of the FP64 path: relative slack far above the FP32
  // rounding of cell offsets (|offset| <= cell side)
  k.rc2f_hi = (float)(k.rc2 * (1.0 + 1e-4));
  // kernel_new.F90:41-93
  k.kernel_type = p.kernel_type;
  if (p.kernel_type == 1) {
    k.h = p.cut_off / 3.0;
    k.coef = (k.d == 2) ? 7.0 / (478.0 * kPi * k.h * k.h) : 3.0 / (359.0 * kPi * k.h * k.h * k.h);
  } else {
    k.h = p.cut_off;
    k.coef = (k.d == 2) ? 5.0 / (kPi * k.h * k.h) : 105.0 / (16.0 * kPi * k.h * k.h * k.h);
  }
  k.coef_grad = -k.coef / k.h;
  k.inv_h = 1.0 / k.h;
  k.w0 = (p.kernel_type == 1) ? k.coef * (243.0 - 6.0 * 32.0 + 15.0) : k.coef;
  k.hf = (float)k.h;
  k.inv_hf = (float)k.inv_h;
  k.coeff = (float)k.coef;
  k.coef_gradf = (float)k.coef_grad;
  k.w0f = (float)k.w0;
  k.etaf = (float)p.eta;
  k.eta_coeff = (float)p.eta_coef;
  k.ktf = (float)p.kt;
  k.wall_axis = -1;
  for (int a = 0; a < k.d; ++a)
    if (p.bcdef[2 * a] == MCFG_BC_WALL_SOLID) k.wall_axis = (k.wall_axis == -1) ? a : -2;
  k.rhs_density_type = p.rhs_density_type;
  k.rhs_force_type = p.rhs_force_type;
  k.eos_type = p.stateEquation_type;
  k.c2 = p.c * p.c;
  k.rho_ref = p.rho_ref;
  k.gamma = p.gamma;
  if (p.stateEquation_type == 2)  // stateEquation_new.F90:102-103
    k.p0 = p.c * p.c * p.rho * std::pow(p.rho_ref / p.rho, p.gamma) / p.gamma;
  k.eta = p.eta;
  k.eta_coef = p.eta_coef;
  k.kt = p.kt;
  k.machine_zero = 1e-14;  // technique_new.F90:361-363
  k.noise = (p.Brownian && p.kt > k.machine_zero) ? 1 : 0;
  k.wall_rho_type = p.wall_rho_type;
  k.wall_noslip_type = p.wall_noslip_type;
  k.init_density = p.init_density;
  for (int f = 0; f < 6; ++f)
    for (int a = 0; a < 3; ++a) {
      k.wall_v[f][a] = p.wall_v[f][a];
      k.wall_vf[f][a] = (float)p.wall_v[f][a];
      k.wall_v_end[f][a] = p.wall_v[f][a];
    }
  if (k.le) k.le_dv = p.wall_v[3][0] - p.wall_v[2][0];
  k.stress = p.stress_tensor ? 1 : 0;
  k.newtonian = p.Newtonian ? 1 : 0;
  k.G = p.n_p * p.kt_p;
  k.tau = p.tau;
  k.inv_tau = p.Newtonian ? 0.0 : 1.0 / p.tau;
  k.key0 = (uint32_t)p.seed;
  k.key1 = (uint32_t)(p.seed >> 32);
  for (int r = 0; r < 10; ++r) {
    k.rk[2 * r] = k.key0 + (uint32_t)r * 0x9E3779B9u;
    k.rk[2 * r + 1] = k.key1 + (uint32_t)r * 0xBB67AE85u;
  }
  k.body_force_type = p.body_force_type;
  for (int a = 0; a < 3; ++a) k.body_force[a] = p.body_force[a];
}

}  // namespace mcfg

namespace {

void fill_consts(Handle* h) {
  make_consts(h->p, h->k);
  h->le_skin = h->k.reuse ? 2.0 * std::sqrt(h->k.half_skin2) : 0.0;
  h->le_reach = h->p.cut_off + h->le_skin;
  h->k.le_y0 = 0.5 * (h->k.min_phys[1] + h->k.max_phys[1]);
}

// conformation tensor: host (d*d, N) interleaved -> device [c][n]; identity
// when no host array is given (particles_init_partial_inter.F90:145-148)
__global__ void k_upload_ct(int n, int d, const double* __restrict__ hct, double* __restrict__ ct,
                            double* __restrict__ act) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int d2 = d * d;
  for (int c = 0; c < d2; ++c) {
    ct[(size_t)c * n + i] = hct ? hct[(size_t)i * d2 + c] : ((c % (d + 1)) == 0 ? 1.0 : 0.0);
    act[(size_t)c * n + i] = 0.0;
  }
}

__global__ void k_upload(int n, int d, const double* __restrict__ hx, const double* __restrict__ hv,
                         const double* __restrict__ hm, const int* __restrict__ hid,
                         double4_32a* __restrict__ x, double4_32a* __restrict__ v,
                         double4_32a* __restrict__ f, double* __restrict__ m, int* __restrict__ pid,
                         int* __restrict__ sid, int* __restrict__ hidx, int* __restrict__ slot_of) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* xp = hx + (size_t)i * d;
  const double* vp = hv + (size_t)i * d;
  x[i] = make_double4_32a(xp[0], xp[1], d == 3 ? xp[2] : 0.0, 0.0);
  v[i] = make_double4_32a(vp[0], vp[1], d == 3 ? vp[2] : 0.0, 0.0);
  f[i] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
  m[i] = hm[i];
  pid[i] = hid[2 * i];
  sid[i] = hid[2 * i + 1];
  hidx[i] = i;
  slot_of[i] = i;
}

// host-order state written into the particles' current slots; positions
// taken in the periodic image the device holds (between list rebuilds it
// may keep a particle up to skin/2 past a face, the host copy is wrapped)
__global__ void k_update_state(Consts k, int n, const int* __restrict__ slot_of,
                               const double* __restrict__ hx, const double* __restrict__ hv,
                               const double* __restrict__ hf, double4_32a* __restrict__ x,
                               double4_32a* __restrict__ v, double4_32a* __restrict__ f) {
  const int hi = blockIdx.x * blockDim.x + threadIdx.x;
  if (hi >= n) return;
  const int s = slot_of[hi];
  const int d = k.d;
  if (hx) {
    const double4_32a xd = x[s];
    const double cur[3] = {xd.x, xd.y, xd.z};
    double xs[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < d; ++a) {
      xs[a] = hx[(size_t)hi * d + a];
      if (k.periodic[a]) {
        const double sh = rint((cur[a] - xs[a]) / k.len[a]);
        if (sh != 0.0) xs[a] = xs[a] + sh * k.len[a];
      }
    }
    x[s] = make_double4_32a(xs[0], xs[1], xs[2], 0.0);
  }
  if (hv) {
    const double* p = hv + (size_t)hi * d;
    v[s] = make_double4_32a(p[0], p[1], d == 3 ? p[2] : 0.0, 0.0);
  }
  if (hf) {
    const double* p = hf + (size_t)hi * d;
    f[s] = make_double4_32a(p[0], p[1], d == 3 ? p[2] : 0.0, 0.0);
  }
}

// scatter sorted state back to host order: interleaved (d, N) layout
__global__ void k_download(int n, int d, const int* __restrict__ hidx, const double4_32a* __restrict__ a4,
                           double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int hi = hidx[i];
  const double4_32a v = a4[i];
  double* o = out + (size_t)hi * d;
  o[0] = v.x;
  o[1] = v.y;
  if (d == 3) o[2] = v.z;
}

// positions in host order, wrapped into the periodic box (after list-reuse
// steps the stored positions may lie up to skin/2 outside a periodic face)
__global__ void k_download_pos(Consts k, int n, const int* __restrict__ hidx,
                               const double4_32a* __restrict__ x, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a v = x[i];
  double xs[3] = {v.x, v.y, v.z};
  for (int a = 0; a < k.d; ++a) {
    if (xs[a] < k.min_phys[a] && k.bc_lo[a] == MCFG_BC_PERIODIC) xs[a] = __dadd_rn(xs[a], k.len[a]);
    if (xs[a] >= k.max_phys[a] && k.bc_hi[a] == MCFG_BC_PERIODIC) xs[a] = __dsub_rn(xs[a], k.len[a]);
  }
  double* o = out + (size_t)hidx[i] * k.d;
  for (int a = 0; a < k.d; ++a) o[a] = xs[a];
}

__global__ void k_download_scalar(int n, const int* __restrict__ hidx, const double* __restrict__ a,
                                  double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[hidx[i]] = a[i];
}

// stress: device [d2][n] component-major -> host (d2, N) interleaved
__global__ void k_download_tensor(int n, int d2, const int* __restrict__ hidx,
                                  const double* __restrict__ a, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int hi = hidx[i];
  for (int c = 0; c < d2; ++c) out[(size_t)hi * d2 + c] = a[(size_t)c * n + i];
}

int ensure_capacity(Handle* h, int64_t n64) {
  if (n64 > (int64_t)0x7fffffff / 4) return set_error(h, MCFG_EINVAL, "too many particles");
  const int n = (int)n64;
  const int d = h->p.num_dim;
  int rc;
  if (n > h->cap_n || !h->x) {
    free_all(h);
    const size_t cap = (size_t)(n > 0 ? n : 1);
    int neigh = h->p.reserved[0];
    if (neigh <= 0) {
      // room for the neighbourhood at the uploaded mean number density
      // (pi rc^2 or 4/3 pi rc^3 of it, plus 30% and 16 for compression and
      // disorder), at least 96 in 2D and 256 in 3D: cut-offs of 4-5 lattice
      // spacings, as MCF's own decks use, need more than the default
      double vol = 1.0;
      for (int a = 0; a < d; ++a) vol *= h->p.max_phys_t[a] - h->p.min_phys_t[a];
      const double rc = h->p.cut_off;
      const double reach = (d == 3) ? 4.0 / 3.0 * M_PI * rc * rc * rc : M_PI * rc * rc;
      const double est = vol > 0.0 ? (double)n / vol * reach : 0.0;
      neigh = std::max(d == 3 ? 256 : 96, (int)std::ceil(1.3 * est + 16.0));
      neigh = std::min((neigh + 7) / 8 * 8, 4096);
    }
    h->neigh_cap = neigh;
    const int nbins = h->k.ncell + 1;
    const int ntiles = (nbins + 4095) / 4096 + 1;
    if ((rc = dalloc(h, &h->x, cap)) || (rc = dalloc(h, &h->v, cap)) ||
        (rc = dalloc(h, &h->f, cap)) || (rc = dalloc(h, &h->m, cap)) ||
        (rc = dalloc(h, &h->pid, cap)) || (rc = dalloc(h, &h->sid, cap)) ||
        (rc = dalloc(h, &h->hidx, cap)) || (rc = dalloc(h, &h->rho, cap)) ||
        (rc = dalloc(h, &h->pr, cap)) || (rc = dalloc(h, &h->x2, cap)) ||
        (rc = dalloc(h, &h->v2, cap)) || (rc = dalloc(h, &h->f2, cap)) ||
        (rc = dalloc(h, &h->m2, cap)) || (rc = dalloc(h, &h->pid2, cap)) ||
        (rc = dalloc(h, &h->sid2, cap)) || (rc = dalloc(h, &h->hidx2, cap)) ||
        (rc = dalloc(h, &h->key, cap)) || (rc = dalloc(h, &h->rank, cap)) ||
        (rc = dalloc(h, &h->order, cap)) || (rc = dalloc(h, &h->off, cap)) ||
        (rc = dalloc(h, &h->cell_of, cap)) || (rc = dalloc(h, &h->ncount, cap)) ||
        (rc = dalloc(h, &h->nhs, cap)) || (rc = dalloc(h, &h->slot_of, cap)) ||
        (rc = dalloc(h, &h->nl, cap * (size_t)neigh)) ||
        (rc = dalloc(h, &h->cnt, (size_t)nbins + 1)) ||
        (rc = dalloc(h, &h->cell_start, (size_t)nbins + 2)) ||
        (rc = dalloc(h, &h->scan_part, (size_t)ntiles + 1)) ||
        (rc = dalloc(h, &h->red, (size_t)1024 * 13 + 64)) ||
        (rc = dalloc(h, &h->d_err, 1)) || (rc = dalloc(h, &h->d_stats, 4)) ||
        (rc = dalloc(h, &h->d_pairs, 1)))
      return rc;
    if (h->k.reuse) {
      // candidates within rc + skin: the list grows with the volume ratio
      const double rv = std::sqrt((double)h->k.rv2f) / h->p.cut_off;
      h->vcap = (int)std::ceil(neigh * std::pow(rv, d) * 1.05) + 8;
      if ((rc = dalloc(h, &h->x_ref, cap)) || (rc = dalloc(h, &h->vl, cap * (size_t)h->vcap)) ||
          (rc = dalloc(h, &h->vcount, cap)) || (rc = dalloc(h, &h->d_rebuild, 2)))
        return rc;
      h->partitioned = h->p.precision != MCFG_PRECISION_FP64;
      if (cuda_check(h, cudaMemsetAsync(h->d_rebuild, 0, 2 * sizeof(int), h->stream),
                     "memset rebuild"))
        return MCFG_ECUDA;
    }
    if (h->p.precision == MCFG_PRECISION_FP64) {
      if ((rc = dalloc(h, &h->pc, cap)) || (rc = dalloc(h, &h->rxc, cap))) return rc;
    } else {
      if ((rc = dalloc(h, &h->rxcf, cap))) return rc;
      if ((rc = dalloc(h, &h->pcf, cap)) || (rc = dalloc(h, &h->vf, cap)) ||
          (rc = dalloc(h, &h->wd, cap)))
        return rc;
    }
    if (!h->p.Newtonian) {
      const size_t d2 = (size_t)d * d;
      const size_t elt = (h->p.precision == MCFG_PRECISION_FP64) ? 8 : 4;
      char* q = nullptr;
      if ((rc = dalloc(h, &h->ct, cap * d2)) || (rc = dalloc(h, &h->act, cap * d2)) ||
          (rc = dalloc(h, &h->vgt, cap * d2)) || (rc = dalloc(h, &h->ct2, cap * d2)) ||
          (rc = dalloc(h, &h->act2, cap * d2)) || (rc = dalloc(h, &q, cap * (1 + d2) * elt)))
        return rc;
      h->qq = q;
    }
    if (h->p.stress_tensor) {
      if ((rc = dalloc(h, &h->st, cap * (size_t)(d * d)))) return rc;
    } else if (h->p.precision == MCFG_PRECISION_FP64) {
      // symmetric FP64 force partial sums: (forward slots + owner) x 3 planes
      const size_t planes = (size_t)((d == 3 ? 14 : 5) + 1) * 3;
      double* pj = nullptr;
      if ((rc = dalloc(h, &pj, cap * planes))) return rc;
      h->jp = pj;
    }
    if ((rc = dalloc(h, &h->up_x, cap * 9)) || (rc = dalloc(h, &h->up_v, cap * 3)) ||
        (rc = dalloc(h, &h->up_m, cap)) || (rc = dalloc(h, &h->up_id, cap * 2)))
      return rc;
    h->up_cap = cap;
    h->cap_n = n;
    if (cuda_check(h, cudaMemsetAsync(h->d_err, 0, sizeof(unsigned), h->stream), "memset err"))
      return MCFG_ECUDA;
  }
  return MCFG_OK;
}

int set_device(Handle* h) {
  return cuda_check(h, cudaSetDevice(h->device), "cudaSetDevice") ? MCFG_ECUDA : MCFG_OK;
}

#define GUARD(h)                                                    \
  do {                                                              \
    if (!(h)) return MCFG_EINVAL;                                   \
    int _rc = set_device(h);                                        \
    if (_rc) return _rc;                                            \
  } while (0)

#define TRY(expr)          \
  do {                     \
    int _rc = (expr);      \
    if (_rc) return _rc;   \
  } while (0)

}  // namespace

namespace mcfg {

int rhs(Handle* h, int64_t step, int fuse_mode, double dt) {
  {
    PhaseScope ps(h, kPhaseList);
    TRY(build_cell_list(h));
  }
  h->have_list = true;
  if (h->io_x_out) TRY(download_x_async(h));
  {
    PhaseScope ps(h, kPhaseDensity);
    TRY(compute_density(h, true));
  }
  h->have_density = h->have_pressure = true;
  {
    PhaseScope ps(h, kPhaseForce);
    TRY(compute_force(h, step, fuse_mode, dt));
  }
  h->have_force = true;
  return MCFG_OK;
}

int kdw(Handle* h, double dt) {
  PhaseScope ps(h, kPhaseUpdate);
  return kick_drift_wrap(h, dt);
}

}  // namespace mcfg

namespace {

// opens the rebuild body of a captured step when the kick-drift kernel has
// raised the rebuild flag
__global__ void k_set_rebuild_cond(cudaGraphConditionalHandle c, const int* __restrict__ flag) {
  cudaGraphSetConditional(c, flag[0] != 0 ? 1u : 0u);
}

}  // namespace

namespace mcfg {

// Inside a stream capture: the gated rebuild as the body of a conditional
// node after the kernel that sets its condition.  Any refusal by the
// runtime returns MCFG_ENOTSUP (the caller recaptures without it).
static int rebuild_conditional(Handle* h) {
  if (!h->cond_stream &&
      cudaStreamCreateWithFlags(&h->cond_stream, cudaStreamNonBlocking) != cudaSuccess)
    return MCFG_ENOTSUP;
  cudaStream_t s = h->stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t graph = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive || graph == nullptr)
    return MCFG_ENOTSUP;
  cudaGraphConditionalHandle cond;
  if (cudaGraphConditionalHandleCreate(&cond, graph, 0, cudaGraphCondAssignDefault) !=
      cudaSuccess)
    return MCFG_ENOTSUP;
  k_set_rebuild_cond<<<1, 1, 0, s>>>(cond, h->d_rebuild);
  h->launches++;
  if (cudaGetLastError() != cudaSuccess ||
      cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps) != cudaSuccess)
    return MCFG_ENOTSUP;
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = cond;
  np.conditional.type = cudaGraphCondTypeIf;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &np) != cudaSuccess)
    return MCFG_ENOTSUP;
  cudaGraph_t body = np.conditional.phGraph_out[0];
  // the rebuild kernels, launched on the handle's stream, go into the body
  if (cudaStreamBeginCaptureToGraph(h->cond_stream, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return MCFG_ENOTSUP;
  h->stream = h->cond_stream;
  // the body runs on rebuild steps only: a replay's launch count leaves it out
  const int64_t launches0 = h->launches;
  int rc = wrap_gated(h);
  if (rc == MCFG_OK) rc = gated_cell_list(h);
  if (rc == MCFG_OK) rc = verlet_build_gated(h);
  h->launches = launches0;
  h->stream = s;
  cudaGraph_t ended = nullptr;
  const bool body_ok = cudaStreamEndCapture(h->cond_stream, &ended) == cudaSuccess;
  if (rc != MCFG_OK) return rc;
  if (!body_ok ||
      cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                          cudaStreamSetCaptureDependencies) != cudaSuccess)
    return MCFG_ENOTSUP;
  return MCFG_OK;
}

// the right-hand side in list-reuse mode: the rebuild kernels return at once
// unless a particle has moved more than skin/2 (or no candidate list matches
// the particles yet), then the density over the candidate list and the force
int rhs_reuse(Handle* h, int64_t step, int fuse_mode, double dt) {
  {
    PhaseScope ps(h, kPhaseList);
    if (!h->reuse_valid &&
        cuda_check(h, cudaMemsetAsync(h->d_rebuild, 0xff, sizeof(int), h->stream), "rebuild flag"))
      return MCFG_ECUDA;
    if (h->graph_capturing && !h->cond_off) {
      TRY(rebuild_conditional(h));
    } else {
      TRY(wrap_gated(h));
      TRY(gated_cell_list(h));
      TRY(verlet_build_gated(h));
    }
    h->reuse_valid = true;
  }
  h->have_list = false;  // stage entry points rebuild MCF's list themselves
  if (h->io_x_out) TRY(download_x_async(h));
  {
    PhaseScope ps(h, kPhaseDensity);
    TRY(compute_density(h, true, true));
  }
  h->have_density = h->have_pressure = true;
  {
    PhaseScope ps(h, kPhaseForce);
    TRY(compute_force(h, step, fuse_mode, dt));
  }
  h->have_force = true;
  return MCFG_OK;
}

// one VV step of mcfg_step_vv / mcfg_run_vv
int download_x_async(Handle* h) {
  const int n = (int)h->n, d = h->p.num_dim;
  double* stage = h->up_x;  // x | v | (x in) regions of n*3 doubles
  const int tb = 256, gb = (n + tb - 1) / tb;
  k_download_pos<<<gb, tb, 0, h->stream>>>(h->k, n, h->hidx, h->x, stage);
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "x out kernel") ||
      cuda_check(h, cudaEventRecord(h->ev_x, h->stream), "x out event") ||
      cuda_check(h, cudaStreamWaitEvent(h->copy_stream, h->ev_x, 0), "x out wait") ||
      cuda_check(h, cudaMemcpyAsync(h->io_x_out, stage, sizeof(double) * (size_t)n * d,
                                    cudaMemcpyDeviceToHost, h->copy_stream),
                 "x out"))
    return MCFG_ECUDA;
  return MCFG_OK;
}

// boundary_update_boundary.F90 (shear velocities of oscillating walls at
// time_v, Lees-Edwards shear_length at time_r) into the constants the
// kernels take by value; wall_v_end is the end-of-step update at
// (time_r, time_r) of marching_integrate_VV.F90:1657.  Host libm cos, as
// MCF's.
void boundary_update(Handle* h, double time_r, double time_v) {
  Consts& k = h->k;
  const mcfg_params& p = h->p;
  for (int f = 0; f < 6; ++f) {
    // :78-98, only with walls (num_wall > 0)
    const bool osc = k.walls && h->shear_type[f] == 2;
    for (int a = 0; a < 3; ++a) {
      const double v0 = p.wall_v[f][a];
      const double vh = osc ? v0 * std::cos(h->shear_freq[f] * time_v) : v0;
      const double ve = osc ? v0 * std::cos(h->shear_freq[f] * time_r) : v0;
      k.wall_v[f][a] = vh;
      k.wall_vf[f][a] = (float)vh;
      k.wall_v_end[f][a] = ve;
    }
  }
  if (k.le) {
    // :102-122: images above the y+ face shift by (v0(y+) - v0(y-)) time_r
    // along x
    const double S = (p.wall_v[3][0] - p.wall_v[2][0]) * time_r;
    k.le_S = S;
    // the stencil of the rows across the face follows S mod L_x.  With a
    // candidate list in place the rows keep the rebuild's cells and the
    // images move by dS.  Measured from the shear the faces impose (x
    // velocity dv (y - y0) / L_y, which carries a particle's image across a
    // face with the particle), a pair's separation changes by the two
    // particles' displacements from that flow plus the flow's own change
    // over the pair, at most |dS| (rc + skin) / L_y: the list holds while
    // twice the largest displacement stays below skin minus that (past it
    // the list is dropped)
    const double dS = S - h->le_S_ref;
    const double m = 0.5 * (h->le_skin - std::fabs(dS) * h->le_reach / k.len[1]);
    if (k.reuse && h->reuse_valid && m > 0.0) {
      k.le_dS = dS;
      k.le_aff = dS / k.len[1];
      k.half_skin_le2 = m * m;
    } else {
      le_map(h);
      h->reuse_valid = false;
    }
  }
}

// the cells of the Lees-Edwards crossing rows for the current shift, which
// becomes the reference of the next candidate list
void le_map(Handle* h) {
  Consts& k = h->k;
  const double S = k.le_S;
  const double L = k.len[0];
  double sm = std::fmod(S, L);
  if (sm < 0.0) sm += L;
  const double q = sm * k.rdx[0];
  const double cu = std::ceil(q), cl = std::floor(q);
  k.le_cu = (int)cu % k.nm[0];
  k.le_cl = (int)cl % k.nm[0];
  k.le_pu = cu - q;
  k.le_pl = q - cl;
  k.le_dS = 0.0;
  k.le_aff = 0.0;
  k.half_skin_le2 = k.half_skin2;
  h->le_S_ref = S;
}

int vv_step(Handle* h, int64_t step, double dt) {
  // marching_marching.F90:1393 advances time_current before the step; the
  // step updates the boundaries at (time + dt, time + dt/2),
  // marching_integrate_VV.F90:783-806
  h->time_current = h->time_current + dt;
  if (h->k.walls || h->k.le)
    boundary_update(h, h->time_current + dt, h->time_current + 0.5 * dt);
  // the colloids' rigid-body update (marching_integrate_VV.F90:455-765); it
  // touches only colloid boundary particles, so running it before the
  // fluid's half kick and drift gives MCF's state
  if (h->cdyn) {
    PhaseScope ps(h, kPhaseUpdate);
    TRY(colloid_section(h, step, dt));
  }
  if (!h->k.reuse) {
    TRY(kdw(h, dt));
    return rhs(h, step, kForceBodyKick, dt);
  }
  if (h->reuse_valid) {
    PhaseScope ps(h, kPhaseUpdate);
    h->unwrapped = true;
    TRY(kick_drift_reuse(h, dt));
    if (h->k.le) {
      // a rebuild in this step takes the crossing rows' cells of the
      // current shift: the host reads the device's decision
      int flag = 0;
      if (cuda_check(h, cudaMemcpyAsync(&flag, h->d_rebuild, sizeof(int), cudaMemcpyDeviceToHost,
                                        h->stream),
                     "rebuild flag") ||
          cuda_check(h, cudaStreamSynchronize(h->stream), "rebuild flag sync"))
        return MCFG_ECUDA;
      if (flag != 0) le_map(h);
    }
  } else {
    // no candidate list yet: MCF's kick-drift-wrap; the rebuild follows
    TRY(kdw(h, dt));
  }
  return rhs_reuse(h, step, kForceBodyKick, dt);
}

__global__ void k_step_set(int64_t* __restrict__ d_step, int64_t value) { *d_step = value; }
__global__ void k_step_advance(int64_t* __restrict__ d_step) { *d_step += 1; }

void destroy_graphs(Handle* h) {
  for (auto& g : h->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = Handle::GraphSlot{};
  }
  for (auto& g : h->hgraphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = Handle::HostGraph{};
  }
}

// run_vv may replay captured steps: list reuse (the rebuild is decided on the
// device), a candidate list in place, no profiling, and constants that do
// not change from step to step (no oscillating walls; Lees-Edwards runs
// without list reuse anyway)
static bool graph_eligible(const Handle* h) {
  if (!h->k.reuse || !h->reuse_valid || h->profiling || h->graph_off || h->k.le) return false;
  if (h->k.walls)
    for (int f = 0; f < 6; ++f)
      if (h->shear_type[f] == 2) return false;
  return true;
}

// the graph of two list-reuse VV steps for the handle's current state
// (captured on first use and whenever constants, buffers or dt change)
static Handle::GraphSlot* graph_for(Handle* h, double dt) {
  for (auto& g : h->graphs)
    if (g.exec && g.gen == h->graph_gen && g.dt == dt && g.v == (const void*)h->v) return &g;
  if (!h->d_step && cudaMalloc(&h->d_step, sizeof(int64_t)) != cudaSuccess) {
    cudaGetLastError();
    h->graph_off = true;
    return nullptr;
  }
  Handle::GraphSlot* slot = &h->graphs[0];
  for (auto& g : h->graphs)
    if (!g.exec || g.gen != h->graph_gen || g.dt != dt) {
      slot = &g;
      break;
    }
  if (slot->exec) cudaGraphExecDestroy(slot->exec);
  *slot = Handle::GraphSlot{};
  double4_32a* const v0 = h->v;
  double4_32a* const v20 = h->v2;
  const int64_t launches0 = h->launches;
  const double t0 = h->time_current;
  bool ok = false;
  int64_t captured = 0;
  // with the rebuild in a conditional node first; if the runtime refuses
  // that, once more with the gated kernels in the graph itself
  for (int attempt = 0; attempt < 2 && !ok; ++attempt) {
    if (attempt == 1) {
      if (h->cond_off) break;
      h->cond_off = true;
    }
    cudaGraph_t graph = nullptr;
    ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      h->graph_capturing = true;
      for (int q = 0; q < 2 && ok; ++q) {
        ok = (!h->cdyn || colloid_section(h, 0, dt) == MCFG_OK) &&
             kick_drift_reuse(h, dt) == MCFG_OK &&
             rhs_reuse(h, 0, kForceBodyKick, dt) == MCFG_OK;
        k_step_advance<<<1, 1, 0, h->stream>>>(h->d_step);
      }
      h->graph_capturing = false;
      const bool ended = cudaStreamEndCapture(h->stream, &graph) == cudaSuccess;
      ok = ok && ended && graph != nullptr &&
           cudaGraphInstantiate(&slot->exec, graph, 0) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
    }
    h->time_current = t0;  // the capture ran no step
    captured = h->launches - launches0;
    h->launches = launches0;
    if (!ok || h->v != v0) {
      // nothing ran: the buffers the captured kicks swapped go back
      ok = false;
      cudaGetLastError();
      if (slot->exec) cudaGraphExecDestroy(slot->exec);
      *slot = Handle::GraphSlot{};
      h->v = v0;
      h->v2 = v20;
      h->err.clear();
    }
  }
  if (!ok) {
    // plain launches for this handle from now on
    h->graph_off = true;
    return nullptr;
  }
  slot->gen = h->graph_gen;
  slot->dt = dt;
  slot->v = v0;
  slot->launches = captured + 2;
  return slot;
}

// page-locked host memory (pinned, or registered with mcfg_host_register):
// what a captured memcpy node may read and write
static bool page_locked(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// the staging regions of mcfg_step_vv_host in up_x: x out | v out | x in
static double* stage_x_in(Handle* h) { return h->up_x + (size_t)h->n * 6; }
static double* stage_v_out(Handle* h) { return h->up_x + (size_t)h->n * 3; }

// one host step's device work after its inputs are enqueued: the state
// update, the step (positions back on the copy stream from its list phase),
// the velocities back
static int host_step_body(Handle* h, int64_t step, double dt, double* x, double* v) {
  const int n = (int)h->n, d = h->p.num_dim;
  const size_t bytes = sizeof(double) * (size_t)n * d;
  const int tb = 256, gb = (n + tb - 1) / tb;
  cudaStream_t s = h->stream;
  k_update_state<<<gb, tb, 0, s>>>(h->k, n, h->slot_of, stage_x_in(h), h->up_v, nullptr, h->x,
                                   h->v, h->f);
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "update state kernel")) return MCFG_ECUDA;
  h->have_list = h->have_density = h->have_pressure = false;
  h->dt = dt;
  h->io_x_out = x;
  const int rc = vv_step(h, step, dt);
  h->io_x_out = nullptr;
  if (rc != MCFG_OK) return rc;
  k_download<<<gb, tb, 0, s>>>(n, d, h->hidx, h->v, stage_v_out(h));
  h->launches++;
  if (cuda_check(h, cudaMemcpyAsync(v, stage_v_out(h), bytes, cudaMemcpyDeviceToHost, s),
                 "v out"))
    return MCFG_ECUDA;
  return MCFG_OK;
}

// the captured host step for these arrays and the current velocity buffer,
// or null (not eligible, or the capture failed: plain launches then)
static Handle::HostGraph* host_graph_for(Handle* h, double dt, double* x, double* v) {
  if (!graph_eligible(h) || h->hgraph_off || !page_locked(x) || !page_locked(v)) return nullptr;
  for (auto& g : h->hgraphs)
    if (g.exec && g.gen == h->graph_gen && g.dt == dt && g.v == (const void*)h->v && g.hx == x &&
        g.hv == v)
      return &g;
  if (!h->d_step && cudaMalloc(&h->d_step, sizeof(int64_t)) != cudaSuccess) {
    cudaGetLastError();
    h->hgraph_off = true;
    return nullptr;
  }
  // a slot that no longer matches, else the one of the other velocity buffer
  Handle::HostGraph* slot = nullptr;
  for (auto& g : h->hgraphs)
    if (!g.exec || g.gen != h->graph_gen || g.dt != dt || g.hx != x || g.hv != v) {
      slot = &g;
      break;
    }
  if (!slot) slot = (h->hgraphs[0].v != (const void*)h->v) ? &h->hgraphs[0] : &h->hgraphs[1];
  if (slot->exec) cudaGraphExecDestroy(slot->exec);
  *slot = Handle::HostGraph{};
  // the capture runs no step: the host-side state it changes is put back
  double4_32a* const v0 = h->v;
  double4_32a* const v20 = h->v2;
  const int64_t launches0 = h->launches;
  const double t0 = h->time_current;
  const bool unwrapped0 = h->unwrapped, hl = h->have_list, hd = h->have_density,
             hp = h->have_pressure, hf = h->have_force;
  const double dt0 = h->dt;
  const size_t bytes = sizeof(double) * (size_t)h->n * h->p.num_dim;
  cudaStream_t s = h->stream;
  bool ok = false;
  for (int attempt = 0; attempt < 2 && !ok; ++attempt) {
    if (attempt == 1) {
      // once more with the gated rebuild kernels in the graph itself
      if (h->cond_off) break;
      h->cond_off = true;
      cudaGetLastError();
      if (slot->exec) cudaGraphExecDestroy(slot->exec);
      slot->exec = nullptr;
      h->launches = launches0;
      h->v = v0;
      h->v2 = v20;
    }
    cudaGraph_t graph = nullptr;
    ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      h->graph_capturing = true;
      ok = cudaMemcpyAsync(stage_x_in(h), x, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess &&
           cudaMemcpyAsync(h->up_v, v, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess &&
           host_step_body(h, 0, dt, x, v) == MCFG_OK;
      // the copy stream's positions joined back into the captured stream
      const bool joined = cudaEventRecord(h->ev_join, h->copy_stream) == cudaSuccess &&
                          cudaStreamWaitEvent(s, h->ev_join, 0) == cudaSuccess;
      h->graph_capturing = false;
      const bool ended = cudaStreamEndCapture(s, &graph) == cudaSuccess;
      ok = ok && joined && ended && graph != nullptr &&
           cudaGraphInstantiate(&slot->exec, graph, 0) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
    }
  }
  const int64_t captured = h->launches - launches0;
  h->launches = launches0;
  h->v = v0;
  h->v2 = v20;
  h->time_current = t0;
  h->unwrapped = unwrapped0;
  h->have_list = hl;
  h->have_density = hd;
  h->have_pressure = hp;
  h->have_force = hf;
  h->dt = dt0;
  if (!ok) {
    cudaGetLastError();
    if (slot->exec) cudaGraphExecDestroy(slot->exec);
    *slot = Handle::HostGraph{};
    h->hgraph_off = true;
    h->err.clear();
    return nullptr;
  }
  slot->gen = h->graph_gen;
  slot->dt = dt;
  slot->v = v0;
  slot->hx = x;
  slot->hv = v;
  slot->launches = captured;
  return slot;
}

}  // namespace mcfg

namespace {

// one value per particle from host order into the sorted slots
__global__ void k_scalar_from_host(int n, const double* __restrict__ src,
                                   const int* __restrict__ hidx, double* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[hidx[i]];
}

__global__ void k_upload_force(int n, int d, const double* __restrict__ hf,
                               const int* __restrict__ hidx, double4_32a* __restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* fp = hf + (size_t)hidx[i] * d;
  f[i] = make_double4_32a(fp[0], fp[1], d == 3 ? fp[2] : 0.0, 0.0);
}

}  // namespace

extern "C" {

int64_t mcfg_sizeof_params(void) { return (int64_t)sizeof(mcfg_params); }

const char* mcfg_create_error(void) {
  std::lock_guard<std::mutex> lk(g_create_mu);
  return g_create_err.c_str();
}

int mcfg_create(const mcfg_params* params, mcfg_handle** out) {
  if (!out) return MCFG_EINVAL;
  *out = nullptr;
  const char* msg = validate_params(params);
  if (msg) {
    std::lock_guard<std::mutex> lk(g_create_mu);
    g_create_err = msg;
    return MCFG_EINVAL;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= params->device || params->device < 0) {
    std::lock_guard<std::mutex> lk(g_create_mu);
    g_create_err = std::string("no usable CUDA device: ") +
                   (e != cudaSuccess ? cudaGetErrorString(e) : "ordinal out of range");
    return MCFG_ENODEV;
  }
  mcfg_handle* h = new mcfg_handle();
  h->p = *params;
  h->device = params->device;
  h->dt = params->dt;
  fill_consts(h);
  for (int a = 0; a < h->k.d; ++a) {
    if ((h->k.periodic[a] || (h->k.le && a == 1)) && h->k.nm[a] < 3) {
      std::lock_guard<std::mutex> lk(g_create_mu);
      g_create_err = "a periodic axis needs at least 3 cells (box >= 3*1.0001*cut_off)";
      delete h;
      return MCFG_EINVAL;
    }
  }
  if (h->k.le && h->k.nm[0] < 4) {
    // the row across a Lees-Edwards face spans four x cells
    std::lock_guard<std::mutex> lk(g_create_mu);
    g_create_err = "Lees-Edwards needs at least 4 cells along x (box >= 4*1.0001*cut_off)";
    delete h;
    return MCFG_EINVAL;
  }
  boundary_update(h, h->time_current, h->time_current);
  if (cudaSetDevice(h->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_create_mu);
    g_create_err = "cannot create a CUDA stream";
    delete h;
    return MCFG_ECUDA;
  }
  *out = h;
  return MCFG_OK;
}

int mcfg_destroy(mcfg_handle* h) {
  if (!h) return MCFG_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  resolve_phases(h);
  for (auto& ev : h->ev_pool) {
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  h->ev_pool.clear();
  free_all(h);
  if (h->copy_stream) {
    cudaStreamSynchronize(h->copy_stream);
    cudaStreamDestroy(h->copy_stream);
  }
  if (h->ev_x) cudaEventDestroy(h->ev_x);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->cond_stream) cudaStreamDestroy(h->cond_stream);
  if (h->h_status) cudaFreeHost(h->h_status);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return MCFG_OK;
}

const char* mcfg_last_error(const mcfg_handle* h) {
  if (!h) return "null handle";
  return h->err.empty() ? "no error" : h->err.c_str();
}

int mcfg_get_info(const mcfg_handle* h, mcfg_info* info) {
  if (!h || !info) return MCFG_EINVAL;
  memset(info, 0, sizeof *info);
  info->num_part = h->n;
  for (int a = 0; a < 3; ++a) info->num_cell_dim[a] = h->k.nm[a];
  info->num_cell = h->k.ncell;
  info->num_outside = h->num_outside;
  info->num_pairs = h->num_pairs;
  info->max_neigh = h->max_neigh;
  info->neigh_capacity = h->neigh_cap;
  info->kernel_launches = h->launches;
  info->device_bytes = h->device_bytes;
  if (h->k.reuse) {
    info->skin = 2.0 * std::sqrt(h->k.half_skin2);
    int cntr[2] = {0, 0};
    if (h->d_rebuild && cudaSetDevice(h->device) == cudaSuccess &&
        cudaMemcpyAsync(cntr, h->d_rebuild, sizeof cntr, cudaMemcpyDeviceToHost, h->stream) ==
            cudaSuccess &&
        cudaStreamSynchronize(h->stream) == cudaSuccess)
      info->list_rebuilds = cntr[1];
  }
  info->time_current = h->time_current;
  info->shear_length = h->k.le ? h->k.le_S : 0.0;
  return MCFG_OK;
}

int mcfg_upload(mcfg_handle* h, int64_t n, const double* x, const double* v, const double* m,
                const int32_t* id, const double* ct) {
  GUARD(h);
  h->graph_gen++;
  if (n < 0 || (n > 0 && (!x || !v || !m || !id)))
    return set_error(h, MCFG_EINVAL, "mcfg_upload: NULL array");
  if (ct && h->p.Newtonian) return set_error(h, MCFG_EINVAL, "conformation tensor of a Newtonian run");
  TRY(ensure_capacity(h, n));
  const int d = h->p.num_dim;
  h->n = n;
  h->k.n = (int)n;
  if (n > 0) {
    cudaStream_t s = h->stream;
    if (cuda_check(h, cudaMemcpyAsync(h->up_x, x, sizeof(double) * (size_t)(n * d),
                                      cudaMemcpyHostToDevice, s), "upload x") ||
        cuda_check(h, cudaMemcpyAsync(h->up_v, v, sizeof(double) * (size_t)(n * d),
                                      cudaMemcpyHostToDevice, s), "upload v") ||
        cuda_check(h, cudaMemcpyAsync(h->up_m, m, sizeof(double) * (size_t)n,
                                      cudaMemcpyHostToDevice, s), "upload m") ||
        cuda_check(h, cudaMemcpyAsync(h->up_id, id, sizeof(int32_t) * (size_t)(2 * n),
                                      cudaMemcpyHostToDevice, s), "upload id"))
      return MCFG_ECUDA;
    const int tb = 256, gb = (int)((n + tb - 1) / tb);
    k_upload<<<gb, tb, 0, s>>>((int)n, d, h->up_x, h->up_v, h->up_m, h->up_id, h->x, h->v, h->f,
                               h->m, h->pid, h->sid, h->hidx, h->slot_of);
    h->launches++;
    if (!h->p.Newtonian) {
      double* hct = nullptr;
      if (ct) {
        // staged through up_x (n*9 doubles)
        if (cuda_check(h, cudaStreamSynchronize(s), "upload sync") ||
            cuda_check(h, cudaMemcpyAsync(h->up_x, ct, sizeof(double) * (size_t)(n * d * d),
                                          cudaMemcpyHostToDevice, s), "upload ct"))
          return MCFG_ECUDA;
        hct = h->up_x;
      }
      k_upload_ct<<<gb, tb, 0, s>>>((int)n, d, hct, h->ct, h->act);
      h->launches++;
    }
    if (cuda_check(h, cudaGetLastError(), "upload kernel")) return MCFG_ECUDA;
    if (h->p.stress_tensor)
      if (cuda_check(h, cudaMemsetAsync(h->st, 0, sizeof(double) * (size_t)(n * d * d), s),
                     "memset stress"))
        return MCFG_ECUDA;
    if (cuda_check(h, cudaMemsetAsync(h->rho, 0, sizeof(double) * (size_t)n, s), "memset rho") ||
        cuda_check(h, cudaMemsetAsync(h->pr, 0, sizeof(double) * (size_t)n, s), "memset p"))
      return MCFG_ECUDA;
  }
  // pageable host buffers: the copies above are complete only after a sync
  if (cuda_check(h, cudaStreamSynchronize(h->stream), "upload sync")) return MCFG_ECUDA;
  // boundary particles of each colloid (host indices), for the drag sums
  {
    int maxc = 0;
    int64_t nb = 0;
    for (int64_t i = 0; i < n; ++i) {
      maxc = std::max(maxc, (int)id[2 * i + 1]);
      nb += (id[2 * i + 1] != 0) ? 1 : 0;
    }
    h->n_boundary = nb;
    h->h_coll_start.assign((size_t)maxc + 1, 0);
    h->h_coll_mem.clear();
    if (maxc > 0) {
      for (int64_t i = 0; i < n; ++i)
        if (id[2 * i + 1] > 0) h->h_coll_start[(size_t)id[2 * i + 1]]++;
      for (int c = 0; c < maxc; ++c) h->h_coll_start[(size_t)c + 1] += h->h_coll_start[(size_t)c];
      h->h_coll_mem.assign((size_t)h->h_coll_start[(size_t)maxc], 0);
      std::vector<int> pos(h->h_coll_start.begin(), h->h_coll_start.end() - 1);
      for (int64_t i = 0; i < n; ++i)
        if (id[2 * i + 1] > 0) h->h_coll_mem[(size_t)pos[(size_t)id[2 * i + 1] - 1]++] = (int)i;
      int rc2;
      if ((rc2 = dalloc(h, &h->coll_start, (size_t)maxc + 1)) ||
          (rc2 = dalloc(h, &h->coll_mem, h->h_coll_mem.size())))
        return rc2;
      if (cuda_check(h, cudaMemcpy(h->coll_start, h->h_coll_start.data(),
                                   sizeof(int) * h->h_coll_start.size(), cudaMemcpyHostToDevice),
                     "upload colloid lists") ||
          cuda_check(h, cudaMemcpy(h->coll_mem, h->h_coll_mem.data(),
                                   sizeof(int) * h->h_coll_mem.size(), cudaMemcpyHostToDevice),
                     "upload colloid lists"))
        return MCFG_ECUDA;
    }
    h->coll_nmem = (int)h->h_coll_mem.size();
  }
  h->have_particles = true;
  h->reuse_valid = false;
  h->unwrapped = false;
  h->have_list = h->have_density = h->have_pressure = h->have_force = false;
  return MCFG_OK;
}

int mcfg_upload_force(mcfg_handle* h, const double* f) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  if (!f) return set_error(h, MCFG_EINVAL, "mcfg_upload_force: NULL array");
  const int n = (int)h->n, d = h->p.num_dim;
  if (n == 0) return MCFG_OK;
  cudaStream_t s = h->stream;
  if (cuda_check(h, cudaMemcpyAsync(h->up_x, f, sizeof(double) * (size_t)n * d,
                                    cudaMemcpyHostToDevice, s), "upload f"))
    return MCFG_ECUDA;
  const int tb = 256, gb = (n + tb - 1) / tb;
  k_upload_force<<<gb, tb, 0, s>>>(n, d, h->up_x, h->hidx, h->f);
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "upload force kernel") ||
      cuda_check(h, cudaStreamSynchronize(s), "upload force sync"))
    return MCFG_ECUDA;
  h->have_force = true;
  return MCFG_OK;
}

int mcfg_update_state(mcfg_handle* h, const double* x, const double* v, const double* f) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  const int n = (int)h->n, d = h->p.num_dim;
  if (n == 0) return MCFG_OK;
  cudaStream_t s = h->stream;
  const size_t bytes = sizeof(double) * (size_t)n * d;
  double* dx = x ? h->up_x : nullptr;
  double* df = f ? h->up_x + (size_t)n * 3 : nullptr;
  double* dv = v ? h->up_v : nullptr;
  if ((x && cuda_check(h, cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, s), "update x")) ||
      (v && cuda_check(h, cudaMemcpyAsync(dv, v, bytes, cudaMemcpyHostToDevice, s), "update v")) ||
      (f && cuda_check(h, cudaMemcpyAsync(df, f, bytes, cudaMemcpyHostToDevice, s), "update f")))
    return MCFG_ECUDA;
  const int tb = 256, gb = (n + tb - 1) / tb;
  k_update_state<<<gb, tb, 0, s>>>(h->k, n, h->slot_of, dx, dv, df, h->x, h->v, h->f);
  h->launches++;
  if (cuda_check(h, cudaGetLastError(), "update state kernel") ||
      cuda_check(h, cudaStreamSynchronize(s), "update state sync"))
    return MCFG_ECUDA;
  if (f) h->have_force = true;
  // derived per-step data (densities, lists of the stage entry points) are stale
  h->have_list = h->have_density = h->have_pressure = false;
  return MCFG_OK;
}

int mcfg_adjust_particles(mcfg_handle* h) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  TRY(adjust_particles(h));
  h->have_list = h->have_density = h->have_pressure = false;
  return MCFG_OK;
}

int mcfg_build_list(mcfg_handle* h, int32_t* num_cell_dim, int32_t* cell_start, int32_t* lpdx) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  TRY(build_cell_list(h));
  h->have_list = true;
  h->have_density = h->have_pressure = false;
  if (num_cell_dim)
    for (int a = 0; a < 3; ++a) num_cell_dim[a] = h->k.nm[a];
  cudaStream_t s = h->stream;
  int outside_start = 0;
  if (cuda_check(h, cudaMemcpyAsync(&outside_start, h->cell_start + h->k.ncell, sizeof(int),
                                    cudaMemcpyDeviceToHost, s), "copy cell_start"))
    return MCFG_ECUDA;
  if (cell_start &&
      cuda_check(h, cudaMemcpyAsync(cell_start, h->cell_start, sizeof(int) * (size_t)(h->k.ncell + 1),
                                    cudaMemcpyDeviceToHost, s), "copy cell_start"))
    return MCFG_ECUDA;
  if (lpdx && h->n > 0 &&
      cuda_check(h, cudaMemcpyAsync(lpdx, h->hidx, sizeof(int) * (size_t)h->n,
                                    cudaMemcpyDeviceToHost, s), "copy lpdx"))
    return MCFG_ECUDA;
  if (cuda_check(h, cudaStreamSynchronize(s), "build_list sync")) return MCFG_ECUDA;
  h->num_outside = h->n - outside_start;
  return check_device_errors(h);
}

int mcfg_compute_density(mcfg_handle* h) {
  GUARD(h);
  if (!h->have_list) return set_error(h, MCFG_ESTATE, "mcfg_build_list must come first");
  TRY(compute_density(h, false));
  TRY(check_device_errors(h));
  h->have_density = true;
  h->have_pressure = false;
  return MCFG_OK;
}

int mcfg_update_density(mcfg_handle* h, const double* rho) {
  GUARD(h);
  if (!rho) return set_error(h, MCFG_EINVAL, "mcfg_update_density: NULL rho");
  if (!h->have_density) return set_error(h, MCFG_ESTATE, "mcfg_compute_density must come first");
  const int n = (int)h->n;
  if (n > 0) {
    if (cuda_check(h, cudaMemcpyAsync(h->up_m, rho, sizeof(double) * (size_t)n,
                                      cudaMemcpyHostToDevice, h->stream), "density copy"))
      return MCFG_ECUDA;
    const int tb = 256, gb = (n + tb - 1) / tb;
    k_scalar_from_host<<<gb, tb, 0, h->stream>>>(n, h->up_m, h->hidx, h->rho);
    h->launches++;
    if (cuda_check(h, cudaGetLastError(), "density update launch")) return MCFG_ECUDA;
  }
  h->have_pressure = false;
  return MCFG_OK;
}

int mcfg_compute_pressure(mcfg_handle* h) {
  GUARD(h);
  if (!h->have_density) return set_error(h, MCFG_ESTATE, "mcfg_compute_density must come first");
  TRY(compute_pressure(h));
  h->have_pressure = true;
  return MCFG_OK;
}

int mcfg_compute_interaction(mcfg_handle* h, int64_t step) {
  GUARD(h);
  if (!h->have_pressure) return set_error(h, MCFG_ESTATE, "mcfg_compute_pressure must come first");
  TRY(compute_force(h, step, kForceOnly, h->dt));
  TRY(check_device_errors(h));
  h->have_force = true;
  return MCFG_OK;
}

int mcfg_apply_body_force(mcfg_handle* h) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  return apply_body_force(h);
}

int mcfg_integrate_velocity(mcfg_handle* h, double dt, double lambda) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  return integrate_velocity(h, dt, lambda);
}

int mcfg_integrate_position(mcfg_handle* h, double dt) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  TRY(integrate_position(h, dt));
  h->have_list = h->have_density = h->have_pressure = false;
  return MCFG_OK;
}

int mcfg_init_force(mcfg_handle* h, int64_t step) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  // marching_marching.F90:437: boundaries at time_current
  boundary_update(h, h->time_current, h->time_current);
  TRY(adjust_particles(h));
  TRY(rhs(h, step, kForceBody, h->dt));
  if (h->cdyn) TRY(colloid_initial(h));  // marching_marching.F90:995-1110
  return check_device_errors(h);
}

int mcfg_write_particles(mcfg_handle* h, const char* path, int32_t kind, int32_t flags) {
  GUARD(h);
  if (!path) return set_error(h, MCFG_EINVAL, "NULL path");
  if (kind != 0 && kind != 1) return set_error(h, MCFG_EINVAL, "kind must be 0 (output) or 1 (restart)");
  if (kind == 1 && (flags & 1)) return set_error(h, MCFG_EINVAL, "the restart file has no stress");
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  return write_particle_file(h, path, kind, flags);
}

int mcfg_host_register(mcfg_handle* h, void* ptr, int64_t bytes) {
  GUARD(h);
  if (!ptr || bytes <= 0) return set_error(h, MCFG_EINVAL, "host_register: NULL pointer or size");
  if (cuda_check(h, cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterPortable),
                 "cudaHostRegister"))
    return MCFG_ECUDA;
  return MCFG_OK;
}

int mcfg_host_unregister(mcfg_handle* h, void* ptr) {
  GUARD(h);
  if (!ptr) return set_error(h, MCFG_EINVAL, "host_unregister: NULL pointer");
  if (cuda_check(h, cudaHostUnregister(ptr), "cudaHostUnregister")) return MCFG_ECUDA;
  return MCFG_OK;
}

int mcfg_write_statistic(mcfg_handle* h, const char* path, int64_t step, double time) {
  GUARD(h);
  if (!path) return set_error(h, MCFG_EINVAL, "NULL path");
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  return write_statistic_line(h, path, step, time);
}

int mcfg_set_boundary_motion(mcfg_handle* h, const int32_t* shear_type, const double* shear_freq,
                             double time) {
  GUARD(h);
  h->graph_gen++;
  if (!shear_type || !shear_freq) return set_error(h, MCFG_EINVAL, "NULL shear_type / shear_freq");
  for (int f = 0; f < 6; ++f) {
    if (shear_type[f] == 2 && h->p.bcdef[f] != MCFG_BC_WALL_SOLID)
      return set_error(h, MCFG_EINVAL, "shear_type 2 (oscillating) needs a solid-wall face");
    h->shear_type[f] = shear_type[f];
    h->shear_freq[f] = shear_freq[f];
  }
  h->time_current = time;
  boundary_update(h, time, time);
  return MCFG_OK;
}

int mcfg_step_vv(mcfg_handle* h, int64_t step, double dt) {
  GUARD(h);
  if (!h->have_force) return set_error(h, MCFG_ESTATE, "mcfg_init_force must come first");
  if (!(dt > 0.0)) return set_error(h, MCFG_EINVAL, "dt must be positive");
  h->dt = dt;
  TRY(vv_step(h, step, dt));
  return check_device_errors(h);
}

int mcfg_step_vv_host(mcfg_handle* h, int64_t step, double dt, double* x, double* v) {
  GUARD(h);
  if (!h->have_force) return set_error(h, MCFG_ESTATE, "mcfg_init_force must come first");
  if (!(dt > 0.0)) return set_error(h, MCFG_EINVAL, "dt must be positive");
  if (!x || !v) return set_error(h, MCFG_EINVAL, "NULL x or v");
  const int n = (int)h->n, d = h->p.num_dim;
  if (n == 0) return mcfg_step_vv(h, step, dt);
  if (!h->copy_stream &&
      (cuda_check(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking),
                  "copy stream") ||
       cuda_check(h, cudaEventCreateWithFlags(&h->ev_x, cudaEventDisableTiming), "copy event") ||
       cuda_check(h, cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming),
                  "join event")))
    return MCFG_ECUDA;
  cudaStream_t s = h->stream;
  const size_t bytes = sizeof(double) * (size_t)n * d;
  Handle::HostGraph* g = host_graph_for(h, dt, x, v);
  if (g) {
    // the captured step (list reuse, arrays page-locked): the Philox step
    // from the device counter; the host-side state the step changes
    k_step_set<<<1, 1, 0, s>>>(h->d_step, step);
    if (cuda_check(h, cudaGraphLaunch(g->exec, s), "host step graph")) return MCFG_ECUDA;
    h->launches += g->launches + 1;
    h->time_current = h->time_current + dt;
    std::swap(h->v, h->v2);
    h->unwrapped = true;
    h->dt = dt;
    h->have_list = false;
    h->have_density = h->have_pressure = h->have_force = true;
    if (h->cdyn) h->coll_host_stale = true;  // the replayed step moved the colloids
  } else {
    // the step's inputs: x, v into their particles' current slots
    if (cuda_check(h, cudaMemcpyAsync(stage_x_in(h), x, bytes, cudaMemcpyHostToDevice, s),
                   "x in") ||
        cuda_check(h, cudaMemcpyAsync(h->up_v, v, bytes, cudaMemcpyHostToDevice, s), "v in"))
      return MCFG_ECUDA;
    const int rc = host_step_body(h, step, dt, x, v);
    if (rc != MCFG_OK) {
      cudaStreamSynchronize(h->copy_stream);
      return rc;
    }
  }
  // the status words behind the velocities, then one synchronisation
  if (status_copy_async(h) != MCFG_OK ||
      cuda_check(h, cudaStreamSynchronize(s), "step sync") ||
      cuda_check(h, cudaStreamSynchronize(h->copy_stream), "x out sync"))
    return MCFG_ECUDA;
  return status_evaluate(h);
}

int mcfg_run_vv(mcfg_handle* h, int64_t step0, int32_t nsteps, double dt) {
  GUARD(h);
  if (!h->have_force) return set_error(h, MCFG_ESTATE, "mcfg_init_force must come first");
  if (!(dt > 0.0)) return set_error(h, MCFG_EINVAL, "dt must be positive");
  h->dt = dt;
  int32_t q = 1;
  while (q <= nsteps) {
    Handle::GraphSlot* g = (nsteps - q >= 1 && graph_eligible(h)) ? graph_for(h, dt) : nullptr;
    if (!g) {
      TRY(vv_step(h, step0 + q, dt));
      ++q;
      continue;
    }
    // pairs of steps from the graph: the device counter carries the step
    k_step_set<<<1, 1, 0, h->stream>>>(h->d_step, step0 + q);
    h->launches++;
    h->unwrapped = true;
    for (; nsteps - q >= 1; q += 2) {
      if (cuda_check(h, cudaGraphLaunch(g->exec, h->stream), "graph launch")) return MCFG_ECUDA;
      h->launches += g->launches;
      h->time_current = h->time_current + dt;
      h->time_current = h->time_current + dt;
    }
    // the replayed steps moved the colloids on the device
    if (h->cdyn) h->coll_host_stale = true;
  }
  return check_device_errors(h);
}

int mcfg_download(mcfg_handle* h, double* x, double* v, double* rho, double* p, double* f,
                  double* ct, double* s) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  if (ct && h->p.Newtonian) return set_error(h, MCFG_EINVAL, "no conformation tensor (Newtonian)");
  if (s && !h->p.stress_tensor) return set_error(h, MCFG_EINVAL, "stress_tensor is off");
  const int n = (int)h->n, d = h->p.num_dim;
  if (n == 0) return MCFG_OK;
  cudaStream_t st = h->stream;
  const int tb = 256, gb = (n + tb - 1) / tb;
  // x, v, f, rho and p gathered into separate staging regions and copied
  // asynchronously, one synchronisation for all of them
  double* stage = h->up_x;  // n*9 doubles: x | v | f
  const size_t nd = (size_t)n * d;
  auto vec_out = [&](const double4_32a* a4, double* dst, double* host) -> int {
    k_download<<<gb, tb, 0, st>>>(n, d, h->hidx, a4, dst);
    h->launches++;
    return cuda_check(h, cudaMemcpyAsync(host, dst, sizeof(double) * nd, cudaMemcpyDeviceToHost,
                                         st), "download")
               ? MCFG_ECUDA
               : MCFG_OK;
  };
  auto sca_out = [&](const double* a, double* dst, double* host) -> int {
    k_download_scalar<<<gb, tb, 0, st>>>(n, h->hidx, a, dst);
    h->launches++;
    return cuda_check(h, cudaMemcpyAsync(host, dst, sizeof(double) * (size_t)n,
                                         cudaMemcpyDeviceToHost, st), "download")
               ? MCFG_ECUDA
               : MCFG_OK;
  };
  if (x) {
    k_download_pos<<<gb, tb, 0, st>>>(h->k, n, h->hidx, h->x, stage);
    h->launches++;
    if (cuda_check(h, cudaMemcpyAsync(x, stage, sizeof(double) * nd, cudaMemcpyDeviceToHost, st),
                   "download"))
      return MCFG_ECUDA;
  }
  if (v) TRY(vec_out(h->v, stage + (size_t)3 * n, v));
  if (f) TRY(vec_out(h->f, stage + (size_t)6 * n, f));
  if (rho) TRY(sca_out(h->rho, h->up_v, rho));
  if (p) TRY(sca_out(h->pr, h->up_v + n, p));
  if (cuda_check(h, cudaStreamSynchronize(st), "download sync")) return MCFG_ECUDA;
  if (ct) {
    k_download_tensor<<<gb, tb, 0, st>>>(n, d * d, h->hidx, h->ct, stage);
    h->launches++;
    if (cuda_check(h, cudaMemcpyAsync(ct, stage, sizeof(double) * (size_t)n * d * d,
                                      cudaMemcpyDeviceToHost, st), "download ct") ||
        cuda_check(h, cudaStreamSynchronize(st), "download sync"))
      return MCFG_ECUDA;
  }
  if (s) {
    k_download_tensor<<<gb, tb, 0, st>>>(n, d * d, h->hidx, h->st, stage);
    h->launches++;
    if (cuda_check(h, cudaMemcpyAsync(s, stage, sizeof(double) * (size_t)n * d * d,
                                      cudaMemcpyDeviceToHost, st), "download s") ||
        cuda_check(h, cudaStreamSynchronize(st), "download sync"))
      return MCFG_ECUDA;
  }
  return MCFG_OK;
}

// host copies and the device table [nc][12] (X V Omega R) of the colloids
static int put_colloid_state(Handle* h, int nc, const double* x, const double* v,
                             const double* omega) {
  const int d = h->p.num_dim;
  h->cx.assign(x, x + (size_t)nc * d);
  h->cv.assign(v, v + (size_t)nc * d);
  h->com.assign(omega, omega + (size_t)nc * 3);
  std::vector<double> buf((size_t)nc * 12, 0.0);
  for (int c = 0; c < nc; ++c) {
    for (int a = 0; a < d; ++a) {
      buf[(size_t)c * 12 + a] = x[(size_t)c * d + a];
      buf[(size_t)c * 12 + 3 + a] = v[(size_t)c * d + a];
    }
    for (int a = 0; a < 3; ++a) buf[(size_t)c * 12 + 6 + a] = omega[(size_t)c * 3 + a];
    buf[(size_t)c * 12 + 9] = h->crad[(size_t)c];
  }
  if (nc > 0 &&
      (cuda_check(h, cudaMemcpyAsync(h->coll, buf.data(), sizeof(double) * buf.size(),
                                     cudaMemcpyHostToDevice, h->stream), "upload colloids") ||
       cuda_check(h, cudaStreamSynchronize(h->stream), "upload colloids")))
    return MCFG_ECUDA;
  return MCFG_OK;
}

int mcfg_set_colloids(mcfg_handle* h, const mcfg_colloid_params* cp, const double* x,
                      const double* v, const double* omega, const double* radius) {
  GUARD(h);
  h->graph_gen++;
  if (!cp || cp->num_colloid < 0) return set_error(h, MCFG_EINVAL, "bad colloid parameters");
  const int nc = cp->num_colloid;
  if (nc > 0 && (!x || !v || !omega || !radius))
    return set_error(h, MCFG_EINVAL, "mcfg_set_colloids: NULL array");
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "upload the particles first");
  if ((int)h->h_coll_start.size() - 1 > nc)
    return set_error(h, MCFG_EINVAL, "a particle's sid exceeds num_colloid");
  if (cp->noslip_type < 1 || cp->noslip_type > 2)
    return set_error(h, MCFG_ENOTSUP, "colloid noslip_type must be 1 (frozen) or 2 (Morris)");
  if (h->k.le && nc > 0)
    return set_error(h, MCFG_ENOTSUP, "colloids with Lees-Edwards faces are not supported");
  h->cp = *cp;
  h->cdyn = false;  // new colloids: mcfg_set_colloid_dynamics again to integrate them
  h->coll_host_stale = false;
  h->crad.assign(radius, radius + nc);
  if (nc > 0) {
    int rc;
    if ((rc = dalloc(h, &h->coll, (size_t)nc * 12)) ||
        (rc = dalloc(h, &h->coll_out, (size_t)nc * 12)))
      return rc;
  }
  TRY(put_colloid_state(h, nc, x, v, omega));
  Consts& k = h->k;
  k.ncoll = nc;
  k.coll = h->coll;
  k.coll_noslip = cp->noslip_type;
  k.coll_rho_type = cp->rho_type;
  k.coll_translate = cp->translate;
  k.coll_rotate = cp->rotate;
  k.pp_cc = cp->pp_interact_cc;
  k.coll_dout = cp->dout;
  h->have_density = h->have_pressure = false;
  return MCFG_OK;
}

int mcfg_move_colloids(mcfg_handle* h, const double* x_new, const double* rot, const double* v,
                       const double* omega) {
  GUARD(h);
  h->graph_gen++;
  const int nc = h->k.ncoll, d = h->p.num_dim;
  if (nc == 0) return set_error(h, MCFG_ESTATE, "mcfg_set_colloids must come first");
  if (!x_new || !v || !omega) return set_error(h, MCFG_EINVAL, "mcfg_move_colloids: NULL array");
  if (h->cdyn)
    return set_error(h, MCFG_ESTATE,
                     "mcfg_move_colloids: the colloids are integrated on the device "
                     "(mcfg_set_colloid_dynamics); call mcfg_set_colloids to hand them back");
  // staging: the new centres in coll_out (nc*12 doubles), the rotations in
  // the upload staging (nc*9 <= 3 n: every colloid owns boundary particles)
  double* dx = h->coll_out;
  double* dr = rot ? h->up_v : nullptr;
  if (rot && (size_t)nc * 9 > h->up_cap * 3)
    return set_error(h, MCFG_EINVAL, "more colloids than staging room");
  if (cuda_check(h, cudaMemcpyAsync(dx, x_new, sizeof(double) * (size_t)nc * d,
                                    cudaMemcpyHostToDevice, h->stream), "colloid move") ||
      (rot && cuda_check(h, cudaMemcpyAsync(dr, rot, sizeof(double) * (size_t)nc * 9,
                                            cudaMemcpyHostToDevice, h->stream), "colloid move")))
    return MCFG_ECUDA;
  TRY(colloid_move(h, dx, dr));
  TRY(put_colloid_state(h, nc, x_new, v, omega));
  h->have_list = h->have_density = h->have_pressure = false;
  return MCFG_OK;
}

int mcfg_set_colloid_dynamics(mcfg_handle* h, const mcfg_colloid_dynamics* cd,
                              const double* mass, const double* mmi, const double* v_hist,
                              const double* omega_hist, const double* f_hist,
                              const double* alpha_hist, const double* acc_matrix,
                              const double* theta) {
  GUARD(h);
  h->graph_gen++;
  const int nc = h->k.ncoll, d = h->p.num_dim;
  if (nc == 0) return set_error(h, MCFG_ESTATE, "mcfg_set_colloids must come first");
  if (!cd || !mass || !mmi) return set_error(h, MCFG_EINVAL, "mcfg_set_colloid_dynamics: NULL");
  if (cd->integrate_AB < 1 || cd->integrate_AB > 5)
    return set_error(h, MCFG_EINVAL, "integrate_AB must be 1..5");
  if (cd->sub_time_step < 1) return set_error(h, MCFG_EINVAL, "sub_time_step must be >= 1");
  if (cd->body_force_type != 0 && cd->body_force_type != 1)
    return set_error(h, MCFG_ENOTSUP, "colloid body_force_type must be 0 or 1");
  if (cd->reserved0 != 0) return set_error(h, MCFG_EINVAL, "reserved0 must be 0");
  for (int c = 0; c < nc; ++c) {
    if (!(mass[c] > 0.0)) return set_error(h, MCFG_EPHYS, "colloid mass must be positive");
    for (int a = 0; a < 3; ++a)
      if (h->cp.rotate && (d == 3 || a == 2) && !(mmi[(size_t)c * 3 + a] > 0.0))
        return set_error(h, MCFG_EPHYS, "colloid moment of inertia must be positive");
  }
  const int AB = cd->integrate_AB;
  TRY(colloid_sync_host(h));
  // the device record, laid out as colloid.cu's kRec* offsets
  std::vector<double> rec((size_t)nc * kCollRec, 0.0);
  for (int c = 0; c < nc; ++c) {
    double* r = &rec[(size_t)c * kCollRec];
    r[0] = mass[c];
    for (int a = 0; a < 3; ++a) r[1 + a] = mmi[(size_t)c * 3 + a];
    for (int a = 0; a < 3; ++a) r[4 + a] = theta ? theta[(size_t)c * 3 + a] : 0.0;
    for (int q = 0; q < 9; ++q) {
      r[13 + q] = (q % 4 == 0) ? 1.0 : 0.0;
      r[22 + q] = acc_matrix ? acc_matrix[(size_t)c * 9 + q] : r[13 + q];
    }
    for (int l = 0; l < AB; ++l)
      for (int a = 0; a < 3; ++a) {
        const size_t iv = ((size_t)l * nc + c) * d + a, i3 = ((size_t)l * nc + c) * 3 + a;
        double vv = 0.0, ff = 0.0;
        if (a < d) {
          vv = v_hist ? v_hist[iv] : (l == 0 ? h->cv[(size_t)c * d + a] : 0.0);
          ff = f_hist ? f_hist[iv] : 0.0;
        }
        r[31 + 3 * l + a] = vv;
        r[46 + 3 * l + a] = omega_hist ? omega_hist[i3] : (l == 0 ? h->com[(size_t)c * 3 + a] : 0.0);
        r[61 + 3 * l + a] = ff;
        r[76 + 3 * l + a] = alpha_hist ? alpha_hist[i3] : 0.0;
      }
  }
  int rc;
  if ((rc = dalloc(h, &h->crec, rec.size())) || (rc = dalloc(h, &h->cxnew, (size_t)nc * 3)))
    return rc;
  if (cuda_check(h, cudaMemcpyAsync(h->crec, rec.data(), sizeof(double) * rec.size(),
                                    cudaMemcpyHostToDevice, h->stream), "colloid dynamics"))
    return MCFG_ECUDA;
  // level 1 of the histories is the colloids' velocity in the table the
  // sweeps read
  std::vector<double> v1((size_t)nc * d), w1((size_t)nc * 3);
  for (int c = 0; c < nc; ++c) {
    for (int a = 0; a < d; ++a) v1[(size_t)c * d + a] = rec[(size_t)c * kCollRec + 31 + a];
    for (int a = 0; a < 3; ++a) w1[(size_t)c * 3 + a] = rec[(size_t)c * kCollRec + 46 + a];
  }
  std::vector<double> x0(h->cx);
  TRY(put_colloid_state(h, nc, x0.data(), v1.data(), w1.data()));
  h->cdp = *cd;
  h->cdyn = true;
  return MCFG_OK;
}

int mcfg_colloid_integrate(mcfg_handle* h, int64_t step, double dt) {
  GUARD(h);
  if (!h->cdyn) return set_error(h, MCFG_ESTATE, "mcfg_set_colloid_dynamics must come first");
  if (!h->have_force) return set_error(h, MCFG_ESTATE, "no force computed yet");
  if (step - h->cdp.step_start < 1)
    return set_error(h, MCFG_EINVAL, "step must follow step_start (Adams-Bashforth order >= 1)");
  h->graph_gen++;
  TRY(colloid_section(h, step, dt));
  h->have_list = h->have_density = h->have_pressure = false;
  h->reuse_valid = false;
  return check_device_errors(h);
}

int mcfg_get_colloid_state(mcfg_handle* h, double* x, double* v_hist, double* omega_hist,
                           double* f_hist, double* alpha_hist, double* drag, double* torque,
                           double* rot_matrix, double* acc_matrix, double* acc_vector,
                           double* theta) {
  GUARD(h);
  const int nc = h->k.ncoll, d = h->p.num_dim;
  if (nc == 0) return set_error(h, MCFG_ESTATE, "no colloids");
  TRY(colloid_sync_host(h));
  if (x) std::copy(h->cx.begin(), h->cx.end(), x);
  if (!h->cdyn) {
    if (v_hist || omega_hist || f_hist || alpha_hist || drag || torque || rot_matrix ||
        acc_matrix || acc_vector || theta)
      return set_error(h, MCFG_ESTATE, "no device dynamics (mcfg_set_colloid_dynamics)");
    return MCFG_OK;
  }
  const int AB = h->cdp.integrate_AB;
  std::vector<double> rec((size_t)nc * kCollRec);
  if (cuda_check(h, cudaMemcpyAsync(rec.data(), h->crec, sizeof(double) * rec.size(),
                                    cudaMemcpyDeviceToHost, h->stream), "colloid record") ||
      cuda_check(h, cudaStreamSynchronize(h->stream), "colloid record"))
    return MCFG_ECUDA;
  for (int c = 0; c < nc; ++c) {
    const double* r = &rec[(size_t)c * kCollRec];
    for (int l = 0; l < AB; ++l)
      for (int a = 0; a < 3; ++a) {
        const size_t iv = ((size_t)l * nc + c) * d + a, i3 = ((size_t)l * nc + c) * 3 + a;
        if (a < d && v_hist) v_hist[iv] = r[31 + 3 * l + a];
        if (a < d && f_hist) f_hist[iv] = r[61 + 3 * l + a];
        if (omega_hist) omega_hist[i3] = r[46 + 3 * l + a];
        if (alpha_hist) alpha_hist[i3] = r[76 + 3 * l + a];
      }
    for (int a = 0; a < 3; ++a) {
      if (a < d && drag) drag[(size_t)c * d + a] = r[7 + a];
      if (torque) torque[(size_t)c * 3 + a] = r[10 + a];
      if (theta) theta[(size_t)c * 3 + a] = r[4 + a];
    }
    for (int q = 0; q < 9; ++q) {
      if (rot_matrix) rot_matrix[(size_t)c * 9 + q] = r[13 + q];
      if (acc_matrix) acc_matrix[(size_t)c * 9 + q] = r[22 + q];
    }
    if (acc_vector) {
      // tool_rotation_vector.F90 on the accumulated matrix (as MCF's
      // colloid_compute_accumulation_vector, which divides by sin(phi)
      // also when phi is 0)
      const double* am = r + 22;
      const double phi = std::acos((am[0] + am[4] + am[8] - 1.0) / 2.0);
      double* av = acc_vector + (size_t)c * 4;
      av[0] = (am[2 + 3 * 1] - am[1 + 3 * 2]) / (2.0 * std::sin(phi));
      av[1] = (am[0 + 3 * 2] - am[2 + 3 * 0]) / (2.0 * std::sin(phi));
      av[2] = (am[1 + 3 * 0] - am[0 + 3 * 1]) / (2.0 * std::sin(phi));
      av[3] = phi;
    }
  }
  return MCFG_OK;
}

int mcfg_colloid_drag(mcfg_handle* h, double* drag, double* torque) {
  GUARD(h);
  if (!h->have_force) return set_error(h, MCFG_ESTATE, "no force computed yet");
  return colloid_drag(h, drag, torque);
}

int mcfg_colloid_repulsion(mcfg_handle* h, double* force) {
  GUARD(h);
  if (!force) return set_error(h, MCFG_EINVAL, "NULL output");
  TRY(colloid_sync_host(h));
  const int nc = h->k.ncoll, d = h->p.num_dim;
  const mcfg_colloid_params& cp = h->cp;
  for (int q = 0; q < nc * d; ++q) force[q] = 0.0;
  if (cp.cc_repul_type < 1) return MCFG_OK;
  const double hn = cp.cc_repul_cut_off, hm = cp.cc_repul_cut_on, F0 = cp.cc_repul_F0;
  for (int i = 0; i < nc; ++i)
    for (int j = i + 1; j < nc; ++j) {
      double R12[3] = {0, 0, 0}, rr = 0.0;
      for (int a = 0; a < d; ++a) {
        double r = h->cx[(size_t)i * d + a] - h->cx[(size_t)j * d + a];
        if (h->k.periodic[a]) {
          if (r > 0.5 * h->k.len[a])
            r -= h->k.len[a];
          else if (r < -0.5 * h->k.len[a])
            r += h->k.len[a];
        }
        R12[a] = r;
        rr += r * r;
      }
      const double r = std::sqrt(rr);
      double gap = r - (h->crad[i] + h->crad[j]);
      if (!(gap < 5.0 * hn)) continue;
      double F = 0.0;
      if (cp.cc_repul_type == 1) {  // Hookean
        if (gap < hn) {
          if (gap < hm) gap = hm;
          F = F0 - F0 * gap / hn;
        }
      } else {  // DLVO
        if (gap < hm) gap = hm;
        F = F0 / hn * std::exp(-gap / hn) / (1.0 - std::exp(-gap / hn)) -
            F0 / hn * std::exp(-5.0) / (1.0 - std::exp(-5.0));
      }
      // colloid_compute_repulsion_cc.F90:155-156: R12 / r, then F times it
      for (int a = 0; a < d; ++a) {
        const double fij = F * (R12[a] / r);
        force[(size_t)i * d + a] += fij;
        force[(size_t)j * d + a] -= fij;
      }
    }
  return MCFG_OK;
}

int mcfg_statistics(mcfg_handle* h, double* k_energy, double* momentum, double* stress) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  return statistics(h, k_energy, momentum, stress, h->n);
}

int mcfg_statistics_owned(mcfg_handle* h, int64_t n_owned, double* k_energy, double* momentum,
                          double* stress) {
  GUARD(h);
  if (!h->have_particles) return set_error(h, MCFG_ESTATE, "no particles uploaded");
  if (n_owned < 0 || n_owned > h->n)
    return set_error(h, MCFG_EINVAL, "n_owned must lie in [0, n]");
  return statistics(h, k_energy, momentum, stress, n_owned);
}

void* mcfg_get_stream(mcfg_handle* h) { return h ? (void*)h->stream : nullptr; }

int mcfg_set_profiling(mcfg_handle* h, int mode) {
  GUARD(h);
  if (mode == 2) {
    if (cuda_check(h, cudaStreamSynchronize(h->stream), "synchronize")) return MCFG_ECUDA;
    resolve_phases(h);
    for (int ph = 0; ph < 5; ++ph) {
      h->phase_ms[ph] = 0.0;
      h->phase_cnt[ph] = 0;
    }
    return MCFG_OK;
  }
  if (mode != 0 && mode != 1) return set_error(h, MCFG_EINVAL, "profiling mode must be 0, 1 or 2");
  h->profiling = mode == 1;
  return MCFG_OK;
}

int mcfg_get_phase_times(mcfg_handle* h, double* ms, int64_t* counts) {
  GUARD(h);
  if (cuda_check(h, cudaStreamSynchronize(h->stream), "synchronize")) return MCFG_ECUDA;
  resolve_phases(h);
  for (int ph = 0; ph < 5; ++ph) {
    if (ms) ms[ph] = h->phase_ms[ph];
    if (counts) counts[ph] = h->phase_cnt[ph];
  }
  return MCFG_OK;
}

int mcfg_synchronize(mcfg_handle* h) {
  GUARD(h);
  if (cuda_check(h, cudaStreamSynchronize(h->stream), "synchronize")) return MCFG_ECUDA;
  return check_device_errors(h);
}

}  // extern "C"
