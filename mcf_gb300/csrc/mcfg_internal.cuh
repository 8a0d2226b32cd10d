// mcfg_internal.cuh -- handle layout and device helpers shared by the
// translation units of libmcfg (GB300-native SDPD step, sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/mcfg.h"

namespace mcfg {

constexpr int kWarp = 32;
constexpr int kMaxStencil = 30;   // 3D full stencil 27 (2D 9) + 3 (1) Lees-Edwards slots
// neighbour-slot shift word: 2 bits per axis (1: image at x + L, 2: the home
// particle's image at x + L), and the Lees-Edwards crossings: kLeUp, the
// neighbour is a particle of the bottom row imaged above the y+ face;
// kLeDown, the home particle is the bottom-row one imaged above
constexpr int kLeUp = 1 << 8;
constexpr int kLeDown = 1 << 9;
constexpr int kLocalBits = 11;    // neighbour entry: slot<<11 | local index
constexpr int kMaxCellCount = 1 << kLocalBits;  // particles per cell limit
constexpr double kPi = 3.141592653589793238;    // mcf_header.F90:50

// device-side error flags (bitmask in Handle::d_err)
enum DevErr : unsigned {
  kErrNeighOverflow = 1u,   // neighbour list capacity exceeded
  kErrCellOverflow = 2u,    // a cell holds more than kMaxCellCount particles
  kErrZeroDensity = 4u,     // non-positive density met in a pair
  kErrNonFinite = 8u,       // NaN/Inf produced
};

// Constants of one configuration, passed by value to kernels.
struct Consts {
  int d;
  int n;                 // particles
  int ncell;             // real cells
  int nm[3];             // cells per dimension
  int periodic[3];
  int bc_lo[3], bc_hi[3];   // bcdef of the lower / upper face per axis
  double xmin[3], xmax[3];  // mesh extent (min_phys_t, max_phys_t)
  double rdx[3];            // Nm/(xmax-xmin), ppm_util_rank3d.F90:352-354
  double cs[3];             // cell side (xmax-xmin)/Nm
  double len[3];            // period per dimension
  float csf[3];
  double rc2;               // cut_off**2
  float rc2f, rc2f_hi;      // FP32 cut-off^2 and its prefilter bound
  // neighbour-list reuse (mcfg_params.reserved[1] != 0): the candidates
  // within rc + skin are listed at a rebuild and re-tested every step; a
  // rebuild happens when a particle has moved more than skin/2 since the
  // last one.  skin = 0.99 (smallest cell side - rc), so the 27/9-cell
  // stencil of the rebuild still holds every pair of the step.
  int reuse;
  double half_skin2;        // (skin/2)^2
  float rv2f;               // FP32 bound of the candidate list, (rc + skin)^2 with slack
  // kernel
  int kernel_type;
  double h, inv_h, coef, coef_grad, w0;
  float hf, inv_hf, coeff, coef_gradf, w0f;
  // FP32 copies of the pair constants (the FP32 path never converts from
  // double inside a pair loop: GB300's FP64 pipe is narrow)
  float etaf, eta_coeff, ktf;
  float wall_vf[6][3];   // FP32 copy of wall_v
  int wall_axis;         // the single solid-wall axis, -1 if none, -2 if several
  // moving boundaries (boundary_update_boundary.F90): wall_v holds MCF's
  // shear_v at the step's half time (the no-slip velocity), wall_v_end at its
  // end (particles_set_boundary_velocity.F90); with solid walls, wall
  // particles drift with their velocity and take wall_v_end after the step
  int walls;
  double wall_v_end[6][3];
  // Lees-Edwards y faces (planes sliding along x): stencil of ns slots (27/9
  // + 3/1 when le), images above the y+ face at x + le_S modulo L_x with
  // velocity + le_dv; the crossing rows' x cells start le_cu + 1 cells left
  // (top row) / le_cl - 1 cells right (bottom row) of the home cell, and
  // their FP32 slot offsets are shifted by -le_pu / -le_pl cell sides.
  // With list reuse the crossing rows' cells stay those of the shift at the
  // last rebuild (le_cu .. le_pl computed from it) and le_dS = le_S minus
  // that shift moves the images of their slot offsets (0 otherwise).  The
  // rebuild test then measures displacements against the shear the faces
  // impose: x - x_ref - le_aff (y_ref - le_y0), le_aff = le_dS / L_y,
  // against a bound whose square is half_skin_le2.
  int le, ns;
  double le_S, le_dv;
  int le_cu, le_cl;
  double le_pu, le_pl;
  double le_dS, le_aff, le_y0;
  double half_skin_le2;
  // physics
  int rhs_density_type, rhs_force_type, eos_type;
  double c2, rho_ref, gamma, p0;
  double eta, eta_coef, kt;
  int noise;             // Brownian && kt > machine_zero
  int wall_rho_type, wall_noslip_type;
  double init_density;
  double min_phys[3], max_phys[3];
  double wall_v[6][3];
  int stress;
  // colloids (boundary particles sid = 1..ncoll)
  int ncoll, coll_noslip, coll_rho_type, coll_translate, coll_rotate, pp_cc;
  double coll_dout;
  const double* coll;    // device [ncoll][12]: X(3) V(3) Omega(3) R pad(2)
  // Oldroyd-B conformation model (Newtonian == 0)
  int newtonian;
  double G, tau, inv_tau;  // G = n_p kt_p
  uint32_t key0, key1;   // Philox key (seed)
  uint32_t rk[20];       // its round keys (key + r * Weyl increment), taken
                         // from the parameter bank by the unrolled rounds
  int body_force_type;
  double body_force[3];
  double machine_zero;
};

struct Handle {
  mcfg_params p{};
  Consts k{};
  int device = 0;
  cudaStream_t stream = nullptr;
  // mcfg_step_vv_host: a copy stream for the positions' device-to-host copy
  // (overlapping the density and force sweeps), its event, and the host
  // array it fills (null outside that call)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_x = nullptr;
  cudaEvent_t ev_join = nullptr;  // the copy stream joined back (captured host step)
  double* io_x_out = nullptr;
  // device status words (error flags, list statistics, pair count) copied
  // to pinned memory behind a host step, read after its one synchronisation
  struct HostStatus {
    unsigned err;
    int stats[4];
    unsigned long long pairs;
  };
  HostStatus* h_status = nullptr;
  std::string err;
  bool have_particles = false, have_list = false, have_density = false,
       have_pressure = false, have_force = false;
  int64_t n = 0;
  int64_t n_boundary = 0;  // uploaded particles with sid != 0 (walls, colloids)
  int cap_n = 0;           // allocated particle capacity
  int neigh_cap = 0;       // neighbour list capacity per particle
  double dt = 0.0;
  // moving boundaries: MCF's shear_type / shear_freq per face and time_current
  int32_t shear_type[6] = {0, 0, 0, 0, 0, 0};
  double shear_freq[6] = {0, 0, 0, 0, 0, 0};
  double time_current = 0.0;
  // Lees-Edwards with list reuse: the shift of the last rebuild, the skin
  // and the candidate radius rc + skin
  double le_S_ref = 0.0, le_skin = 0.0, le_reach = 0.0;
  int64_t launches = 0;
  int64_t device_bytes = 0;
  int64_t num_outside = 0;
  int64_t num_pairs = 0;
  int max_neigh = 0;

  // ---- state, sorted by cell (index = sorted slot) ----
  double4_32a* x = nullptr;   // position (w unused)
  double4_32a* v = nullptr;   // velocity
  double4_32a* f = nullptr;   // acceleration
  double* m = nullptr;
  int* pid = nullptr;
  int* sid = nullptr;
  int* hidx = nullptr;    // host index of the particle in this slot
  double* rho = nullptr;
  double* pr = nullptr;
  double* st = nullptr;   // stress, [d*d][cap] component-major
  // Oldroyd-B state, [d*d][cap] component-major (component a + d*b)
  double* ct = nullptr;   // conformation tensor
  double* act = nullptr;  // d(ct)/dt of the last right-hand side
  double* vgt = nullptr;  // velocity gradient tensor
  double *ct2 = nullptr, *act2 = nullptr;
  void* qq = nullptr;     // per-particle 1/n and G*ct/n^2, [1+d*d][cap] (T)
  // colloids
  mcfg_colloid_params cp{};
  std::vector<double> cx, cv, com, crad;  // host copies (repulsion)
  double* coll = nullptr;      // device [nc][12]
  int* coll_start = nullptr;   // [nc+1] CSR of boundary particles (host indices)
  int* coll_mem = nullptr;
  int coll_nmem = 0;
  std::vector<int> h_coll_start, h_coll_mem;
  int* slot_of = nullptr;      // host index -> sorted slot
  double4_32a* rxc = nullptr;  // FP64 path: boundary particle minus its colloid image centre
  float4* rxcf = nullptr;      // FP32 path: same in FP32
  double* coll_out = nullptr;  // [nc][6] drag + torque
  // rigid-body dynamics of the colloids on the device (colloid.cu)
  bool cdyn = false;             // mcfg_set_colloid_dynamics was called
  mcfg_colloid_dynamics cdp{};
  double* crec = nullptr;        // [nc][kCollRec] masses, histories, matrices
  double* cxnew = nullptr;       // [nc][3] centres after a sub-step
  bool coll_host_stale = false;  // cx/cv/com behind the device table
  // double buffers for the permutation
  double4_32a *x2 = nullptr, *v2 = nullptr, *f2 = nullptr;
  double* m2 = nullptr;
  int *pid2 = nullptr, *sid2 = nullptr, *hidx2 = nullptr;
  // ---- cell list ----
  int* key = nullptr;        // cell of each particle (pre-sort order)
  int* rank = nullptr;       // arrival rank within the cell
  int* cnt = nullptr;        // [ncell+1] counts (last bin: outside)
  int* cell_start = nullptr; // [ncell+2]
  int* scan_part = nullptr;  // scan partials
  int* order = nullptr;      // pre-sort index per unsorted slot
  float4* off = nullptr;     // FP32 offset to the cell origin, w = cell id
  int* cell_of = nullptr;    // cell per sorted particle (ncell = outside)
  // ---- neighbours ----
  uint16_t* nl = nullptr;    // [neigh_cap][cap] entries slot<<11|local; FP32 list reuse:
                             // fluid-fluid pairs from row 0 up, the others from the
                             // last row down, ncount = fluid-fluid | other << 16
  int* ncount = nullptr;     // [cap]
  int* nhs = nullptr;        // [cap] first entry of the owned (forward) half
  void* jp = nullptr;        // symmetric force partial sums [(NSF+1)*3][cap] (T)
  // ---- pair records ----
  double4_32a* pc = nullptr;     // FP64 path: (p/n^2 or p, 1/n^2, 1/m, rho)
  float4* pcf = nullptr;     // FP32 path: same in float
  float4* vf = nullptr;      // FP32 path: velocity (w = packed id bits)
  float2* wd = nullptr;      // FP32 path: signed distances to the wall-axis faces
  // ---- reductions & errors ----
  double* red = nullptr;     // block partials
  unsigned* d_err = nullptr; // device error bitmask
  int* d_stats = nullptr;    // [0] outside count, [1] max neigh, [2] pairs lo
  unsigned long long* d_pairs = nullptr;
  void* h_pinned = nullptr;  // small pinned staging
  // upload staging (device copies of host-order arrays)
  double* up_x = nullptr;
  double* up_v = nullptr;
  double* up_m = nullptr;
  int* up_id = nullptr;
  size_t up_cap = 0;
  // ---- neighbour-list reuse ----
  double4_32a* x_ref = nullptr;  // positions at the last rebuild
  uint16_t* vl = nullptr;        // [vcap][n] candidates within rc + skin (slot<<11 | local);
                                 // FP32 handles: fluid-fluid pairs from row 0 up, the
                                 // others from row vcap-1 down (sweep32.cu)
  bool partitioned = false;      // FP32 lists: fluid-fluid rows up, the others down
  int* vcount = nullptr;         // [n]
  int vcap = 0;
  int* d_rebuild = nullptr;      // [0] rebuild request, [1] rebuilds done
  bool reuse_valid = false;      // the candidate list matches the particle order
  bool unwrapped = false;        // positions may lie outside periodic faces (list reuse)
  // ---- CUDA graph of two list-reuse VV steps (mcfg_run_vv) ----
  // The step is launch-bound below ~50k particles (14 launches a step); run_vv
  // replays a captured pair of steps instead (two: the fused second kick
  // swaps v and v2, so two steps bring the buffers back).  The force sweeps
  // of the captured steps read the Philox step from d_step, which a one-thread
  // kernel advances after every step.  A graph is reused while the handle's
  // constants and buffers are those it captured (graph_gen, v).
  int64_t* d_step = nullptr;
  bool graph_capturing = false;
  bool graph_off = false;        // capture failed once: plain launches from then on
  uint64_t graph_gen = 1;        // bumped whenever constants or buffers change
  struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    uint64_t gen = 0;
    double dt = 0.0;
    const void* v = nullptr;
    int64_t launches = 0;
  } graphs[2];
  // mcfg_step_vv_host with page-locked host arrays replays a captured step:
  // inputs over, the step (positions back on the copy stream), velocities
  // back; one graph per velocity buffer (the fused kick swaps v and v2) and
  // pair of host arrays, baked into the memcpy nodes
  struct HostGraph {
    cudaGraphExec_t exec = nullptr;
    uint64_t gen = 0;
    double dt = 0.0;
    const void* v = nullptr;
    const double* hx = nullptr;
    const double* hv = nullptr;
    int64_t launches = 0;
  } hgraphs[2];
  bool hgraph_off = false;  // a host-step capture failed: plain launches from then on
  // In a captured step the gated rebuild (wrap, MCF's cell list, candidate
  // list) sits in the body of a conditional node that a one-thread kernel
  // opens when the kick-drift kernel raised the rebuild flag, so the steps
  // without a rebuild launch none of its kernels.  The body is captured on
  // cond_stream.  cond_off: the runtime refused it once; the gated kernels
  // then sit in the graph itself.
  cudaStream_t cond_stream = nullptr;
  bool cond_off = false;
  // ---- particle-file text (output.cu), grow-only, null until the first write ----
  char* out_dev = nullptr;
  char* out_host = nullptr;  // pinned
  size_t out_cap = 0;
  // ---- adjoint buffers (adjoint.cu), null until mcfg_adjoint_run ----
  struct AdjBuffers* adj = nullptr;
  // ---- per-phase device timers ----
  bool profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pending[5];
  double phase_ms[5] = {0, 0, 0, 0, 0};
  int64_t phase_cnt[5] = {0, 0, 0, 0, 0};
};

enum Phase { kPhaseList = 0, kPhaseDensity = 1, kPhaseForce = 2, kPhaseUpdate = 3, kPhaseOther = 4 };

// Records CUDA events around one phase when profiling is on.
struct PhaseScope {
  Handle* h;
  int phase;
  std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
  PhaseScope(Handle* hh, int ph) : h(hh), phase(ph) {
    if (!h->profiling) return;
    if (h->ev_pool.empty()) {
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess) return;
      if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return;
      }
      h->ev_pool.push_back({a, b});
    }
    ev = h->ev_pool.back();
    h->ev_pool.pop_back();
    cudaEventRecord(ev.first, h->stream);
  }
  ~PhaseScope() {
    if (!ev.first) return;
    cudaEventRecord(ev.second, h->stream);
    h->ev_pending[phase].push_back(ev);
  }
};

// accumulate completed phase events (call after a stream synchronize)
void resolve_phases(Handle* h);

// parameter checks and derived constants shared by all entry points
const char* validate_params(const mcfg_params* p);
void make_consts(const mcfg_params& p, Consts& k);

// set err and return code
int set_error(Handle* h, int code, const std::string& msg);
int cuda_check(Handle* h, cudaError_t e, const char* what);

}  // namespace mcfg

// the opaque handle of the C ABI
struct mcfg_handle : public mcfg::Handle {};

namespace mcfg {

// launches (implemented in the .cu files)
int build_cell_list(Handle* h);
// list-reuse step pieces: a rebuild (wrap, cell list, candidate list) whose
// kernels all return at once unless a particle has moved more than skin/2
// (device flag), the density sweep over the candidate list, and the kick /
// drift that leaves positions unwrapped and raises the flag
int rebuild_if_needed(Handle* h);
int kick_drift_reuse(Handle* h, double dt);
int wrap_gated(Handle* h);
int gated_cell_list(Handle* h);
int verlet_build_gated(Handle* h);
int compute_density(Handle* h, bool with_pressure, bool reuse = false);
int compute_pressure(Handle* h);
int compute_force(Handle* h, int64_t step, int fuse_mode, double dt);
// FP32-mixed sweeps over the partitioned candidate list (sweep32.cu)
int density_list(Handle* h, bool with_pressure);
int apply_body_force(Handle* h);
int integrate_velocity(Handle* h, double dt, double lambda);
int integrate_position(Handle* h, double dt);
int adjust_particles(Handle* h);
int kick_drift_wrap(Handle* h, double dt);
// FP64 sums over the particles of host index < owned (all of them: owned = n)
int statistics(Handle* h, double* ke, double* mom, double* stress, int64_t owned);
// second half kick v += (0.5 a) dt and, Oldroyd-B, ct += (act dt) 0.5 (the
// unfused tail of a VV step, bit-identical to the fused force epilogue)
int kick_ct_half(Handle* h, double dt);
// right-hand side (cell list, density, pressure, force) and the first half
// of a VV step (kick, drift, wrap, ct half step), with phase timers
int rhs(Handle* h, int64_t step, int fuse_mode, double dt);
int kdw(Handle* h, double dt);
void free_adjoint(Handle* h);
// MCF's boundary_update_boundary(time_r, time_v) into the constants: wall
// shear velocities at time_v (and at time_r for the end of the step),
// Lees-Edwards offset at time_r
void boundary_update(Handle* h, double time_r, double time_v);
// inside mcfg_step_vv_host, once the step's list phase has fixed the
// positions: gather them to host order and copy them to h->io_x_out on the
// copy stream while the sweeps run
int download_x_async(Handle* h);
// release the captured step graphs (buffers or constants changed)
void destroy_graphs(Handle* h);
// MCF's particle output (kind 0) or restart (kind 1) file formatted on the
// device; flags & 1 adds the stress columns s(2), s(3)
int write_particle_file(Handle* h, const char* path, int kind, int flags);
void le_map(Handle* h);
int write_statistic_line(Handle* h, const char* path, int64_t step, double time);
int colloid_drag(Handle* h, double* drag, double* torque);
int colloid_move(Handle* h, const double* d_xnew, const double* d_rot);
int check_device_errors(Handle* h);

// the colloid part of a VV step, the initial colloid accelerations, the
// drag/torque sums into coll_out, host copies of the colloid table
int colloid_section(Handle* h, int64_t step, double dt);
int colloid_initial(Handle* h);
int colloid_drag_launch(Handle* h);
int colloid_sync_host(Handle* h);
// doubles per colloid of the device record of the dynamics (colloid.cu)
constexpr int kCollRec = 96;

// fuse_mode of compute_force
enum { kForceOnly = 0, kForceBody = 1, kForceBodyKick = 2 };

// ------------------------------------------------------------------------
// Device helpers
// ------------------------------------------------------------------------

// Philox4x32-10, Salmon et al., SC'11 ("Parallel random numbers: as easy as
// 1, 2, 3"): multipliers and Weyl key increments of the published algorithm.
// rk: the 10 round keys, rk[2r] = k0 + r * 0x9E3779B9, rk[2r+1] = k1 + r *
// 0xBB67AE85 (Consts::rk, expanded once per configuration).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, const uint32_t* rk) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    // one 32x32 -> 64-bit product per word (low and high halves together)
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
    c = make_uint4(hi1 ^ c.y ^ rk[2 * r], lo1, hi0 ^ c.w ^ rk[2 * r + 1], lo0);
  }
  return c;
}

// odd multiple of 2^-24 in (0,1), exact in FP32: (2*(r>>9)+1)*2^-24 formed
// from the bits of 1 + (r>>9)*2^-23 (no integer-to-float conversion)
__device__ __forceinline__ float u01(uint32_t r) {
  return (__uint_as_float(0x3f800000u | (r >> 9)) - 1.0f) + 5.9604644775390625e-8f;
}

// -2 ln u for the Box-Muller radius: the hardware log2 (2 ulp below 1/2,
// 2^-22 absolute in [1/2, 2]), which keeps the radius within ~4e-6 of the
// exact one for u <= 1 - 2^-10; above, where that absolute error would
// swamp ln u, the series -2 ln(1 - t) = 2t (1 + t/2 + t^2/3 + ...) in the
// exact t = 1 - u (t <= 2^-10: the dropped terms are below 2^-32 of the sum).
// The branch is taken by one lane in a thousand, so warps rarely diverge.
__device__ __forceinline__ float neg2log(float u) {
  if (u > 0.9990234375f) {
    const float t = 1.0f - u;
    return 2.0f * t * fmaf(t, fmaf(t, 0.33333334f, 0.5f), 1.0f);
  }
  return -1.3862943611198906f * __log2f(u);  // -2 ln 2 log2 u
}

// Box-Muller with the angle centred on [-pi, pi], where the hardware sine
// and cosine (absolute error ~2^-21) are at their best.
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
  const float u1 = u01(a), u2 = u01(b);
  const float rad = sqrtf(neg2log(u1));
  float sn, cs;
  __sincosf(6.2831853071795865f * u2 - 3.1415926535897932f, &sn, &cs);
  z0 = rad * cs;
  z1 = rad * sn;
}

// normals of a pair: 3D z[0..5] (diagonal 0..2, off-diagonal 3..5),
// 2D z[0..2]; the counter is (min pid, max pid, step, call) so the draw is
// the same from both particles of the pair.
template <int D>
__device__ __forceinline__ void pair_normals(const uint32_t* rk, uint32_t step,
                                             int pa, int pb, float* z) {
  const uint32_t a = (uint32_t)min(pa, pb), b = (uint32_t)max(pa, pb);
  uint4 r = philox4x32_10(make_uint4(a, b, step, 0u), rk);
  float t0, t1;
  box_muller(r.x, r.y, z[0], z[1]);
  box_muller(r.z, r.w, t0, t1);
  z[2] = t0;
  if (D == 3) {
    z[3] = t1;
    r = philox4x32_10(make_uint4(a, b, step, 1u), rk);
    box_muller(r.x, r.y, z[4], z[5]);
  }
}

// What a pair draws for its random force, by force form, from the stream of
// pair_normals (the first normals of the same counter):
//   type 2 (Espanol-Revenga): the 6 (3D) / 3 (2D) normals of the matrix dW;
//   type 3 (Hu-Adams, also non-Newtonian): d normals g for We = dW e drawn
//     from its law given e (see pair_force), z[5] = +1 when pa < pb, -1
//     otherwise (orients We so that the pair's two sides are opposite);
//   type 4 (angular): one normal.
template <int D>
__device__ __forceinline__ void pair_draw(int type, const uint32_t* rk, uint32_t step,
                                          int pa, int pb, float* z) {
  if (type == 2) {
    pair_normals<D>(rk, step, pa, pb, z);
    return;
  }
  const uint32_t a = (uint32_t)min(pa, pb), b = (uint32_t)max(pa, pb);
  const uint4 r = philox4x32_10(make_uint4(a, b, step, 0u), rk);
  box_muller(r.x, r.y, z[0], z[1]);
  if (type == 3) {
    if (D == 3) {
      float t1;
      box_muller(r.z, r.w, z[2], t1);
    }
    z[5] = (pa < pb) ? 1.0f : -1.0f;
  }
}

}  // namespace mcfg
