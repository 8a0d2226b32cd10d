// output.cu -- MCF's particle files, formatted on the device.
//
// MCF writes its particle output (io_write_particles.F90:225-403) and
// restart files (io_write_restart_particles.F90:100-215) through ppm_io in
// ASCII mode: WRITE(unit, '(<data_dim>E16.8)') of the (data_dim, N) array,
// one record per particle, columns x(d) v(d) rho m pid sid (the output file
// adds the stress components s(2), s(3) when MCF is built with
// __IO_PARTICLES_STRESS_TOTAL); the restart file first writes the particle
// count list-directed (ppm_io_write_ascii.F90).  Formatting a million
// particles' text with the Fortran runtime takes seconds; here one thread
// per value writes its 16 characters into a device buffer (rows in host
// order), and the host copies the text once and writes it.
//
// E16.8: [-]0.dddddddd followed by E+ee (|exponent| <= 99) or +eee,
// right-justified in 16 columns.  The eight digits are the correctly
// rounded decimal value of the double, ties to even (what the C library's
// %.7E gives), computed exactly with 128-bit integers for magnitudes in
// [1e-18, 1e30); outside that range from an FP64 estimate (error below
// 1e-15 relative, so only values within that distance of a rounding
// boundary can differ).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "mcfg_internal.cuh"

namespace mcfg {
namespace {

struct U128 {
  uint64_t lo, hi;
};

__device__ __forceinline__ U128 mul64(uint64_t a, uint64_t b) { return {a * b, __umul64hi(a, b)}; }

// a * b, the product below 2^128
__device__ __forceinline__ U128 mul128(U128 a, uint64_t b) {
  U128 r = mul64(a.lo, b);
  r.hi += a.hi * b;
  return r;
}

// a << s, 0 <= s < 128, no bit shifted out
__device__ __forceinline__ U128 shl(U128 a, int s) {
  if (s == 0) return a;
  if (s >= 64) return {0, a.lo << (s - 64)};
  return {a.lo << s, (a.hi << s) | (a.lo >> (64 - s))};
}

__device__ __forceinline__ int cmp(U128 a, U128 b) {
  if (a.hi != b.hi) return a.hi < b.hi ? -1 : 1;
  if (a.lo != b.lo) return a.lo < b.lo ? -1 : 1;
  return 0;
}

__device__ __forceinline__ uint64_t pow5(int k) {
  uint64_t r = 1;
  for (int i = 0; i < k; ++i) r *= 5;
  return r;
}

// m 2^q 10^p as an exact ratio A / D with A < 2^124 and D < 2^100, for
// -22 <= p <= 26; false outside that range
__device__ bool scaled_ratio(uint64_t m, int q, int p, U128& A, U128& D) {
  if (p >= 0) {
    if (p > 26) return false;
    A = mul64(m, pow5(p));  // < 2^53 * 5^26 < 2^114
    const int k = -(q + p);
    if (k <= 0 || k >= 100) return false;
    D = shl(U128{1, 0}, k);
    return true;
  }
  const int a = -p;
  if (a > 22) return false;
  const int s = q - a;  // value = m 2^s / 5^a
  const uint64_t p5 = pow5(a);
  if (s >= 0) {
    if (s > 70) return false;
    A = shl(U128{m, 0}, s);
    D = U128{p5, 0};
  } else {
    if (-s > 40) return false;
    A = U128{m, 0};
    D = shl(U128{p5, 0}, -s);
  }
  return true;
}

// N = round(A / D), ties to even, from an estimate within a few units
__device__ uint32_t round_ratio(U128 A, U128 D, uint32_t N) {
  const U128 A2 = shl(A, 1);
  for (int it = 0; it < 4 && cmp(A2, mul128(D, 2ull * N + 1)) > 0; ++it) ++N;
  for (int it = 0; it < 4 && N > 0 && cmp(A2, mul128(D, 2ull * N - 1)) < 0; ++it) --N;
  if ((N & 1u) && cmp(A2, mul128(D, 2ull * N + 1)) == 0)
    ++N;
  else if ((N & 1u) && N > 0 && cmp(A2, mul128(D, 2ull * N - 1)) == 0)
    --N;
  return N;
}

// |x| = 0.d1...d8 x 10^E with N = d1...d8 in [10^7, 10^8), x finite, > 0
__device__ void dec8(double ax, uint32_t& N, int& E) {
  const uint64_t bits = (uint64_t)__double_as_longlong(ax);
  const int eb = (int)((bits >> 52) & 0x7ff);
  uint64_t m = bits & 0xFFFFFFFFFFFFFull;
  int q;
  if (eb == 0) {
    q = -1074;
  } else {
    m |= 1ull << 52;
    q = eb - 1075;
  }
  int E0 = (int)floor(log10(ax)) + 1;
  N = 10000000u;
  E = E0;
  for (int pass = 0; pass < 4; ++pass) {
    const int p = 8 - E0;
    const int p1 = p / 2;
    const double est = (ax * exp10((double)p1)) * exp10((double)(p - p1));
    const uint32_t Ne = (uint32_t)fmin(fmax(rint(est), 0.0), 4.0e9);
    U128 A, D;
    const uint32_t Nr = scaled_ratio(m, q, p, A, D) ? round_ratio(A, D, Ne) : Ne;
    if (Nr >= 100000000u) {
      ++E0;
      continue;
    }
    if (Nr < 10000000u) {
      --E0;
      continue;
    }
    N = Nr;
    E = E0;
    return;
  }
}

// Fortran E16.8 of x into out[0..15]
__device__ void fmt_e16_8(double x, char* out) {
  char t[16];
  int k = 0;
  if (isnan(x)) {
    t[k++] = 'N';
    t[k++] = 'a';
    t[k++] = 'N';
  } else if (isinf(x)) {
    if (x < 0) t[k++] = '-';
    const char inf[] = "Infinity";
    for (int i = 0; i < 8; ++i) t[k++] = inf[i];
  } else {
    const double ax = fabs(x);
    uint32_t N = 0;
    int E = 0;
    if (ax != 0.0) dec8(ax, N, E);
    if (signbit(x)) t[k++] = '-';
    t[k++] = '0';
    t[k++] = '.';
#pragma unroll
    for (int i = 7; i >= 0; --i) {
      t[k + i] = (char)('0' + N % 10u);
      N /= 10u;
    }
    k += 8;
    const int ae = E < 0 ? -E : E;
    if (ae <= 99) {
      t[k++] = 'E';
      t[k++] = E < 0 ? '-' : '+';
    } else {
      t[k++] = E < 0 ? '-' : '+';
      t[k++] = (char)('0' + ae / 100);
    }
    t[k++] = (char)('0' + (ae / 10) % 10);
    t[k++] = (char)('0' + ae % 10);
  }
  const int pad = 16 - k;
  for (int i = 0; i < 16; ++i) out[i] = (i < pad) ? ' ' : t[i - pad];
}

// one thread per (particle, column); rows in host order.  Columns:
// x(d) (wrapped like mcfg_download), v(d), rho, m, pid, sid, then the
// stress components s(2), s(3) when requested.
template <int D>
__global__ void k_format_particles(Consts k, int n, int ncol, int line,
                                   const int* __restrict__ hidx,
                                   const double4_32a* __restrict__ x,
                                   const double4_32a* __restrict__ v,
                                   const double* __restrict__ rho, const double* __restrict__ m,
                                   const int* __restrict__ pid, const int* __restrict__ sid,
                                   const double* __restrict__ st, char* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * ncol) return;
  const int i = (int)(t / ncol), c = (int)(t - (int64_t)i * ncol);
  double val;
  if (c < D) {
    const double4_32a xv = x[i];
    double xa = (c == 0) ? xv.x : (c == 1 ? xv.y : xv.z);
    if (xa < k.min_phys[c] && k.bc_lo[c] == MCFG_BC_PERIODIC) xa = __dadd_rn(xa, k.len[c]);
    if (xa >= k.max_phys[c] && k.bc_hi[c] == MCFG_BC_PERIODIC) xa = __dsub_rn(xa, k.len[c]);
    val = xa;
  } else if (c < 2 * D) {
    const double4_32a vv = v[i];
    const int a = c - D;
    val = (a == 0) ? vv.x : (a == 1 ? vv.y : vv.z);
  } else if (c == 2 * D) {
    val = rho[i];
  } else if (c == 2 * D + 1) {
    val = m[i];
  } else if (c == 2 * D + 2) {
    val = (double)pid[i];
  } else if (c == 2 * D + 3) {
    val = (double)sid[i];
  } else {
    val = st[(size_t)(c - 2 * D - 3) * n + i];  // s(2), s(3): components 1, 2
  }
  char* o = out + (size_t)hidx[i] * line + (size_t)c * 16;
  fmt_e16_8(val, o);
  if (c == ncol - 1) o[16] = '\n';
}

}  // namespace

int write_particle_file(Handle* h, const char* path, int kind, int flags) {
  const int n = (int)h->n, d = h->p.num_dim;
  const bool stress = (flags & 1) != 0;
  if (stress && !h->p.stress_tensor) return set_error(h, MCFG_EINVAL, "stress_tensor is off");
  if (stress && !h->have_force)
    return set_error(h, MCFG_ESTATE, "no stress yet: run mcfg_init_force first");
  const int ncol = 2 * d + 4 + (stress ? 2 : 0);
  const int line = 16 * ncol + 1;
  const size_t bytes = (size_t)n * line;
  if (bytes > h->out_cap) {
    if (h->out_dev) cudaFree(h->out_dev);
    if (h->out_host) cudaFreeHost(h->out_host);
    h->out_dev = nullptr;
    h->out_host = nullptr;
    h->out_cap = 0;
    if (cudaMalloc(&h->out_dev, bytes) != cudaSuccess ||
        cudaMallocHost(&h->out_host, bytes) != cudaSuccess) {
      if (h->out_dev) cudaFree(h->out_dev);
      h->out_dev = nullptr;
      h->out_host = nullptr;
      cudaGetLastError();
      return set_error(h, MCFG_ENOMEM, "output text buffers");
    }
    h->out_cap = bytes;
  }
  if (n > 0) {
    const int64_t total = (int64_t)n * ncol;
    const int tb = 256;
    const int gb = (int)((total + tb - 1) / tb);
    if (d == 3)
      k_format_particles<3><<<gb, tb, 0, h->stream>>>(h->k, n, ncol, line, h->hidx, h->x, h->v,
                                                      h->rho, h->m, h->pid, h->sid, h->st,
                                                      h->out_dev);
    else
      k_format_particles<2><<<gb, tb, 0, h->stream>>>(h->k, n, ncol, line, h->hidx, h->x, h->v,
                                                      h->rho, h->m, h->pid, h->sid, h->st,
                                                      h->out_dev);
    h->launches++;
    if (cuda_check(h, cudaGetLastError(), "format launch") ||
        cuda_check(h, cudaMemcpyAsync(h->out_host, h->out_dev, bytes, cudaMemcpyDeviceToHost,
                                      h->stream),
                   "output copy") ||
        cuda_check(h, cudaStreamSynchronize(h->stream), "output sync"))
      return MCFG_ECUDA;
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(h, MCFG_EINVAL, std::string("cannot open ") + path);
  bool ok = true;
  // the restart file's particle count, list-directed (a blank, then I11)
  if (kind == 1) ok = std::fprintf(f, "%12d\n", n) > 0;
  if (ok && bytes > 0) ok = std::fwrite(h->out_host, 1, bytes, f) == bytes;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return set_error(h, MCFG_EINVAL, std::string("write failed: ") + path);
  return MCFG_OK;
}

// Fortran E16.8 on the host, for the few values of a statistic line: the C
// library's %.7E prints the same eight correctly rounded digits (ties to
// even) as d.dddddddE+xx, one decimal exponent below E16.8's 0.dddddddd.
static void host_e16_8(double x, std::string& line) {
  char t[48];
  std::string body;
  if (std::isnan(x)) {
    body = "NaN";
  } else if (std::isinf(x)) {
    body = x < 0 ? "-Infinity" : "Infinity";
  } else {
    const double ax = std::fabs(x);
    std::string digits = "00000000";
    int e = 0;
    if (ax != 0.0) {
      std::snprintf(t, sizeof t, "%.7E", ax);
      digits[0] = t[0];
      for (int i = 0; i < 7; ++i) digits[1 + i] = t[2 + i];
      e = std::atoi(t + 10) + 1;
    }
    if (std::signbit(x)) body += '-';
    body += "0.";
    body += digits;
    const int ae = e < 0 ? -e : e;
    if (ae <= 99)
      std::snprintf(t, sizeof t, "E%c%02d", e < 0 ? '-' : '+', ae);
    else
      std::snprintf(t, sizeof t, "%c%03d", e < 0 ? '-' : '+', ae);
    body += t;
  }
  if (body.size() < 16) line.append(16 - body.size(), ' ');
  line += body;
}

int write_statistic_line(Handle* h, const char* path, int64_t step, double time) {
  const int d = h->p.num_dim;
  double ke = 0.0, mom[3] = {0.0, 0.0, 0.0}, st[9] = {0.0};
  const int rc = statistics(h, &ke, mom, st, h->n);
  if (rc != MCFG_OK) return rc;
  std::string line;
  if (step >= -99999999 && step <= 999999999) {
    char t[16];
    std::snprintf(t, sizeof t, "%9lld", (long long)step);
    line = t;
  } else {
    line = "*********";
  }
  host_e16_8(time, line);
  host_e16_8(ke, line);
  for (int a = 0; a < d; ++a) host_e16_8(mom[a], line);
  if (h->p.stress_tensor) {
    host_e16_8(st[1], line);
    host_e16_8(st[2], line);
  }
  line += '\n';
  FILE* f = std::fopen(path, "ab");
  if (!f) return set_error(h, MCFG_EINVAL, std::string("cannot open ") + path);
  const bool ok = std::fwrite(line.data(), 1, line.size(), f) == line.size();
  if (!((std::fclose(f) == 0) && ok))
    return set_error(h, MCFG_EINVAL, std::string("write failed: ") + path);
  return MCFG_OK;
}

}  // namespace mcfg
