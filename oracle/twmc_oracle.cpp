// twmc_oracle.cpp -- FP64 CPU restatement of the reference's TWMC hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle: tests/, the smoke check
// and bench.py's CPU-baseline leg load it as the checker (or as the timed CPU
// reference arm). The product path (pincosimulator_gb300) never links, loads
// or calls it.
//
// Parity status: the reference itself cannot be built here (it needs FFTW3,
// Eigen3, cpptoml, CLI11 and easylogging++, none of which is installed or
// vendored), and the reference ships no tests or golden vectors. Parity with
// the reference is therefore UNPINNED by reference outputs; this restatement
// is pinned instead by closed-form known-answer tests of the discrete Euler
// recursion (tests/test_oracle_kat.py), by an independent numpy restatement
// (oracle/twmc_oracle.py, numpy's pocketfft instead of this file's FFT), and
// its Philox4x32-10 by an independent Python implementation and cuRAND's
// host-side Philox4x32-10 generator.
//
// What it restates (paths relative to the reference project root):
//   * TWMCBaseSolver::Setup / Compute     src/TWMC/Solvers/TWMCBaseSolver.cpp:24-92, 94-283
//       k-space hopping table             :78-88
//       hot loop (Euler-Maruyama)         :232-266
//       frame capture / truncation        :220-229, 257-274
//   * TWMCLiebSolver::Setup / Compute     src/TWMC/Solvers/TWMCLiebSolver.cpp:29-104, 109-299
//       coupling triplets                 :52-85
//       hot loop                          :250-280
//   * NoisyMatrix::GetAtTimeWithSuggestion src/Base/NoisyMatrix.cpp:252-265
//     NoisyMatrix::SetTemporalValue       src/Base/NoisyMatrix.cpp:164-250
//   * TWMCSystemData frame grid           src/TWMC/TWMCSystemData.cpp:66-134
// The reference draws its noise from std::mt19937 + std::normal_distribution,
// whose stream is implementation-defined; this oracle takes the noise either
// from a caller-supplied buffer (deterministic-noise mode) or from the
// counter-based Philox4x32-10 stream the GPU solver uses.
//
// Build: oracle/build_oracle.py (g++ -O2 -ffp-contract=off, no fast-math).

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <random>
#include <atomic>
#include <limits>
#include <thread>
#include <vector>

using cd = std::complex<double>;

namespace {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11). Round function: two 32x32->64 multiplies, key bumped by
// the Weyl constants between rounds.
// ---------------------------------------------------------------------------
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = uint64_t(kPhiloxM0) * c0;
    uint64_t p1 = uint64_t(kPhiloxM1) * c2;
    uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
    uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += kPhiloxW0; k1 += kPhiloxW1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Noise streams (counter word 2). Shared convention with the GPU solver.
enum Stream : uint32_t { kStreamWiener = 0, kStreamInit = 1, kStreamU = 2, kStreamOmega = 3, kStreamF = 4 };
// The Wiener stream has a fixed key (hex digits of pi) and the trajectory in
// the counter: ctr = (site pair, step, tid, seed). The other streams use
// key = (seed, tid), ctr = (site pair, step, stream, 0).
constexpr uint32_t kWienerKey0 = 0x243F6A88u, kWienerKey1 = 0x85A308D3u;

// Box-Muller from two 32-bit words, FP64 flavour: u = (a + 1/2) 2^-32.
void normal_pair_f64(uint32_t a, uint32_t b, double* z0, double* z1) {
  const double u1 = (double(a) + 0.5) * 0x1p-32;
  const double u2 = (double(b) + 0.5) * 0x1p-32;
  const double r = std::sqrt(-2.0 * std::log(u1));
  const double th = 2.0 * M_PI * u2 - M_PI;
  *z0 = r * std::cos(th);
  *z1 = r * std::sin(th);
}

// FP32 flavour: the uniforms are formed exactly as the FP32 kernel forms them
// (one correctly rounded float fma each), the transcendental part in FP64.
void normal_pair_f32(uint32_t a, uint32_t b, double* z0, double* z1) {
  const float u1 = std::fma(float(a), 0x1p-32f, 0x1p-33f);
  // th = 2 pi u2 - pi with u2 = float(b) 2^-32 + 2^-33, as one FP32 fma of float(b)
  const float th = std::fma(float(b), float(2.0 * M_PI * 0x1p-32), float(2.0 * M_PI * 0x1p-33 - M_PI));
  const double r = std::sqrt(std::max(0.0, -2.0 * std::log(double(u1))));
  *z0 = r * std::cos(double(th));
  *z1 = r * std::sin(double(th));
}

// Pairing of sites onto Philox calls: with half = ceil(N/2), site p < half
// takes words (0,1) of call p, site p >= half takes words (2,3) of call p-half.
inline void site_counter(int64_t p, int64_t n, uint32_t* c0, int* lane) {
  const int64_t half = (n + 1) / 2;
  if (p < half) { *c0 = uint32_t(p); *lane = 0; }
  else { *c0 = uint32_t(p - half); *lane = 2; }
}

// Complex normal xi = z0 + i z1 for one site.
cd site_normal(uint32_t seed, uint32_t tid, uint32_t step, uint32_t stream, int64_t p, int64_t n,
               int f32_flavour) {
  uint32_t c0; int lane;
  site_counter(p, n, &c0, &lane);
  const bool wiener = stream == kStreamWiener;
  const uint32_t ctr[4] = {c0, step, wiener ? tid : stream, wiener ? seed : 0u};
  const uint32_t key[2] = {wiener ? kWienerKey0 : seed, wiener ? kWienerKey1 : tid};
  uint32_t w[4];
  philox4x32_10(ctr, key, w);
  double z0, z1;
  if (f32_flavour) normal_pair_f32(w[lane], w[lane + 1], &z0, &z1);
  else normal_pair_f64(w[lane], w[lane + 1], &z0, &z1);
  return cd(z0, z1);
}

// ---------------------------------------------------------------------------
// FFT with FFTW's conventions (unnormalised; FORWARD = e^{-2 pi i nk/N},
// BACKWARD = e^{+2 pi i nk/N}; a 2-D transform is over a row-major n0 x n1
// array). Iterative radix-2 for powers of two, direct DFT otherwise.
// ---------------------------------------------------------------------------
void fft1d_inplace(cd* x, int64_t n, int64_t stride, int sign, std::vector<cd>& tmp) {
  if (n <= 1) return;
  tmp.resize(size_t(n));
  for (int64_t i = 0; i < n; ++i) tmp[size_t(i)] = x[i * stride];
  if ((n & (n - 1)) == 0) {
    // bit reversal
    for (int64_t i = 1, j = 0; i < n; ++i) {
      int64_t bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(tmp[size_t(i)], tmp[size_t(j)]);
    }
    // twiddles exp(sign 2 pi i k / len) for every stage, cached per (n, sign)
    thread_local std::vector<cd> tw_cache;
    thread_local int64_t tw_n = 0;
    thread_local int tw_sign = 0;
    if (tw_n != n || tw_sign != sign) {
      tw_cache.clear();
      for (int64_t len = 2; len <= n; len <<= 1)
        for (int64_t k = 0; k < len / 2; ++k) {
          const double ang = sign * 2.0 * M_PI * double(k) / double(len);
          tw_cache.emplace_back(std::cos(ang), std::sin(ang));
        }
      tw_n = n;
      tw_sign = sign;
    }
    size_t tw_off = 0;
    for (int64_t len = 2; len <= n; len <<= 1, tw_off += size_t(len / 4)) {
      for (int64_t i = 0; i < n; i += len) {
        for (int64_t k = 0; k < len / 2; ++k) {
          const cd w = tw_cache[tw_off + size_t(k)];
          const cd u = tmp[size_t(i + k)];
          const cd v = tmp[size_t(i + k + len / 2)] * w;
          tmp[size_t(i + k)] = u + v;
          tmp[size_t(i + k + len / 2)] = u - v;
        }
      }
    }
    for (int64_t i = 0; i < n; ++i) x[i * stride] = tmp[size_t(i)];
  } else {
    std::vector<cd> out(static_cast<size_t>(n));
    for (int64_t k = 0; k < n; ++k) {
      cd acc(0.0, 0.0);
      for (int64_t j = 0; j < n; ++j) {
        const int64_t e = (j * k) % n;
        const double ang = sign * 2.0 * M_PI * double(e) / double(n);
        acc += tmp[size_t(j)] * cd(std::cos(ang), std::sin(ang));
      }
      out[size_t(k)] = acc;
    }
    for (int64_t i = 0; i < n; ++i) x[i * stride] = out[size_t(i)];
  }
}

// Radix-2 DIT over the row index of a row-major n0 x n1 array (n0 a power
// of two) for all n1 columns at once: every butterfly runs over the
// contiguous columns, so the inner loops vectorise. Per column this is
// exactly fft1d_inplace's arithmetic (same bit reversal, same twiddles in the
// same order), so the results are bit for bit those of the column loop.
void fft_rows_batched(cd* x, int64_t n0, int64_t n1, int sign) {
  for (int64_t i = 1, j = 0; i < n0; ++i) {
    int64_t bit = n0 >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap_ranges(x + i * n1, x + (i + 1) * n1, x + j * n1);
  }
  thread_local std::vector<cd> tw;
  thread_local int64_t tw_n = 0;
  thread_local int tw_sign = 0;
  if (tw_n != n0 || tw_sign != sign) {
    tw.clear();
    for (int64_t len = 2; len <= n0; len <<= 1)
      for (int64_t k = 0; k < len / 2; ++k) {
        const double ang = sign * 2.0 * M_PI * double(k) / double(len);
        tw.emplace_back(std::cos(ang), std::sin(ang));
      }
    tw_n = n0;
    tw_sign = sign;
  }
  size_t off = 0;
  for (int64_t len = 2; len <= n0; len <<= 1, off += size_t(len / 4)) {
    const int64_t h = len / 2;
    for (int64_t i = 0; i < n0; i += len)
      for (int64_t k = 0; k < h; ++k) {
        const cd w = tw[off + size_t(k)];
        cd* __restrict__ u = x + (i + k) * n1;
        cd* __restrict__ v = x + (i + k + h) * n1;
        for (int64_t c = 0; c < n1; ++c) {
          const cd t = v[c] * w;
          v[c] = u[c] - t;
          u[c] = u[c] + t;
        }
      }
  }
}

void transpose(const cd* in, cd* out, int64_t n0, int64_t n1) {
  for (int64_t r = 0; r < n0; ++r)
    for (int64_t c = 0; c < n1; ++c) out[c * n0 + r] = in[r * n1 + c];
}

void fft2d(cd* x, int64_t n0, int64_t n1, int sign) {
  const bool pow2 = n0 > 1 && n1 > 1 && (n0 & (n0 - 1)) == 0 && (n1 & (n1 - 1)) == 0;
  if (pow2) {  // rows (along the column index) through a transpose, then columns
    thread_local std::vector<cd> t;
    t.resize(size_t(n0 * n1));
    transpose(x, t.data(), n0, n1);
    fft_rows_batched(t.data(), n1, n0, sign);
    transpose(t.data(), x, n1, n0);
    fft_rows_batched(x, n0, n1, sign);
    return;
  }
  std::vector<cd> tmp;
  for (int64_t r = 0; r < n0; ++r) fft1d_inplace(x + r * n1, n1, 1, sign, tmp);
  for (int64_t c = 0; c < n1; ++c) fft1d_inplace(x + c, n0, n1, sign, tmp);
}

// ---------------------------------------------------------------------------
// Time-tabulated matrix (NoisyMatrix temporal mode).
// ---------------------------------------------------------------------------
struct TimeTable {
  std::vector<double> times;     // records + DBL_MAX sentinel
  std::vector<cd> vals;          // (nrec+1) x nsite
  std::vector<cd> slopes;        // (nrec+1) x nsite  (dVals)
  int64_t nsite = 0;
};

// Builds times/values/slopes as NoisyMatrix::SetTemporalValue does
// (NoisyMatrix.cpp:164-250): NaN gaps are filled by linear interpolation in
// time (or by the nearest known value at the ends), slopes are forward
// differences, the last record gets slope 0 and a DBL_MAX sentinel.
TimeTable build_time_table(const double* times, const double* vals_ri, int64_t nrec, int64_t nsite) {
  TimeTable tt;
  tt.nsite = nsite;
  tt.times.assign(times, times + nrec);
  std::vector<cd> m(static_cast<size_t>(nrec * nsite));
  for (int64_t i = 0; i < nrec * nsite; ++i) m[size_t(i)] = cd(vals_ri[2 * i], vals_ri[2 * i + 1]);
  for (int64_t s = 0; s < nsite; ++s) {
    for (int64_t pt = 0; pt < nrec; ++pt) {
      cd v = m[size_t(pt * nsite + s)];
      if (std::isnan(v.real()) || std::isnan(v.imag())) {
        cd prev(NAN, NAN);
        int64_t tp;
        for (tp = pt - 1; tp >= 0 && std::isnan(prev.real()); --tp) prev = m[size_t(tp * nsite + s)];
        ++tp;
        cd next(NAN, NAN);
        int64_t tn;
        for (tn = pt + 1; tn < nrec && std::isnan(next.real()); ++tn) next = m[size_t(tn * nsite + s)];
        --tn;
        if (std::isnan(prev.real()) && std::isnan(next.real())) {
          break;
        } else if (std::isnan(next.real())) {
          m[size_t(pt * nsite + s)] = prev;
        } else if (std::isnan(prev.real())) {
          m[size_t(pt * nsite + s)] = next;
        } else {
          m[size_t(pt * nsite + s)] =
              prev + (next - prev) / (tt.times[size_t(tn)] - tt.times[size_t(tp)]) *
                         (tt.times[size_t(pt)] - tt.times[size_t(tp)]);
        }
      }
    }
  }
  tt.vals = m;
  tt.slopes.assign(size_t((nrec + 1) * nsite), cd(0, 0));
  for (int64_t i = 1; i < nrec; ++i)
    for (int64_t s = 0; s < nsite; ++s)
      tt.slopes[size_t((i - 1) * nsite + s)] =
          (m[size_t(i * nsite + s)] - m[size_t((i - 1) * nsite + s)]) / (tt.times[size_t(i)] - tt.times[size_t(i - 1)]);
  tt.vals.resize(size_t((nrec + 1) * nsite));
  for (int64_t s = 0; s < nsite; ++s) tt.vals[size_t(nrec * nsite + s)] = m[size_t((nrec - 1) * nsite + s)];
  tt.times.push_back(std::numeric_limits<double>::max());
  return tt;
}

// GetAtTimeWithSuggestion (NoisyMatrix.cpp:252-265). Returns the segment id;
// writes the interpolated matrix into out.
int64_t time_table_eval(const TimeTable& tt, double t, int64_t hint, cd* out) {
  if (t <= tt.times[0]) {
    for (int64_t s = 0; s < tt.nsite; ++s) out[s] = tt.vals[size_t(s)];
    return 0;
  }
  int64_t id;
  if (hint >= 0 && hint + 1 < int64_t(tt.times.size()) && tt.times[size_t(hint + 1)] > t)
    id = hint;
  else
    id = int64_t(std::lower_bound(tt.times.begin(), tt.times.end(), t) - tt.times.begin()) - 1;
  const cd dtc(t - tt.times[size_t(id)], 0.0);
  for (int64_t s = 0; s < tt.nsite; ++s)
    out[s] = tt.vals[size_t(id * tt.nsite + s)] + dtc * tt.slopes[size_t(id * tt.nsite + s)];
  return id;
}

}  // namespace

extern "C" {

int orc_version(void) { return 1; }

void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox4x32_10(ctr, key, out); }

// Complex normals for sites [0, n) of one trajectory at one step.
void orc_site_normals(uint32_t seed, uint32_t tid, uint32_t step, uint32_t stream, int64_t n, int f32_flavour,
                      double* out_ri) {
  for (int64_t p = 0; p < n; ++p) {
    cd z = site_normal(seed, tid, step, stream, p, n, f32_flavour);
    out_ri[2 * p] = z.real();
    out_ri[2 * p + 1] = z.imag();
  }
}

// Unnormalised 2-D FFT of a row-major n0 x n1 complex array (interleaved).
void orc_fft2d(double* data_ri, int64_t n0, int64_t n1, int sign) {
  fft2d(reinterpret_cast<cd*>(data_ri), n0, n1, sign);
}

// Frame grid of TWMCSystemData (TWMCSystemData.cpp:66-114, :117-134).
// out: [frame_steps, dt_obs, nFramesTot, t_end_adjusted, n_frames_task]
// where n_frames_task = ComputeNFrames(t_start, t_end_adjusted) (+1 when
// store_initial is set, TWMCBaseSolver.cpp:110-111).
void orc_frame_grid(double t_start, double t_end, double timestep, double frames_freq, double frames_period,
                    double n_frames_setting, int store_initial, double* out) {
  double ff = frames_freq;
  if (ff == 0 && frames_period == 0) ff = n_frames_setting / (t_end - t_start);
  else if (ff == 0 && frames_period != 0) ff = 1.0 / frames_period;
  size_t frame_steps = std::max(size_t(1), size_t(std::ceil(1.0 / (ff * timestep))));
  double dt_obs = timestep * double(frame_steps);
  size_t nft = size_t(std::ceil((t_end - t_start) / dt_obs));
  double te = double(nft) * dt_obs;
  if (dt_obs < timestep) { dt_obs = timestep; frame_steps = 1; }
  size_t nf = size_t(std::nearbyint((te - t_start) / dt_obs));
  if (store_initial) nf += 1;
  out[0] = double(frame_steps);
  out[1] = dt_obs;
  out[2] = double(nft);
  out[3] = te;
  out[4] = double(nf);
}

// Square-lattice loop shared by the base and thermo runs (below).
static int square_run(int64_t nx, int64_t ny, double J, double gamma, double dt, double t_start, double t_end,
                      int64_t frame_steps, int64_t n_frames, int store_initial, const double* omega_ri,
                      const double* U_ri, const double* F_ri, int64_t ft_nrec, const double* ft_times,
                      const double* ft_vals_ri, double* beta_ri, int noise_mode, const double* xi_ri, uint32_t seed,
                      uint32_t tid, double* frames_ri, double* work, double* area, double* out_meta,
                      bool split = false) {
  const int64_t n = nx * ny;
  cd* beta = reinterpret_cast<cd*>(beta_ri);
  const cd* omega = reinterpret_cast<const cd*>(omega_ri);
  const cd* U = reinterpret_cast<const cd*>(U_ri);
  std::vector<cd> F(reinterpret_cast<const cd*>(F_ri), reinterpret_cast<const cd*>(F_ri) + n);
  const cd ij(0.0, 1.0);
  // Setup (:65-91)
  std::vector<cd> rsl(static_cast<size_t>(n)), kstep(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) rsl[size_t(i)] = -ij * omega[i] - gamma / 2.0;
  const double f1x = (nx == 1) ? 0.0 : 1.0, f1y = (ny == 1) ? 0.0 : 1.0;
  for (int64_t i = 0; i < nx; ++i)
    for (int64_t j = 0; j < ny; ++j)
      kstep[size_t(i * ny + j)] = -ij * 2.0 * J *
                                  (f1x * std::cos(2.0 * M_PI / double(nx) * double(i)) +
                                   f1y * std::cos(2.0 * M_PI / double(ny) * double(j)));
  // split step: the hopping integrated exactly over dt, exp(kstep dt) = exp(-i 2J c_k dt)
  std::vector<cd> kprop(static_cast<size_t>(split ? n : 0));
  for (int64_t i = 0; split && i < n; ++i) kprop[size_t(i)] = std::exp(kstep[size_t(i)] * dt);
  const double norm = double(n);
  const double dt4 = std::sqrt(gamma * dt / 4.0);
  std::vector<cd> fin(static_cast<size_t>(n)), a(static_cast<size_t>(n)), xi(static_cast<size_t>(n));
  TimeTable tt;
  const bool timedep = ft_nrec > 0;
  if (timedep) tt = build_time_table(ft_times, ft_vals_ri, ft_nrec, n);
  int64_t tcache = 0;
  const bool thermo = work != nullptr;
  std::vector<cd> Fprev(static_cast<size_t>(n));
  std::vector<double> dW(static_cast<size_t>(n), 0.0), dA(static_cast<size_t>(n), 0.0);
  int64_t i_step = 0, i_frame = 0;
  std::mt19937 gen(seed);  // noise_mode 3 (the reference's generator, TWMCBaseSolver.cpp:119)
  if (store_initial && n_frames > 0) {
    if (frames_ri) std::memcpy(frames_ri, beta, sizeof(cd) * size_t(n));
    if (thermo) {
      std::fill(work, work + n, 0.0);
      std::fill(area, area + n, 0.0);
    }
    i_frame = 1;
  }
  double t = t_start;
  cd* frames = reinterpret_cast<cd*>(frames_ri);
  while (t <= t_end) {
    if (timedep) {
      tcache = time_table_eval(tt, t, tcache, F.data());
      if (i_step == 0) Fprev = F;  // dF/dt is 0 on a run's first step
    }
    fin.assign(beta, beta + n);
    fft2d(fin.data(), nx, ny, -1);
    if (split) {  // beta' = IFFT(exp(-i 2J c_k dt) FFT(beta)) / N, then the local step on beta'
      for (int64_t i = 0; i < n; ++i) fin[size_t(i)] = kprop[size_t(i)] * fin[size_t(i)];
      fft2d(fin.data(), nx, ny, +1);
      for (int64_t i = 0; i < n; ++i) beta[i] = fin[size_t(i)] / norm;
      std::fill(fin.begin(), fin.end(), cd(0.0, 0.0));
    } else {
      for (int64_t i = 0; i < n; ++i) fin[size_t(i)] = kstep[size_t(i)] * fin[size_t(i)];
      fft2d(fin.data(), nx, ny, +1);
      for (int64_t i = 0; i < n; ++i) fin[size_t(i)] = fin[size_t(i)] / norm;
    }
    for (int64_t i = 0; i < n; ++i) {
      const double ab2 = beta[i].real() * beta[i].real() + beta[i].imag() * beta[i].imag();
      a[size_t(i)] = ((rsl[size_t(i)] + ij * U[i] * (ab2 - 1.0)) * beta[i] + fin[size_t(i)] + ij * F[size_t(i)]) * dt;
    }
    if (noise_mode == 0) {
      const cd* src = reinterpret_cast<const cd*>(xi_ri) + i_step * n;
      for (int64_t i = 0; i < n; ++i) xi[size_t(i)] = src[i];
    } else if (noise_mode == 3) {
      // randCMat (TWMCBaseSolver.cpp:285-291): the distribution is passed by
      // value, so each step starts a fresh std::normal_distribution on the
      // trajectory's std::mt19937
      std::normal_distribution<double> nd(0.0, 1.0);
      for (int64_t i = 0; i < n; ++i) {
        const double re = nd(gen);
        xi[size_t(i)] = cd(re, nd(gen));
      }
    } else {
      for (int64_t i = 0; i < n; ++i)
        xi[size_t(i)] = site_normal(seed, tid, uint32_t(i_step), kStreamWiener, i, n, noise_mode == 2);
    }
    for (int64_t i = 0; i < n; ++i) beta[i] = beta[i] + a[size_t(i)] + dt4 * xi[size_t(i)];
    if (thermo) {  // TWMCThermoSolver.cpp:230-236 with dF/dt from consecutive steps
      for (int64_t i = 0; i < n; ++i) {
        const double fd = timedep ? (F[size_t(i)].real() - Fprev[size_t(i)].real()) / dt : 0.0;
        const double x = beta[i].real();
        dW[size_t(i)] += (2.0 * dt) * x * fd;
        dA[size_t(i)] += (dt * fd) * (std::norm(beta[i]) - 0.5);
      }
      if (timedep) Fprev = F;
    }
    t += dt;
    ++i_step;
    if ((i_step % frame_steps == 0) && i_frame < n_frames) {
      if (frames) std::memcpy(frames + i_frame * n, beta, sizeof(cd) * size_t(n));
      if (thermo) {
        std::memcpy(work + i_frame * n, dW.data(), sizeof(double) * size_t(n));
        std::memcpy(area + i_frame * n, dA.data(), sizeof(double) * size_t(n));
        std::fill(dW.begin(), dW.end(), 0.0);
        std::fill(dA.begin(), dA.end(), 0.0);
      }
      ++i_frame;
      if (i_frame == n_frames) break;
    }
  }
  out_meta[0] = double(i_frame);
  out_meta[1] = t;
  out_meta[2] = double(i_step);
  return 0;
}

// One trajectory of TWMCBaseSolver::Compute's hot loop (TWMCBaseSolver.cpp:206-280)
// on an nx x ny lattice (row-major, after the 1-D swap of TWMCSystemData).
//   omega, U, F      per-site complex (interleaved), nx*ny each
//   beta             in: initial field; out: field at the end
//   noise_mode       0 = buffer xi[step][site] (interleaved complex normals)
//                    1 = Philox FP64 flavour, 2 = Philox FP32 flavour
//   frames           out: n_frames * nx*ny complex (may be NULL)
//   out_meta         [frames_written, t_final, steps_run]
// Returns 0.
int orc_base_run(int64_t nx, int64_t ny, double J, double gamma, double dt, double t_start, double t_end,
                 int64_t frame_steps, int64_t n_frames, int store_initial, const double* omega_ri,
                 const double* U_ri, const double* F_ri, double* beta_ri, int noise_mode, const double* xi_ri,
                 uint32_t seed, uint32_t tid, double* frames_ri, double* out_meta) {
  return square_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial, omega_ri, U_ri, F_ri,
                    0, nullptr, nullptr, beta_ri, noise_mode, xi_ri, seed, tid, frames_ri, nullptr, nullptr, out_meta);
}

// The same trajectory with the exponential split step of the engine's
// TWMC_INTEGRATOR_SPLIT (an optional mode; the reference integrates the
// hopping by the Euler step above): beta' = IFFT(exp(-i 2J c_k dt) FFT(beta)) / N,
// then a = ((rsl + iU (|beta'|^2 - 1)) beta' + iF) dt and
// beta = beta' + a + sqrt(gamma dt / 4) xi. Arguments as orc_base_run.
int orc_split_run(int64_t nx, int64_t ny, double J, double gamma, double dt, double t_start, double t_end,
                  int64_t frame_steps, int64_t n_frames, int store_initial, const double* omega_ri,
                  const double* U_ri, const double* F_ri, double* beta_ri, int noise_mode, const double* xi_ri,
                  uint32_t seed, uint32_t tid, double* frames_ri, double* out_meta) {
  return square_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial, omega_ri, U_ri, F_ri,
                    0, nullptr, nullptr, beta_ri, noise_mode, xi_ri, seed, tid, frames_ri, nullptr, nullptr, out_meta,
                    true);
}

// The square-lattice loop with an F(t) table (evaluated at the pre-step t, as
// NoisyMatrix::GetAtTimeWithSuggestion in TWMCThermoSolver.cpp:206-210) and
// the drive's work and area per site (TWMCThermoSolver.cpp:230-236):
//   work += 2 dt Re(b) dF/dt,  area += dt dF/dt (|b|^2 - 1/2)
// with b the field after the step and dF/dt = Re(F(t) - F(t - dt)) / dt (0 on
// the first step), summed between saved frames and reset at each save (an
// initial frame has 0). work, area: out, n_frames * nx*ny doubles each.
int orc_thermo_run(int64_t nx, int64_t ny, double J, double gamma, double dt, double t_start, double t_end,
                   int64_t frame_steps, int64_t n_frames, int store_initial, const double* omega_ri,
                   const double* U_ri, const double* F_ri, int64_t ft_nrec, const double* ft_times,
                   const double* ft_vals_ri, double* beta_ri, int noise_mode, const double* xi_ri, uint32_t seed,
                   uint32_t tid, double* frames_ri, double* work, double* area, double* out_meta) {
  if (!work || !area) return -1;
  return square_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, store_initial, omega_ri, U_ri, F_ri,
                    ft_nrec, ft_times, ft_vals_ri, beta_ri, noise_mode, xi_ri, seed, tid, frames_ri, work, area,
                    out_meta);
}

// One trajectory of TWMCLiebSolver::Compute's hot loop (TWMCLiebSolver.cpp:222-294)
// on ncell unit cells (site 3*c + {0:A, 1:B, 2:C}).
//   E, U, F          per-site complex, 3*ncell each (F ignored when ft_nrec > 0)
//   ft_times/ft_vals time table for F(t) (ft_nrec records of 3*ncell complex)
// Returns 0.
int orc_lieb_run(int64_t ncell, int pbc, double J_AB, double J_BC, double detuning, double gamma, double dt,
                 double t_start, double t_end, int64_t frame_steps, int64_t n_frames, int store_initial,
                 const double* E_ri, const double* U_ri, const double* F_ri, int64_t ft_nrec, const double* ft_times,
                 const double* ft_vals_ri, double* beta_ri, int noise_mode, const double* xi_ri, uint32_t seed,
                 uint32_t tid, double* frames_ri, double* out_meta) {
  const int64_t n = 3 * ncell;
  cd* beta = reinterpret_cast<cd*>(beta_ri);
  const cd* E = reinterpret_cast<const cd*>(E_ri);
  const cd* U = reinterpret_cast<const cd*>(U_ri);
  const cd ij(0.0, 1.0);
  std::vector<cd> F(reinterpret_cast<const cd*>(F_ri), reinterpret_cast<const cd*>(F_ri) + n);
  std::vector<cd> rsl(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) rsl[size_t(i)] = -ij * (-E[i] + detuning) - gamma / 2.0;
  // Triplets of TWMCLiebSolver.cpp:54-85; duplicates summed (setFromTriplets).
  struct Trip { int64_t r, c; double v; };
  std::vector<Trip> trips;
  for (int64_t i = 0; i != ncell; ++i) {
    trips.push_back({3 * i, 3 * i + 1, J_AB});
    trips.push_back({3 * i + 1, 3 * i, J_AB});
    trips.push_back({3 * i + 1, 3 * i + 2, J_BC});
    trips.push_back({3 * i + 2, 3 * i + 1, J_BC});
    if (i == ncell - 1) {
      if (pbc) {
        trips.push_back({3 * i + 2, 1, J_BC});
        trips.push_back({1, 3 * i + 2, J_BC});
      }
      break;
    }
    trips.push_back({3 * i + 2, 3 * (i + 1) + 1, J_BC});
    trips.push_back({3 * (i + 1) + 1, 3 * i + 2, J_BC});
  }
  // Row-major CSR with summed duplicates.
  std::vector<std::vector<std::pair<int64_t, double>>> rows(static_cast<size_t>(n));
  for (const Trip& tr : trips) {
    bool merged = false;
    for (auto& e : rows[size_t(tr.r)]) if (e.first == tr.c) { e.second += tr.v; merged = true; }
    if (!merged) rows[size_t(tr.r)].push_back({tr.c, tr.v});
  }
  for (auto& r : rows) std::sort(r.begin(), r.end());
  TimeTable tt;
  const bool timedep = ft_nrec > 0;
  if (timedep) tt = build_time_table(ft_times, ft_vals_ri, ft_nrec, n);
  int64_t tcache = 0;
  const double dt4 = std::sqrt(gamma * dt / 4.0);
  std::vector<cd> bc(static_cast<size_t>(n)), a(static_cast<size_t>(n)), xi(static_cast<size_t>(n));
  int64_t i_step = 0, i_frame = 0;
  std::mt19937 gen(seed);  // noise_mode 3 (the reference's generator, TWMCLiebSolver.cpp:136)
  cd* frames = reinterpret_cast<cd*>(frames_ri);
  if (store_initial && n_frames > 0) {
    if (frames) std::memcpy(frames, beta, sizeof(cd) * size_t(n));
    i_frame = 1;
  }
  double t = t_start;
  while (t <= t_end) {
    if (timedep) tcache = time_table_eval(tt, t, tcache, F.data());
    // beta (row vector) * C
    std::fill(bc.begin(), bc.end(), cd(0, 0));
    for (int64_t r = 0; r < n; ++r)
      for (const auto& e : rows[size_t(r)]) bc[size_t(e.first)] += beta[r] * e.second;
    for (int64_t i = 0; i < n; ++i) {
      const double ab2 = beta[i].real() * beta[i].real() + beta[i].imag() * beta[i].imag();
      a[size_t(i)] = ((rsl[size_t(i)] + ij * U[i] * (ab2 - 1.0)) * beta[i] - ij * bc[size_t(i)] + ij * F[size_t(i)]) * dt;
    }
    if (noise_mode == 0) {
      const cd* src = reinterpret_cast<const cd*>(xi_ri) + i_step * n;
      for (int64_t i = 0; i < n; ++i) xi[size_t(i)] = src[i];
    } else if (noise_mode == 3) {
      // randCMat (TWMCBaseSolver.cpp:285-291): the distribution is passed by
      // value, so each step starts a fresh std::normal_distribution on the
      // trajectory's std::mt19937
      std::normal_distribution<double> nd(0.0, 1.0);
      for (int64_t i = 0; i < n; ++i) {
        const double re = nd(gen);
        xi[size_t(i)] = cd(re, nd(gen));
      }
    } else {
      for (int64_t i = 0; i < n; ++i)
        xi[size_t(i)] = site_normal(seed, tid, uint32_t(i_step), kStreamWiener, i, n, noise_mode == 2);
    }
    for (int64_t i = 0; i < n; ++i) beta[i] = beta[i] + a[size_t(i)] + dt4 * xi[size_t(i)];
    t += dt;
    ++i_step;
    if ((i_step % frame_steps == 0) && i_frame < n_frames) {
      if (frames) std::memcpy(frames + i_frame * n, beta, sizeof(cd) * size_t(n));
      ++i_frame;
      if (i_frame == n_frames) break;
    }
  }
  out_meta[0] = double(i_frame);
  out_meta[1] = t;
  out_meta[2] = double(i_step);
  return 0;
}

// F(t) evaluation as the Lieb loop sees it, for tests of the table logic.
void orc_time_table_eval(const double* times, const double* vals_ri, int64_t nrec, int64_t nsite, const double* ts,
                         int64_t nt, double* out_ri) {
  TimeTable tt = build_time_table(times, vals_ri, nrec, nsite);
  int64_t hint = 0;
  for (int64_t k = 0; k < nt; ++k) hint = time_table_eval(tt, ts[k], hint, reinterpret_cast<cd*>(out_ri) + k * nsite);
}

// Initial field as TWMCBaseSolver::Compute forms it for ReadFromSettings
// (:126-135): beta = beta_init + beta_init_sigma (*) xi, xi from the
// initial-condition stream, FP64 flavour.
// f32_flavour: the Box-Muller flavour of FP32 runs (as for the Wiener noise);
// the combination with beta_init / beta_init_sigma stays in FP64.
void orc_initial_field(int64_t n, const double* binit_ri, const double* bsigma_ri, uint32_t seed, uint32_t tid,
                       double* out_ri, int f32_flavour) {
  const cd* bi = reinterpret_cast<const cd*>(binit_ri);
  const cd* bs = reinterpret_cast<const cd*>(bsigma_ri);
  cd* out = reinterpret_cast<cd*>(out_ri);
  for (int64_t p = 0; p < n; ++p)
    out[p] = bi[p] + bs[p] * site_normal(seed, tid, 0, kStreamInit, p, n, f32_flavour);
}

// Disorder draw of NoisyMatrix::EvaluateNoise (NoisyMatrix.cpp:131-162) on a
// Philox stream: kind 1 = Gaussian (re/im normals scaled by Re/Im of amp),
// kind 2 = Uniform on [0,1) (u = w 2^-32 from words (0,1) / (2,3)).
void orc_disorder(int64_t n, int kind, const double* base_ri, const double* amp_ri, uint32_t seed, uint32_t tid,
                  uint32_t stream, double* out_ri, int f32_flavour) {
  const cd* base = reinterpret_cast<const cd*>(base_ri);
  const cd* amp = reinterpret_cast<const cd*>(amp_ri);
  cd* out = reinterpret_cast<cd*>(out_ri);
  for (int64_t p = 0; p < n; ++p) {
    cd nz(0, 0);
    if (kind == 1) {
      cd z = site_normal(seed, tid, 0, stream, p, n, f32_flavour);
      nz = cd(z.real() * amp[p].real(), z.imag() * amp[p].imag());
    } else if (kind == 2) {
      uint32_t c0; int lane;
      site_counter(p, n, &c0, &lane);
      const uint32_t ctr[4] = {c0, 0u, stream, 0u};
      const uint32_t key[2] = {seed, tid};
      uint32_t w[4];
      philox4x32_10(ctr, key, w);
      nz = cd(double(w[lane]) * 0x1p-32 * amp[p].real(), double(w[lane + 1]) * 0x1p-32 * amp[p].imag());
    }
    out[p] = base[p] + nz;
  }
}

// ---------------------------------------------------------------------------
// Threaded CPU baseline: one trajectory per task on a pool of worker threads
// (the reference's ThreadedTaskProcessor gives each worker thread one solver
// and one trajectory at a time). noise_mode 1: the Philox FP64 stream of the
// GPU solver; 3: the reference's own generator (std::mt19937 seeded per
// trajectory, std::normal_distribution per step). Vacuum-style initial field
// supplied by the caller (same for all trajectories), frames discarded.
// Returns the number of trajectories completed.
// ---------------------------------------------------------------------------
int64_t orc_base_run_batch(int64_t nx, int64_t ny, double J, double gamma, double dt, double t_start, double t_end,
                           int64_t frame_steps, int64_t n_frames, const double* omega_ri, const double* U_ri,
                           const double* F_ri, const double* beta0_ri, int64_t ntraj, uint32_t seed0, int nthreads,
                           double* final_ri, int noise_mode) {
  const int64_t n = nx * ny;
  std::atomic<int64_t> next(0), done(0);
  auto worker = [&]() {
    std::vector<double> beta(static_cast<size_t>(2 * n));
    double meta[3];
    for (;;) {
      const int64_t k = next.fetch_add(1);
      if (k >= ntraj) break;
      std::memcpy(beta.data(), beta0_ri, sizeof(double) * size_t(2 * n));
      orc_base_run(nx, ny, J, gamma, dt, t_start, t_end, frame_steps, n_frames, 0, omega_ri, U_ri, F_ri,
                   beta.data(), noise_mode == 3 ? 3 : 1, nullptr, seed0 + uint32_t(k), uint32_t(k), nullptr, meta);
      if (final_ri) std::memcpy(final_ri + 2 * n * k, beta.data(), sizeof(double) * size_t(2 * n));
      done.fetch_add(1);
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < std::max(1, nthreads); ++i) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
  return done.load();
}

}  // extern "C"
