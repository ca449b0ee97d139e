// twmc_kernels.cuh -- trajectory step kernels of the TWMC engine.
//
// square_fft_kernel: the per-trajectory Euler-Maruyama step of the
//   reference's TWMCBaseSolver (TWMCBaseSolver.cpp:232-266):
//     X = FFT(beta); X *= -i 2J (cos kx + cos ky); h = IFFT(X)/N;
//     a = ((-i omega - gamma/2 + i U (|beta|^2 - 1)) beta + h + i F) dt;
//     beta += a + sqrt(gamma dt / 4) xi
//   Each trajectory's lattice stays in registers for the whole launch
//   (hundreds of steps); the FFT runs as register-resident radix-4/2 DIF
//   passes with shared-memory exchanges between passes (plans from
//   fft_plan.py). HBM is touched only at the start and end of a launch.
// ell_kernel: the same step with the hopping applied in real space from a
//   neighbour list: the reference's Lieb solver (TWMCLiebSolver.cpp:250-280,
//   h = -i (beta C)) including the time-tabulated F(t), and the square
//   lattice for any nx, ny (the FFT operator above is exactly the
//   nearest-neighbour stencil -i J sum_nn beta).
#pragma once

#include <cooperative_groups.h>

#include "twmc_common.cuh"

namespace twmc {

// ------------------------------------------------------------------------
// arguments
// ------------------------------------------------------------------------
struct StepArgs {
  void* state;            // [ntraj][N] complex (R)
  int64_t ntraj;
  int64_t nsteps;         // steps in this launch
  uint32_t step0;         // global index of the first step (Philox counter word 1)
  const uint32_t* seeds;  // [ntraj] Philox key word 0
  const uint32_t* ids;    // [ntraj] Philox key word 1
  // per-site parameters (complex R); NULL = use the scalar value
  const void* rsl;        // -i omega - gamma/2   (Lieb: -i (detuning - E) - gamma/2)
  const void* iU;         // i U
  const void* iF;         // i F
  int64_t par_stride;     // elements between trajectories (0 = shared)
  double rsl_s[2], iU_s[2], iF_s[2];
  double dt, dt4;
  float f_par[6];         // FP32 copies of rsl_s, iU_s, iF_s
  float f_kn;             // -2 ln(2) gamma dt / 4: FP32 Wiener terms come pre-scaled (scaled_normal_pair)
  float f_dt, f_dt4;      // (FP32 kernels read these: a double-to-float conversion
  float f_J;              //  re-done inside a loop runs on the narrow FP64 pipe)
  // noise
  int noise_mode;         // 0 Philox, 1 buffer
  const void* noise;      // [ntraj][noise_steps][N] complex (R)
  int64_t noise_traj_stride;  // = noise_steps * N
  // outputs
  void* nk;               // optional [ntraj][N] R: |FFT(beta)|^2 / N of the final state
  int* status;            // [ntraj]
  // square FFT kernel tables
  const void* tw;         // [M0 + M1] complex R: W_M^j per dimension
  const void* ktab;       // [M0 + M1] R: 2J cos(2 pi k / n) / N per dimension (columns, then rows)
  const void* kfac;       // exponential split step: [N] complex R, (exp(-i 2J c_k dt) - 1) / N at each
                          // position of the forward plan's output; NULL = the Euler step
  int kfac_smem;          // split step: 1 = table copied to shared memory, 0 = read from global (L2)
  int rsl_re_uniform;     // per-site rsl with the same real part (-gamma/2 + Im omega) everywhere, equal
                          // to rsl_s[0]: the fast FFT kernel then reads the imaginary parts only
  // ell kernel
  int tpt;                // threads per trajectory
  int64_t nsites;         // N
  int64_t nx, ny;         // square-stencil geometry
  int hop_kind;           // 0 = neighbour table, 1 = square stencil
  const int* nbr_idx;     // [N][4]
  const void* nbr_w;      // [N][4] complex R (h = sum w beta_idx)
  double J;
  // Lieb couplings for the cell kernel (TWMCLiebSolver.cpp:52-85)
  int lieb_pbc;
  double lieb_jab, lieb_jbc;
  float f_lieb_jab, f_lieb_jbc;
  // F(t) (ell kernel)
  const void* ft_vals;    // [(nrec+1)][N] complex R: i F at the records
  const void* ft_slopes;  // [(nrec+1)][N] complex R: i dF/dt
  const int* ft_id;       // [total steps] segment id per step
  const double* ft_dt;    // [total steps] t - t_id per step
  const float* ft_dt_f;   // the same in FP32 (no per-step conversion on the FP64 pipe)
  int dbuf;               // ell: double-buffered exchange
  // drive thermodynamics (ell kernel, TWMCThermoSolver.cpp:203-236): per-site
  // accumulators [ntraj][N] (R) of work 2 dt Re(beta) dF/dt and area
  // dt dF/dt (|beta|^2 - 1/2), dF/dt = Re(F(t) - F(t - dt)) / dt; NULL = off
  void* work;
  void* area;
};

__device__ __forceinline__ void set_status(int* status, int64_t traj, bool bad) {
  if (bad && status) status[traj] = -4;  // TWMC_ERR_NONFINITE
}

template <typename T>
__device__ __forceinline__ bool finite_c(T v) {
  return isfinite(v.x) && isfinite(v.y);
}

// Local Euler-Maruyama update, the reference's operation order
// (TWMCBaseSolver.cpp:245-253): a = ((rsl + iU (|b|^2-1)) b + h + iF) dt;
// b = b + a + dt4 xi.
template <typename T, typename R>
__device__ __forceinline__ T local_update(T b, T h, T rsl, T iU, T iF, R dt, R dt4, T xi) {
  const R ab2 = b.x * b.x + b.y * b.y;
  const R f = ab2 - R(1);
  const T c = cmake<T>(rsl.x + iU.x * f, rsl.y + iU.y * f);
  T s = cmul(c, b);
  s = cadd(s, h);
  s = cadd(s, iF);
  const T a = cmake<T>(s.x * dt, s.y * dt);
  T nb = cadd(b, a);
  return cmake<T>(nb.x + dt4 * xi.x, nb.y + dt4 * xi.y);
}

// FP32 form of the same update with dt folded in: b' = (A + B |b|^2) b + h' +
// F' + dt4 xi, A = 1 + dt (rsl - iU), B = dt iU, F' = dt iF, h' = dt h (the
// k-space table carries dt). Equal to local_update up to FP32 rounding.
// MADD: the additive terms summed first and the product c b accumulated onto
// them by four multiply-adds (eight FMA-pipe operations per site for the
// product and the sums instead of ten).
template <bool MADD = false, typename T, typename R>
__device__ __forceinline__ T local_update_fused(T b, T hdt, T rsl, T iU, T iF, R dt, R dt4, T xi) {
  const T A = cmake<T>(R(1) + dt * (rsl.x - iU.x), dt * (rsl.y - iU.y));
  const T B = cmake<T>(dt * iU.x, dt * iU.y);
  const R ab2 = b.x * b.x + b.y * b.y;
  const T c = cmake<T>(A.x + B.x * ab2, A.y + B.y * ab2);
  if constexpr (MADD) {
    const T w = cmake<T>(hdt.x + (dt * iF.x + dt4 * xi.x), hdt.y + (dt * iF.y + dt4 * xi.y));
    return cmake<T>(fma(c.x, b.x, fma(-c.y, b.y, w.x)), fma(c.x, b.y, fma(c.y, b.x, w.y)));
  } else {
    T nb = cmul(c, b);
    nb = cmake<T>(nb.x + hdt.x + dt * iF.x, nb.y + hdt.y + dt * iF.y);
    return cmake<T>(nb.x + dt4 * xi.x, nb.y + dt4 * xi.y);
  }
}

// Wiener term of one Philox word pair in the form the updates add it: FP32
// kernels get sqrt(gamma dt / 4) xi directly from the scaled Box-Muller and
// add it with unit scale (Wiener<float>::scale = 1); FP64 kernels get xi and
// scale it by dt4 in the update. Deterministic-noise buffer values take the
// same form.
template <typename R> struct Wiener;
template <> struct Wiener<float> {
  static __device__ __forceinline__ float2 term(uint32_t a, uint32_t b, const StepArgs& s) {
    return scaled_normal_pair(a, b, s.f_kn);
  }
  static __device__ __forceinline__ float2 buffer(float2 xi, float dt4) { return make_float2(dt4 * xi.x, dt4 * xi.y); }
  static __device__ __forceinline__ float scale(float) { return 1.0f; }
};
template <> struct Wiener<double> {
  static __device__ __forceinline__ double2 term(uint32_t a, uint32_t b, const StepArgs&) {
    return normal_pair(a, b, 0.0);
  }
  static __device__ __forceinline__ double2 buffer(double2 xi, double) { return xi; }
  static __device__ __forceinline__ double scale(double dt4) { return dt4; }
};

// ------------------------------------------------------------------------
// compile-time twiddles: (cos, sin)(2 pi k / M) in double by an exact octant
// reduction of the integer k and Taylor series on |x| <= pi / 4
// ------------------------------------------------------------------------
struct CosSin { double c, s; };
constexpr double kPiD = 3.14159265358979323846264338327950288;
constexpr double taylor_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int n = 1; n < 12; ++n) { term *= -x2 / double((2 * n) * (2 * n + 1)); sum += term; }
  return sum;
}
constexpr double taylor_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int n = 1; n < 12; ++n) { term *= -x2 / double((2 * n - 1) * (2 * n)); sum += term; }
  return sum;
}
constexpr CosSin cossin2pi(int k, int M) {
  k %= M;
  if (k < 0) k += M;
  if (2 * k > M) {  // (pi, 2 pi): the conjugate of 2 pi (M - k) / M
    const CosSin r = cossin2pi(M - k, M);
    return CosSin{r.c, -r.s};
  }
  if (4 * k > M) {  // (pi / 2, pi]: pi - theta
    const CosSin r = cossin2pi(M - 2 * k, 2 * M);  // angle pi - 2 pi k / M = 2 pi (M - 2k) / (2M)
    return CosSin{-r.c, r.s};
  }
  if (8 * k > M) {  // (pi / 4, pi / 2]: pi / 2 - theta
    const double x = kPiD * double(M - 4 * k) / double(2 * M);
    return CosSin{taylor_sin(x), taylor_cos(x)};
  }
  const double x = 2.0 * kPiD * double(k) / double(M);
  return CosSin{taylor_cos(x), taylor_sin(x)};
}

// x * W_M^E (W = e^{-2 pi i / M}) or x * conj(W_M^E) for a compile-time E:
// quarter turns as swaps and sign changes, other twiddles as immediates.
template <typename T, int M, int E, bool CONJ>
__device__ __forceinline__ T cmul_tw(T x) {
  using R = decltype(T::x);
  constexpr int e = ((E % M) + M) % M;
  if constexpr (e == 0) {
    return x;
  } else if constexpr (2 * e == M) {
    return cmake<T>(-x.x, -x.y);
  } else if constexpr (4 * e == M) {  // W = -i
    return CONJ ? cmake<T>(-x.y, x.x) : cmake<T>(x.y, -x.x);
  } else if constexpr (4 * e == 3 * M) {  // W = +i
    return CONJ ? cmake<T>(x.y, -x.x) : cmake<T>(-x.y, x.x);
  } else {
    constexpr CosSin w = cossin2pi(e, M);
    const T wv = cmake<T>(R(w.c), R(-w.s));
    return CONJ ? cmulc(x, wv) : cmul(x, wv);
  }
}

// Whether W_M^E is a general twiddle (not 1, -1 or a quarter turn).
constexpr bool tw_is_general(int M, int E) {
  const int e = ((E % M) + M) % M;
  return e != 0 && 2 * e != M && 4 * e != M && 4 * e != 3 * M;
}
template <int M, int E>
constexpr bool tw_general() {
  return tw_is_general(M, E);
}
// acc + y * W_M^E (or conj(W_M^E)) for a general compile-time twiddle: four
// multiply-adds with immediates.
template <typename T, int M, int E, bool CONJ>
__device__ __forceinline__ T cmla_tw(T acc, T y) {
  using R = decltype(T::x);
  constexpr CosSin w = cossin2pi(((E % M) + M) % M, M);
  return CONJ ? cmlac(acc, y, cmake<T>(R(w.c), R(-w.s))) : cmlac(acc, y, cmake<T>(R(w.c), R(w.s)));
}

// ------------------------------------------------------------------------
// compile-time plan helpers (P = generated Plan_bx_by)
// ------------------------------------------------------------------------
template <class P> struct PlanInfo {
  static constexpr int E = 1 << P::e;
  static constexpr int N = 1 << P::nbits;
  static constexpr int TPT = N / E;
  static constexpr int M0 = 1 << P::m[0];
  static constexpr int M1 = 1 << P::m[1];
  // twiddle entries read: exponents below 3M/4 (radix-4) and M/2 (radix-2)
  static constexpr int TW0 = M0 >= 4 ? 3 * M0 / 4 : 1;
  static constexpr int TW1 = M1 >= 4 ? 3 * M1 / 4 : 1;
  static constexpr int slot_bit(int k, int g) {
    for (int j = 0; j < P::e; ++j) if (P::reg[k][j] == g) return j;
    return -1;
  }
  static constexpr int pos_reg(int k, int s) {
    int p = 0;
    for (int j = 0; j < P::e; ++j) p |= ((s >> j) & 1) << P::reg[k][j];
    return p;
  }
  static constexpr uint32_t thr_mask(int k) {
    uint32_t m = 0;
    for (int i = 0; i < P::nthr; ++i) m |= 1u << P::thr[k][i];
    return P::nthr ? m : 0u;
  }
  static constexpr int bitrev(int v, int nb) {
    int r = 0;
    for (int i = 0; i < nb; ++i) r |= ((v >> i) & 1) << (nb - 1 - i);
    return r;
  }
  // k-space indices of position p after the forward plan (bit reversal per dim)
  static constexpr int ky_of(int p) { return bitrev(p & ((1 << P::by) - 1), P::by); }
  static constexpr int kx_of(int p) { return P::bx ? bitrev(p >> P::by, P::bx) : 0; }
  static constexpr bool last_has_row_reg() {
    for (int j = 0; j < P::e; ++j) if (P::reg[P::npass - 1][j] >= P::by) return true;
    return false;
  }
  // slot index with zero bits inserted at positions j0 (and j1 if >= 0)
  static constexpr int insert0(int q, int j0, int j1) {
    int s = 0, src = 0;
    for (int j = 0; j < P::e; ++j) {
      if (j == j0 || j == j1) continue;
      s |= ((q >> src) & 1) << j;
      ++src;
    }
    return s;
  }
};

// Register slots of the twiddles that depend on thread bits (stages whose
// exponent mixes thread and register bits): one set per distinct register
// part of the exponent, three values (W^e, W^2e, W^3e) for a radix-4 stage
// and one for radix-2. The set is the same for the forward and the inverse
// transform (conjugated there), and loop-invariant per thread, so a kernel
// with registers to spare loads it once per launch.
template <class P> struct TwSlots {
  using I = PlanInfo<P>;
  static constexpr uint32_t lowmask(int K, int SI) {
    return ((1u << P::st[K][SI][1]) - 1u) << P::lo[P::st[K][SI][0]];
  }
  static constexpr bool thr_low(int K, int SI) { return (I::thr_mask(K) & lowmask(K, SI)) != 0u; }
  static constexpr int ngroups(int K, int SI) { return P::st[K][SI][2] == 2 ? I::E / 4 : I::E / 2; }
  static constexpr int low_r(int K, int SI, int Q) {
    const int dim = P::st[K][SI][0], t = P::st[K][SI][1], lo = P::lo[dim];
    const int j0 = I::slot_bit(K, lo + t);
    const int j1 = P::st[K][SI][2] == 2 ? I::slot_bit(K, lo + t + 1) : -1;
    const int s0 = I::insert0(Q, j0, j1);
    return int((uint32_t(I::pos_reg(K, s0)) & lowmask(K, SI)) >> lo);
  }
  // index of group Q's register part among the distinct ones of its stage
  static constexpr int distinct(int K, int SI, int Q) {
    int d = 0;
    for (int q = 0; q < Q; ++q) {
      bool seen = false;
      for (int r = 0; r < q; ++r) seen = seen || low_r(K, SI, r) == low_r(K, SI, q);
      if (seen) continue;
      if (low_r(K, SI, q) == low_r(K, SI, Q)) return d;
      ++d;
    }
    return d;
  }
  static constexpr int ndistinct(int K, int SI) {
    int d = 0;
    for (int q = 0; q < ngroups(K, SI); ++q) {
      bool seen = false;
      for (int r = 0; r < q; ++r) seen = seen || low_r(K, SI, r) == low_r(K, SI, q);
      if (!seen) ++d;
    }
    return d;
  }
  static constexpr int per(int K, int SI) { return P::st[K][SI][2] == 2 ? 3 : 1; }
  static constexpr int base(int K, int SI) {
    int b = 0;
    for (int k = 0; k < P::npass; ++k)
      for (int si = 0; si < P::nst[k]; ++si) {
        if (k == K && si == SI) return b;
        if (thr_low(k, si)) b += ndistinct(k, si) * per(k, si);
      }
    return b;
  }
  static constexpr int total() { return base(P::npass, 0); }
};

// Plans whose single-system FP32 kernel holds the thread-dependent twiddles
// in registers for the whole launch (chains of 1024 sites and more).
template <class P>
constexpr bool plan_reg_twiddles() {
  return P::bx == 0 && P::nbits >= 10 && TwSlots<P>::total() > 0;
}

// Padded position of the CTA-flat element index: one pad slot after every 16
// elements. For indices with disjoint bits pad(a | b) = pad(a) + pad(b), so
// the thread part is a register and the register-slot part an immediate.
__host__ __device__ constexpr int pad16(int p) { return p + (p >> 4); }

// One DIF stage (forward) or its adjoint (inverse) of pass K, stage SI.
template <class P, int K, int SI, bool INV, bool HT, typename T>
__device__ __forceinline__ void fft_stage(T (&x)[PlanInfo<P>::E], const T* __restrict__ tw0,
                                          const T* __restrict__ tw1, int pos_thr, const T* twr) {
  using I = PlanInfo<P>;
  constexpr int dim = P::st[K][SI][0];
  constexpr int t = P::st[K][SI][1];
  constexpr int rb = P::st[K][SI][2];
  constexpr int lo = P::lo[dim];
  constexpr int m = P::m[dim];
  constexpr uint32_t lowmask = ((1u << t) - 1u) << lo;  // global bits of local bits < t
  constexpr bool thr_low = (I::thr_mask(K) & lowmask) != 0u;
  const T* __restrict__ tw = dim ? tw1 : tw0;
  const int low_t = thr_low ? int((uint32_t(pos_thr) & lowmask) >> lo) : 0;
  if constexpr (rb == 2) {
    constexpr int j0 = I::slot_bit(K, lo + t);
    constexpr int j1 = I::slot_bit(K, lo + t + 1);
    static_assert(j0 >= 0 && j1 >= 0, "stage bits must be register bits");
    constexpr int sh = m - t - 2;
    static_for<I::E / 4>([&](auto Q) {
      constexpr int s0 = I::insert0(decltype(Q)::value, j0, j1);
      constexpr int s1 = s0 | (1 << j0), s2 = s0 | (1 << j1), s3 = s0 | (1 << j0) | (1 << j1);
      constexpr int low_r = int((uint32_t(I::pos_reg(K, s0)) & lowmask) >> lo);
      [[maybe_unused]] constexpr bool trivial = !thr_low && low_r == 0;
      // twiddles W_M^{j e1}: from the table when thread bits enter the
      // exponent, compile-time constants (immediates, exact quarter turns)
      // when only register bits do
      [[maybe_unused]] constexpr int MM = 1 << m, ec = low_r << sh;
      [[maybe_unused]] T w1, w2, w3;
      if constexpr (thr_low && HT) {  // the launch-invariant set held in registers
        constexpr int slot = TwSlots<P>::base(K, SI) + 3 * TwSlots<P>::distinct(K, SI, decltype(Q)::value);
        w1 = twr[slot];
        w2 = twr[slot + 1];
        w3 = twr[slot + 2];
      } else if constexpr (thr_low) {
        const int e1 = (low_r + low_t) << sh;
        w1 = tw[e1];
        w2 = tw[2 * e1];
        w3 = tw[3 * e1];
      }
      if constexpr (!INV) {
        const T A = cadd(x[s0], x[s2]), B = cadd(x[s1], x[s3]);
        const T C = csub(x[s0], x[s2]), D = csub(x[s1], x[s3]);
        T y0 = cadd(A, B), y1 = csub(A, B);
        T y2 = cmake<T>(C.x + D.y, C.y - D.x);  // C - iD
        T y3 = cmake<T>(C.x - D.y, C.y + D.x);  // C + iD
        if constexpr (thr_low) {
          y1 = cmul(y1, w2);
          y2 = cmul(y2, w1);
          y3 = cmul(y3, w3);
        } else if constexpr (!trivial) {
          y1 = cmul_tw<T, MM, 2 * ec, false>(y1);
          y2 = cmul_tw<T, MM, ec, false>(y2);
          y3 = cmul_tw<T, MM, 3 * ec, false>(y3);
        }
        x[s0] = y0; x[s1] = y1; x[s2] = y2; x[s3] = y3;
      } else if constexpr (sizeof(decltype(T::x)) == 4) {
        // FP32: each general twiddle product is accumulated onto its partner
        // by multiply-adds (A = y0 + u, C = p + q) and the differences taken
        // as 2 y0 - A, 2 p - C: 24 FMA-pipe operations per butterfly with
        // three general twiddles instead of 28 (measured on GB300: 64x64
        // 2.14e11 -> 2.19e11, 32x32 2.23e11 -> 2.30e11 site-updates/s)
        const T y0 = x[s0];
        T A, B, C, pq, p;
        if constexpr (thr_low) {
          A = cmlac(y0, x[s1], w2);
          B = ctwice_minus(y0, A);
          p = cmulc(x[s2], w1);
          C = cmlac(p, x[s3], w3);
          pq = ctwice_minus(p, C);
        } else {
          if constexpr (!trivial && tw_general<MM, 2 * ec>()) {
            A = cmla_tw<T, MM, 2 * ec, true>(y0, x[s1]);
            B = ctwice_minus(y0, A);
          } else {
            const T u = trivial ? x[s1] : cmul_tw<T, MM, 2 * ec, true>(x[s1]);
            A = cadd(y0, u);
            B = csub(y0, u);
          }
          p = trivial ? x[s2] : cmul_tw<T, MM, ec, true>(x[s2]);
          if constexpr (!trivial && tw_general<MM, 3 * ec>()) {
            C = cmla_tw<T, MM, 3 * ec, true>(p, x[s3]);
            pq = ctwice_minus(p, C);
          } else {
            const T q = trivial ? x[s3] : cmul_tw<T, MM, 3 * ec, true>(x[s3]);
            C = cadd(p, q);
            pq = csub(p, q);
          }
        }
        const T D = cmake<T>(-pq.y, pq.x);  // i (p - q)
        x[s0] = cadd(A, C); x[s2] = csub(A, C); x[s1] = cadd(B, D); x[s3] = csub(B, D);
      } else {
        T u = x[s1], p = x[s2], q = x[s3];
        if constexpr (thr_low) {
          u = cmulc(u, w2);
          p = cmulc(p, w1);
          q = cmulc(q, w3);
        } else if constexpr (!trivial) {
          u = cmul_tw<T, MM, 2 * ec, true>(u);
          p = cmul_tw<T, MM, ec, true>(p);
          q = cmul_tw<T, MM, 3 * ec, true>(q);
        }
        const T A = cadd(x[s0], u), B = csub(x[s0], u);
        const T C = cadd(p, q);
        const T pq = csub(p, q);
        const T D = cmake<T>(-pq.y, pq.x);  // i (p - q)
        x[s0] = cadd(A, C); x[s2] = csub(A, C); x[s1] = cadd(B, D); x[s3] = csub(B, D);
      }
    });
  } else {
    constexpr int j0 = I::slot_bit(K, lo + t);
    static_assert(j0 >= 0, "stage bit must be a register bit");
    constexpr int sh = m - t - 1;
    static_for<I::E / 2>([&](auto Q) {
      constexpr int s0 = I::insert0(decltype(Q)::value, j0, -1);
      constexpr int s1 = s0 | (1 << j0);
      constexpr int low_r = int((uint32_t(I::pos_reg(K, s0)) & lowmask) >> lo);
      [[maybe_unused]] constexpr bool trivial = !thr_low && low_r == 0;
      [[maybe_unused]] constexpr int MM = 1 << m, ec = low_r << sh;
      [[maybe_unused]] T w;
      if constexpr (thr_low && HT) w = twr[TwSlots<P>::base(K, SI) + TwSlots<P>::distinct(K, SI, decltype(Q)::value)];
      else if constexpr (thr_low) w = tw[(low_r + low_t) << sh];
      if constexpr (!INV) {
        T y0 = cadd(x[s0], x[s1]), y1 = csub(x[s0], x[s1]);
        if constexpr (thr_low) y1 = cmul(y1, w);
        else if constexpr (!trivial) y1 = cmul_tw<T, MM, ec, false>(y1);
        x[s0] = y0; x[s1] = y1;
      } else if constexpr (sizeof(decltype(T::x)) == 4 && (thr_low || (!trivial && tw_general<MM, ec>()))) {
        const T y0 = x[s0];
        T A;
        if constexpr (thr_low) A = cmlac(y0, x[s1], w);
        else A = cmla_tw<T, MM, ec, true>(y0, x[s1]);
        x[s0] = A; x[s1] = ctwice_minus(y0, A);
      } else {
        T u = x[s1];
        if constexpr (thr_low) u = cmulc(u, w);
        else if constexpr (!trivial) u = cmul_tw<T, MM, ec, true>(u);
        const T y0 = x[s0];
        x[s0] = cadd(y0, u); x[s1] = csub(y0, u);
      }
    });
  }
}

// The twiddle that forward radix-4 stage SI of pass K puts on register slot
// s: W_M^(mult (low_r + low_t) 2^sh), mult = 0, 2, 1, 3 for the slot's stage
// bits 00, 01, 10, 11 (outputs y0 .. y3), low_r its register part, low_t the
// thread part of the exponent.
template <class P, int K, int SI> struct StageTw {
  using I = PlanInfo<P>;
  static constexpr int dim = P::st[K][SI][0], t = P::st[K][SI][1], lo = P::lo[dim], m = P::m[dim];
  static constexpr uint32_t lowmask = ((1u << t) - 1u) << lo;
  static constexpr bool thr_low = (I::thr_mask(K) & lowmask) != 0u;
  static constexpr int sh = m - t - 2, MM = 1 << m;
  static constexpr int j0 = I::slot_bit(K, lo + t), j1 = I::slot_bit(K, lo + t + 1);
  static constexpr int mult(int s) {
    const int b = ((s >> j0) & 1) | (((s >> j1) & 1) << 1);
    return b == 0 ? 0 : b == 1 ? 2 : b == 2 ? 1 : 3;
  }
  static constexpr int low_r(int s) {
    return int((uint32_t(I::pos_reg(K, s & ~((1 << j0) | (1 << j1)))) & lowmask) >> lo);
  }
  // the stage's butterfly group of slot s (inverse of PlanInfo::insert0)
  static constexpr int group(int s) {
    int q = 0, d = 0;
    for (int j = 0; j < P::e; ++j) {
      if (j == j0 || j == j1) continue;
      q |= ((s >> j) & 1) << d;
      ++d;
    }
    return q;
  }
  static constexpr int ec(int s) { return mult(s) * (low_r(s) << sh); }  // exponent when !thr_low
  static constexpr bool none(int s) { return mult(s) == 0 || (!thr_low && ((ec(s) % MM) + MM) % MM == 0); }
  static constexpr bool general(int s) { return !none(s) && (thr_low || tw_is_general(MM, ec(s))); }
};

// Forward pass of two radix-4 stages with the first stage's output twiddles
// deferred to the second stage's inputs (FP32): in each second-stage
// butterfly the sums x0 + x2, x1 + x3 of twiddled inputs are one product and
// one multiply-accumulate, the differences 2 t - sum -- 20 FMA-pipe
// operations instead of 24 per butterfly whose inputs carry general
// twiddles. The same transform as fft_pass up to rounding, so the inverse is
// unchanged.
template <class P, int K, bool HT, typename T>
__device__ __forceinline__ void fft_pass_fwd_deferred(T (&x)[PlanInfo<P>::E], const T* __restrict__ tw0,
                                                      const T* __restrict__ tw1, int pos_thr, const T* twr) {
  using I = PlanInfo<P>;
  using S1 = StageTw<P, K, 0>;
  // first stage: butterflies only
  static_for<I::E / 4>([&](auto Q) {
    constexpr int s0 = I::insert0(decltype(Q)::value, S1::j0, S1::j1);
    constexpr int s1 = s0 | (1 << S1::j0), s2 = s0 | (1 << S1::j1), s3 = s0 | (1 << S1::j0) | (1 << S1::j1);
    const T A = cadd(x[s0], x[s2]), B = cadd(x[s1], x[s3]);
    const T C = csub(x[s0], x[s2]), D = csub(x[s1], x[s3]);
    x[s0] = cadd(A, B);
    x[s1] = csub(A, B);
    x[s2] = cmake<T>(C.x + D.y, C.y - D.x);  // C - iD
    x[s3] = cmake<T>(C.x - D.y, C.y + D.x);  // C + iD
  });
  const T* __restrict__ tw = S1::dim ? tw1 : tw0;
  const int low_t = S1::thr_low ? int((uint32_t(pos_thr) & S1::lowmask) >> S1::lo) : 0;
  // the deferred twiddle of slot s (thread-dependent: table or register set)
  auto wrt = [&](auto SS) -> T {
    constexpr int s = decltype(SS)::value;
    if constexpr (HT) {
      constexpr int slot = TwSlots<P>::base(K, 0) + 3 * TwSlots<P>::distinct(K, 0, S1::group(s));
      constexpr int m = S1::mult(s);
      return twr[slot + (m == 1 ? 0 : m == 2 ? 1 : 2)];
    } else {
      return tw[S1::mult(s) * ((S1::low_r(s) + low_t) << S1::sh)];
    }
  };
  // z * w(s)
  auto dmul = [&](auto SS, T z) -> T {
    constexpr int s = decltype(SS)::value;
    if constexpr (S1::none(s)) return z;
    else if constexpr (S1::thr_low) return cmul(z, wrt(SS));
    else return cmul_tw<T, S1::MM, S1::ec(s), false>(z);
  };
  // acc + z * w(s) for a general twiddle
  auto dmla = [&](auto SS, T acc, T z) -> T {
    constexpr int s = decltype(SS)::value;
    if constexpr (S1::thr_low) {
      const T w = wrt(SS);
      return cmlac(acc, z, cmake<T>(w.x, -w.y));
    } else {
      return cmla_tw<T, S1::MM, S1::ec(s), false>(acc, z);
    }
  };
  // second stage: twiddled inputs, then its own output twiddles
  constexpr int SI = 1;
  using S2 = StageTw<P, K, SI>;
  const int low_t2 = S2::thr_low ? int((uint32_t(pos_thr) & S2::lowmask) >> S2::lo) : 0;
  const T* __restrict__ tw2 = S2::dim ? tw1 : tw0;
  static_for<I::E / 4>([&](auto Q) {
    constexpr int q = decltype(Q)::value;
    constexpr int s0 = I::insert0(q, S2::j0, S2::j1);
    constexpr int s1 = s0 | (1 << S2::j0), s2 = s0 | (1 << S2::j1), s3 = s0 | (1 << S2::j0) | (1 << S2::j1);
    using C0 = std::integral_constant<int, s0>;
    using C1 = std::integral_constant<int, s1>;
    using C2 = std::integral_constant<int, s2>;
    using C3 = std::integral_constant<int, s3>;
    T A, B, C, D;
    const T t0 = dmul(C0{}, x[s0]);
    if constexpr (S1::general(s2)) {
      A = dmla(C2{}, t0, x[s2]);
      C = ctwice_minus(t0, A);
    } else {
      const T u = dmul(C2{}, x[s2]);
      A = cadd(t0, u);
      C = csub(t0, u);
    }
    const T t1 = dmul(C1{}, x[s1]);
    if constexpr (S1::general(s3)) {
      B = dmla(C3{}, t1, x[s3]);
      D = ctwice_minus(t1, B);
    } else {
      const T u = dmul(C3{}, x[s3]);
      B = cadd(t1, u);
      D = csub(t1, u);
    }
    T y0 = cadd(A, B), y1 = csub(A, B);
    T y2 = cmake<T>(C.x + D.y, C.y - D.x);  // C - iD
    T y3 = cmake<T>(C.x - D.y, C.y + D.x);  // C + iD
    constexpr int low_r = int((uint32_t(I::pos_reg(K, s0)) & S2::lowmask) >> S2::lo);
    constexpr int ec = low_r << S2::sh;
    if constexpr (S2::thr_low) {
      T w1, w2, w3;
      if constexpr (HT) {
        constexpr int slot = TwSlots<P>::base(K, SI) + 3 * TwSlots<P>::distinct(K, SI, q);
        w1 = twr[slot];
        w2 = twr[slot + 1];
        w3 = twr[slot + 2];
      } else {
        const int e1 = (low_r + low_t2) << S2::sh;
        w1 = tw2[e1];
        w2 = tw2[2 * e1];
        w3 = tw2[3 * e1];
      }
      y1 = cmul(y1, w2);
      y2 = cmul(y2, w1);
      y3 = cmul(y3, w3);
    } else if constexpr (low_r != 0) {
      y1 = cmul_tw<T, S2::MM, 2 * ec, false>(y1);
      y2 = cmul_tw<T, S2::MM, ec, false>(y2);
      y3 = cmul_tw<T, S2::MM, 3 * ec, false>(y3);
    }
    x[s0] = y0; x[s1] = y1; x[s2] = y2; x[s3] = y3;
  });
}

// DEF: the single-system kernel (no register cap) takes the deferred
// first-stage twiddles (fft_pass_fwd_deferred) on the plans below 4096 sites;
// measured on GB300: 1x2048 1.99e11 -> 2.05e11, 1x1024 2.08e11 -> 2.11e11,
// 1x256 2.91e11 -> 2.95e11, 16x16 3.33e11 -> 3.36e11 site-updates/s, while
// 64x64 lost 2 % (251 registers against 240); the batch kernel, at its
// 128-register cap, keeps the plain passes.
template <class P, int K, bool INV, bool HT = false, bool DEF = false, typename T>
__device__ __forceinline__ void fft_pass(T (&x)[PlanInfo<P>::E], const T* tw0, const T* tw1, int pos_thr,
                                         const T* twr = nullptr) {
  constexpr int ns = P::nst[K];
  constexpr bool deferred = DEF && !INV && sizeof(decltype(T::x)) == 4 && P::nbits < 12 && ns == 2 &&
                            P::st[K][0][2] == 2 && P::st[K][1][2] == 2 && P::st[K][0][1] > 0;
  if constexpr (deferred) {
    fft_pass_fwd_deferred<P, K, HT>(x, tw0, tw1, pos_thr, twr);
  } else {
    static_for<ns>([&](auto S) {
      constexpr int si = INV ? (ns - 1 - decltype(S)::value) : decltype(S)::value;
      fft_stage<P, K, si, INV, HT>(x, tw0, tw1, pos_thr, twr);
    });
  }
}

// The twiddle register set of TwSlots for this thread (table loads, once).
template <class P, typename T>
__device__ __forceinline__ void load_twiddle_set(T* twr, const T* tw0, const T* tw1, const int* pos_thr) {
  using S = TwSlots<P>;
  static_for<P::npass>([&](auto KK) {
    constexpr int K = decltype(KK)::value;
    static_for<P::nst[K]>([&](auto SS) {
      constexpr int SI = decltype(SS)::value;
      if constexpr (S::thr_low(K, SI)) {
        constexpr int dim = P::st[K][SI][0], t = P::st[K][SI][1], lo = P::lo[dim], m = P::m[dim];
        constexpr int sh = P::st[K][SI][2] == 2 ? m - t - 2 : m - t - 1;
        const T* tw = dim ? tw1 : tw0;
        const int low_t = int((uint32_t(pos_thr[K]) & S::lowmask(K, SI)) >> lo);
        static_for<S::ngroups(K, SI)>([&](auto QQ) {
          constexpr int Q = decltype(QQ)::value;
          constexpr int d = S::distinct(K, SI, Q);
          constexpr bool first = [] {
            for (int q = 0; q < Q; ++q) if (S::distinct(K, SI, q) == S::distinct(K, SI, Q)) return false;
            return true;
          }();
          if constexpr (first) {
            const int e1 = (S::low_r(K, SI, Q) + low_t) << sh;
            if constexpr (S::per(K, SI) == 3) {
              twr[S::base(K, SI) + 3 * d] = tw[e1];
              twr[S::base(K, SI) + 3 * d + 1] = tw[2 * e1];
              twr[S::base(K, SI) + 3 * d + 2] = tw[3 * e1];
            } else {
              twr[S::base(K, SI) + d] = tw[e1];
            }
          }
        });
      }
    });
  });
}

// Exchange from layout of pass KA to layout of pass KB through shared memory.
template <class P, int KA, int KB, bool SYNC_WARP, typename T>
__device__ __forceinline__ void fft_exchange(T (&x)[PlanInfo<P>::E], T* __restrict__ buf, int base_a,
                                             int base_b) {
  using I = PlanInfo<P>;
  static_for<I::E>([&](auto S) {
    constexpr int s = decltype(S)::value;
    constexpr int off = pad16(I::pos_reg(KA, s));
    buf[base_a + off] = x[s];
  });
  if constexpr (SYNC_WARP) __syncwarp(); else __syncthreads();
  static_for<I::E>([&](auto S) {
    constexpr int s = decltype(S)::value;
    constexpr int off = pad16(I::pos_reg(KB, s));
    x[s] = buf[base_b + off];
  });
}

// BETA_SMEM: FP32 threads keep their sites in shared-memory slices during the
// step (registers for the FFT). REG_SMALL: plans of fewer than 4096 sites keep
// them in registers instead -- the single-system kernel, one CTA per SM,
// measured 1.64x (1x32), 1.20x (1x64), 1.06x (1x1024) faster that way and
// 6 % slower on the 4096-site plans; the batch kernel, under its own
// register cap, keeps the slices.
template <class P, int CTA, typename R, bool REG_SMALL = false>
struct SquareCfg {
  static constexpr bool BETA_SMEM = sizeof(R) == 4 && !(REG_SMALL && PlanInfo<P>::N < 4096);
  using I = PlanInfo<P>;
  static constexpr int E = I::E, N = I::N, TPT = I::TPT;
  static constexpr int TPC = CTA / TPT;  // trajectories per CTA
  static constexpr int XSZ = TPC * N + (TPC * N) / 16;  // one padded exchange buffer
  static constexpr bool SYNC_WARP = TPT <= 32;
  static constexpr size_t smem_bytes() {
    using T = c2_t<R>;
    return sizeof(T) * (size_t(I::TW0 + I::TW1) + 2 * size_t(XSZ) + (BETA_SMEM ? size_t(TPC) * N : 0)) +
           sizeof(R) * size_t(I::M0 + I::M1);
  }
  // the split-step factor table behind the rest (16-byte aligned, padded
  // like the exchange buffers), present only when a launch passes kfac
  static constexpr size_t kfac_offset() { return (smem_bytes() + 15) & ~size_t(15); }
  static constexpr size_t smem_bytes_split() { return kfac_offset() + sizeof(c2_t<R>) * size_t(N + N / 16); }
};

// One square-lattice trajectory group (TPC trajectories) for a.nsteps steps:
// the body of square_fft_kernel, shared with the heterogeneous-batch kernel.
// Shared memory: twiddles | 2 padded exchange buffers | state slices (FP32) |
// separable k-space table. FAST: Philox noise and scalar U, F (per-site
// omega allowed) compiled in instead of tested per site.
template <typename R, class P, int CTA, bool FAST = false, bool REG_SMALL = false, bool SPLIT = false>
struct SquareGroup {
  using T = c2_t<R>;
  using I = PlanInfo<P>;
  using Cfg = SquareCfg<P, CTA, R, REG_SMALL>;
  static constexpr int E = I::E, N = I::N, TPT = I::TPT, TPC = Cfg::TPC;
  static constexpr int NP = P::npass;
  static constexpr int LAST = NP - 1;
  static constexpr bool BETA_SMEM = Cfg::BETA_SMEM;
  static_assert(CTA % TPT == 0, "CTA must hold whole trajectories");
  static_assert(P::reg[0][P::e - 1] == P::nbits - 1, "top bit must be a register bit of the first pass");

  T* s_tw;
  T* s_x;
  T* s_beta;
  R* s_kt;
  T* s_kf;
  int tid, slot, t;
  int pos_thr[NP];
  int xbase[NP];

  __device__ __forceinline__ explicit SquareGroup(unsigned char* smem_raw) {
    s_tw = reinterpret_cast<T*>(smem_raw);
    s_x = s_tw + (I::TW0 + I::TW1);
    s_beta = s_x + 2 * Cfg::XSZ;
    s_kt = reinterpret_cast<R*>(s_beta + (BETA_SMEM ? TPC * N : 0));
    s_kf = reinterpret_cast<T*>(smem_raw + Cfg::kfac_offset());
    tid = threadIdx.x;
    // one trajectory per CTA: the trajectory index (and its Philox key) is
    // uniform across the CTA
    slot = TPC == 1 ? 0 : tid / TPT;
    t = TPC == 1 ? tid : tid % TPT;
    static_for<NP>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      int p = 0;
      static_for<P::nthr>([&](auto II) {
        constexpr int i = decltype(II)::value;
        constexpr int b = P::thr[k][i];
        p |= ((t >> i) & 1) << b;
      });
      pos_thr[k] = p;
      xbase[k] = pad16((slot << P::nbits) | p);
    });
  }

  // twiddles and k-space table into shared memory (the caller synchronises)
  __device__ __forceinline__ void load_tables(const StepArgs& a) {
    for (int i = tid; i < I::TW0; i += CTA) s_tw[i] = reinterpret_cast<const T*>(a.tw)[i];
    for (int i = tid; i < I::TW1; i += CTA) s_tw[I::TW0 + i] = reinterpret_cast<const T*>(a.tw)[I::M0 + i];
    for (int i = tid; i < I::M0 + I::M1; i += CTA) s_kt[i] = reinterpret_cast<const R*>(a.ktab)[i];
    if ((SPLIT || !FAST) && a.kfac != nullptr && a.kfac_smem)
      for (int i = tid; i < N; i += CTA) s_kf[pad16(i)] = reinterpret_cast<const T*>(a.kfac)[i];
  }

  __device__ __forceinline__ void run(const StepArgs& a, int64_t g, int& buf) {
    const T* tw0 = s_tw;
    const T* tw1 = s_tw + I::TW0;
    const bool has_rsl = a.rsl != nullptr, has_iU = !FAST && a.iU != nullptr, has_iF = !FAST && a.iF != nullptr;
    // thread parts of the k-space indices in the last pass's layout
    const int ky_t = I::bitrev(pos_thr[LAST] & ((1 << P::by) - 1), P::by);
    const int kx_t = P::bx ? I::bitrev(pos_thr[LAST] >> P::by, P::bx) : 0;
    const R* s_ky = s_kt + ky_t;
    const R* s_kx = s_kt + I::M0 + kx_t;
    const R kx_const = s_kx[0];  // used when no register bit is a row bit
    // split step (compiled in with SPLIT, tested at run time by the general
    // instantiation): the factor table, thread part of the padded position
    // in the last pass's layout
    const bool split = SPLIT ? true : (FAST ? false : a.kfac != nullptr);
    const int kf_thr = pad16(pos_thr[LAST]);
    const T* __restrict__ g_kf = reinterpret_cast<const T*>(a.kfac);
    const R dt = sizeof(R) == 4 ? R(a.f_dt) : R(a.dt), dt4 = sizeof(R) == 4 ? R(a.f_dt4) : R(a.dt4);
    const T rsl_s = sizeof(R) == 4 ? cmake<T>(R(a.f_par[0]), R(a.f_par[1])) : cmake<T>(R(a.rsl_s[0]), R(a.rsl_s[1]));
    const T iU_s = sizeof(R) == 4 ? cmake<T>(R(a.f_par[2]), R(a.f_par[3])) : cmake<T>(R(a.iU_s[0]), R(a.iU_s[1]));
    const T iF_s = sizeof(R) == 4 ? cmake<T>(R(a.f_par[4]), R(a.f_par[5])) : cmake<T>(R(a.iF_s[0]), R(a.iF_s[1]));
    const int64_t traj = g * TPC + slot;
    const bool active = traj < a.ntraj;
    const int64_t tr = active ? traj : 0;
    T* st = reinterpret_cast<T*>(a.state) + tr * N;
    T* my_beta = s_beta + slot * N + t;  // element s at my_beta[s * TPT]
    T rbeta[BETA_SMEM ? 1 : E];
    auto bget = [&](auto S) -> T {
      constexpr int s = decltype(S)::value;
      if constexpr (BETA_SMEM) return my_beta[s * TPT]; else return rbeta[s];
    };
    auto bset = [&](auto S, T v) {
      constexpr int s = decltype(S)::value;
      if constexpr (BETA_SMEM) my_beta[s * TPT] = v; else rbeta[s] = v;
    };
    static_for<E>([&](auto S) {
      constexpr int s = decltype(S)::value;
      bset(S, st[pos_thr[0] | I::pos_reg(0, s)]);
    });
    const T* __restrict__ g_rsl = has_rsl ? reinterpret_cast<const T*>(a.rsl) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iU = has_iU ? reinterpret_cast<const T*>(a.iU) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iF = has_iF ? reinterpret_cast<const T*>(a.iF) + tr * a.par_stride : nullptr;
    const uint32_t seed = a.seeds[tr], id = a.ids[tr];
    const T* noise_tr = reinterpret_cast<const T*>(a.noise) + tr * a.noise_traj_stride;
    // single-system FP32 kernel (no register cap), chains of 1024 sites and
    // more: the thread-dependent twiddles in registers for the whole launch.
    // Their per-step table loads are strided across threads there (bank
    // conflicts on a 3072-entry table); measured on GB300: 1x4096 0.95e11 ->
    // 1.74e11 site-updates/s, 1x1024 1.90e11 -> 2.05e11, while 64x64 (-11 %),
    // 32x32 (-3 %) and 1x256 (-5 %) lost to the extra register pressure.
    constexpr bool HT = REG_SMALL && sizeof(R) == 4 && plan_reg_twiddles<P>();
    // RE_RSL: the fast single-system kernel (launched only when the per-site
    // rsl share one real part, rsl_re_uniform) keeps 16 per-site values
    // instead of 32 for the launch; measured on GB300: 64x64 2.19e11 ->
    // 2.27e11, 32x32 2.30e11 -> 2.35e11, 16x16 3.36e11 -> 3.48e11
    // site-updates/s, while the register-twiddle chains lost 4 %.
    constexpr bool RE_RSL = FAST && REG_SMALL && sizeof(R) == 4 && !HT;
    T twr[HT ? TwSlots<P>::total() : 1];
    if constexpr (HT) load_twiddle_set<P>(twr, tw0, tw1, pos_thr);

    // CARRY: x holds the state at the top of every step, loaded once and then
    // carried from the local update (which also stores it to the slices),
    // instead of reloaded from the slices every step; measured on GB300:
    // 64x64 0.4 % faster, while the chains with their twiddles in registers
    // (HT) lost 6 % to the longer register lifetimes. LU_MADD: the
    // multiply-add form of the local update (local_update_fused<true>) on
    // every plan but 64x64: 1x4096 1.77e11 -> 1.79e11, 1x1024 2.05e11 ->
    // 2.09e11, 32x32 2.34e11 -> 2.47e11 site-updates/s, while 64x64 measured
    // 1 % faster without it.
    constexpr bool CARRY = !HT;
    constexpr bool LU_MADD = HT || P::nbits < 12;
    T x[E];
    static_for<E>([&](auto S) { x[decltype(S)::value] = bget(S); });
    for (int64_t step = 0; step < a.nsteps; ++step) {
      const uint32_t gstep = a.step0 + uint32_t(step);
      if constexpr (!CARRY) static_for<E>([&](auto S) { x[decltype(S)::value] = bget(S); });
      // forward FFT
      static_for<NP>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        if constexpr (k > 0) {
          fft_exchange<P, k - 1, k, Cfg::SYNC_WARP>(x, s_x + buf * Cfg::XSZ, xbase[k - 1], xbase[k]);
          buf ^= 1;
        }
        fft_pass<P, k, false, HT, REG_SMALL>(x, tw0, tw1, pos_thr[k], twr);
      });
      // k-space multiply by -i 2J (cos kx + cos ky) / N (Euler), or by
      // (exp(-i 2J (cos kx + cos ky) dt) - 1) / N (split step: the inverse
      // transform is then beta' - beta)
      if (split) {
        if (a.kfac_smem) {
          static_for<E>([&](auto S) {
            constexpr int s = decltype(S)::value;
            x[s] = cmul(x[s], s_kf[kf_thr + pad16(I::pos_reg(LAST, s))]);
          });
        } else {
          static_for<E>([&](auto S) {
            constexpr int s = decltype(S)::value;
            x[s] = cmul(x[s], __ldg(g_kf + (pos_thr[LAST] | I::pos_reg(LAST, s))));
          });
        }
      } else {
        static_for<E>([&](auto S) {
          constexpr int s = decltype(S)::value;
          constexpr int pr = I::pos_reg(LAST, s);
          R sk = s_ky[I::ky_of(pr)];
          if constexpr (I::last_has_row_reg()) sk += s_kx[I::kx_of(pr)]; else sk += kx_const;
          x[s] = cmake<T>(sk * x[s].y, -sk * x[s].x);
        });
      }
      // inverse FFT (adjoint passes in reverse order)
      static_for<NP>([&](auto KK) {
        constexpr int k = LAST - decltype(KK)::value;
        fft_pass<P, k, true, HT>(x, tw0, tw1, pos_thr[k], twr);
        if constexpr (k > 0) {
          fft_exchange<P, k, k - 1, Cfg::SYNC_WARP>(x, s_x + buf * Cfg::XSZ, xbase[k], xbase[k - 1]);
          buf ^= 1;
        }
      });
      // noise + local update (pass-0 layout: slot bit e-1 is the top site bit)
      static_for<E / 2>([&](auto Q) {
        constexpr int s_lo = decltype(Q)::value;          // top slot bit clear
        constexpr int s_hi = s_lo | (E / 2);
        T xi_lo, xi_hi;
        if (FAST || a.noise_mode == 0) {
          const int p = pos_thr[0] | I::pos_reg(0, s_lo);  // p < N/2
          const u32x4 w = wiener_words(uint32_t(p), gstep, seed, id);
          xi_lo = Wiener<R>::term(w.x, w.y, a);
          xi_hi = Wiener<R>::term(w.z, w.w, a);
        } else {
          const T* nz = noise_tr + (int64_t(gstep)) * N;
          xi_lo = Wiener<R>::buffer(nz[pos_thr[0] | I::pos_reg(0, s_lo)], dt4);
          xi_hi = Wiener<R>::buffer(nz[pos_thr[0] | I::pos_reg(0, s_hi)], dt4);
        }
        T r_lo = rsl_s, r_hi = rsl_s, u_lo = iU_s, u_hi = iU_s, f_lo = iF_s, f_hi = iF_s;
        {
          const int plo = pos_thr[0] | I::pos_reg(0, s_lo);
          const int phi = pos_thr[0] | I::pos_reg(0, s_hi);
          if (has_rsl) {
            if constexpr (RE_RSL) {
              r_lo = cmake<T>(rsl_s.x, __ldg(&g_rsl[plo].y));
              r_hi = cmake<T>(rsl_s.x, __ldg(&g_rsl[phi].y));
            } else {
              r_lo = __ldg(g_rsl + plo);
              r_hi = __ldg(g_rsl + phi);
            }
          }
          if (has_iU) { u_lo = __ldg(g_iU + plo); u_hi = __ldg(g_iU + phi); }
          if (has_iF) { f_lo = __ldg(g_iF + plo); f_hi = __ldg(g_iF + phi); }
        }
        constexpr std::integral_constant<int, s_lo> SL{};
        constexpr std::integral_constant<int, s_hi> SH{};
        T n_lo, n_hi;
        if (split) {  // the local step on beta' = beta + (beta' - beta), no hopping term
          const T zero = cmake<T>(R(0), R(0));
          const T b_lo = cadd(bget(SL), x[s_lo]), b_hi = cadd(bget(SH), x[s_hi]);
          if constexpr (sizeof(R) == 4) {
            n_lo = local_update_fused(b_lo, zero, r_lo, u_lo, f_lo, dt, Wiener<R>::scale(dt4), xi_lo);
            n_hi = local_update_fused(b_hi, zero, r_hi, u_hi, f_hi, dt, Wiener<R>::scale(dt4), xi_hi);
          } else {
            n_lo = local_update(b_lo, zero, r_lo, u_lo, f_lo, dt, Wiener<R>::scale(dt4), xi_lo);
            n_hi = local_update(b_hi, zero, r_hi, u_hi, f_hi, dt, Wiener<R>::scale(dt4), xi_hi);
          }
        } else if constexpr (sizeof(R) == 4) {  // dt is folded into the k-space table
          n_lo = local_update_fused<LU_MADD>(bget(SL), x[s_lo], r_lo, u_lo, f_lo, dt, Wiener<R>::scale(dt4), xi_lo);
          n_hi = local_update_fused<LU_MADD>(bget(SH), x[s_hi], r_hi, u_hi, f_hi, dt, Wiener<R>::scale(dt4), xi_hi);
        } else {
          n_lo = local_update(bget(SL), x[s_lo], r_lo, u_lo, f_lo, dt, Wiener<R>::scale(dt4), xi_lo);
          n_hi = local_update(bget(SH), x[s_hi], r_hi, u_hi, f_hi, dt, Wiener<R>::scale(dt4), xi_hi);
        }
        bset(SL, n_lo);
        bset(SH, n_hi);
        if constexpr (CARRY) {
          x[s_lo] = n_lo;
          x[s_hi] = n_hi;
        }
      });
    }

    // write back, status
    bool bad = false;
    if (active) {
      static_for<E>([&](auto S) {
        constexpr int s = decltype(S)::value;
        const T b = bget(S);
        st[pos_thr[0] | I::pos_reg(0, s)] = b;
        bad |= !finite_c(b);
      });
      set_status(a.status, traj, bad);
    }
    // |FFT(beta)|^2 / N of the final state for the k-space populations
    if (a.nk != nullptr) {
      T x[E];
      static_for<E>([&](auto S) { x[decltype(S)::value] = bget(S); });
      static_for<NP>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        if constexpr (k > 0) {
          fft_exchange<P, k - 1, k, Cfg::SYNC_WARP>(x, s_x + buf * Cfg::XSZ, xbase[k - 1], xbase[k]);
          buf ^= 1;
        }
        fft_pass<P, k, false>(x, tw0, tw1, pos_thr[k]);
      });
      if (active) {
        R* nk = reinterpret_cast<R*>(a.nk) + traj * N;
        static_for<E>([&](auto S) {
          constexpr int s = decltype(S)::value;
          const uint32_t p = uint32_t(pos_thr[LAST] | I::pos_reg(LAST, s));
          const uint32_t pc = p & ((1u << P::by) - 1u), pr = p >> P::by;
          const uint32_t ky = P::by ? (__brev(pc) >> (32 - P::by)) : 0u;
          const uint32_t kx = P::bx ? (__brev(pr) >> (32 - P::bx)) : 0u;
          nk[(kx << P::by) | ky] = (x[s].x * x[s].x + x[s].y * x[s].y) / R(N);
        });
      }
    }
  }
};

// No minimum of resident CTAs: the 4096-site plans then keep their 16 sites
// per thread, twiddles and Philox state in up to 255 registers at one CTA per
// SM, which measured 7 % (64x64) and 17 % (1x4096) faster than two CTAs per
// SM at a 128-register cap with spills; the smaller plans stay below 128
// registers either way.
template <typename R, class P, int CTA, bool FAST = false, bool SPLIT = false>
__global__ void __launch_bounds__(CTA, 1) square_fft_kernel(const StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using G = SquareGroup<R, P, CTA, FAST, true, SPLIT>;
  G grp(smem_raw);
  grp.load_tables(a);
  __syncthreads();
  int buf = 0;
  const int64_t ngroups = (a.ntraj + G::TPC - 1) / G::TPC;
  for (int64_t g = blockIdx.x; g < ngroups; g += gridDim.x) grp.run(a, g, buf);
}

// ------------------------------------------------------------------------
// real-space hopping kernel (Lieb lattice, square stencil, any N)
// Thread t of a trajectory holds VPT sites: for v < VPT/2 site t + v*TPT,
// for v >= VPT/2 site half + t + (v - VPT/2)*TPT (half = ceil(N/2)), so the
// two sites of one Philox call live in the same thread. Site indices are
// recomputed from t (one multiply-add), not stored.
// HOP = 0: neighbour table h = sum_j w_pj b[idx_pj] (Lieb couplings), the
//          indices kept in registers as packed 16-bit pairs (N <= 16384),
//          the weights -- purely imaginary (-i J), as the host builds them --
//          as their imaginary parts in shared memory behind the field
//          buffers, four per site in one 16-byte row (FP32).
// HOP = 1: square stencil h = -i J (wy (b[c+1] + b[c-1]) + wx (b[r+1] + b[r-1])),
//          the (row, column) of each site advanced incrementally through the
//          thread's sites every step, so nothing per site but the field is
//          held in registers (VPT = 16 with 1024 threads fits 64 registers).
// FAST: the common run (Philox noise, no F(t), no work / area) with those
//       features compiled out instead of tested per site.
// ------------------------------------------------------------------------
// Bytes of the real-space kernel's field buffers (one or two per trajectory
// slot), rounded up to 16 so that the Lieb weights behind them start aligned.
__host__ __device__ __forceinline__ size_t ell_state_bytes(bool dbuf, int tpc, int64_t n, size_t csize) {
  return ((dbuf ? 2 : 1) * size_t(tpc) * size_t(n) * csize + 15) & ~size_t(15);
}

// Groups g_begin, g_begin + g_stride, ... (a grid-stride loop by default; a
// work-queue kernel passes one group and a stride past the end).
template <typename R, int VPT, int CTA, int HOP, bool FAST = false>
__device__ __forceinline__ void ell_body(const StepArgs& a, unsigned char* smem_raw, int64_t g_begin,
                                         int64_t g_stride) {
  using T = c2_t<R>;
  constexpr int H = VPT / 2;
  T* s_b = reinterpret_cast<T*>(smem_raw);
  const int N = int(a.nsites);
  const int half = (N + 1) / 2;
  const int tpt = a.tpt;
  const int tpc = CTA / tpt;
  const int tid = threadIdx.x;
  const int slot = tid / tpt;
  const int t = tid % tpt;
  const bool in_slot = slot < tpc;
  // site of slot v and whether it exists
  auto site_of = [&](int v) -> int { return v < H ? t + v * tpt : half + t + (v - H) * tpt; };
  auto valid_of = [&](int v) -> bool { return in_slot && (v < H ? site_of(v) < half : site_of(v) < N); };

  uint32_t nb01[HOP == 0 ? VPT : 1], nb23[HOP == 0 ? VPT : 1];
  // square stencil: (row, column) of the first low-half and high-half site,
  // and the (row, column) increment of one slot (tpt sites)
  const int nx = int(a.nx), ny = int(a.ny);
  int rl0 = 0, cl0 = 0, rh0 = 0, ch0 = 0, dr = 0, dc = 0;
  if constexpr (HOP == 0) {
#pragma unroll
    for (int v = 0; v < VPT; ++v) {
      const int p = valid_of(v) ? site_of(v) : 0;
      int n4[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) n4[j] = a.nbr_idx[int64_t(p) * 4 + j];
      nb01[v] = uint32_t(n4[0]) | (uint32_t(n4[1]) << 16);
      nb23[v] = uint32_t(n4[2]) | (uint32_t(n4[3]) << 16);
    }
  } else {
    rl0 = t / ny; cl0 = t % ny;
    rh0 = (half + t) / ny; ch0 = (half + t) % ny;
    dr = tpt / ny; dc = tpt % ny;
  }
  const T* __restrict__ g_w = reinterpret_cast<const T*>(a.nbr_w);
  uint32_t swa = 0;  // shared-memory address of the weights (HOP = 0)
  if constexpr (HOP == 0) {
    const size_t sbytes = ell_state_bytes(a.dbuf != 0, tpc, N, sizeof(T));
    R* s_wt = reinterpret_cast<R*>(smem_raw + sbytes);
    for (int i = tid; i < 4 * N; i += CTA) s_wt[i] = g_w[i].y;  // covered by the first step's barrier
    swa = smem_addr(s_wt);
  }
  const R wy = ny > 1 ? R(1) : R(0), wx = nx > 1 ? R(1) : R(0);
  constexpr bool F32 = sizeof(R) == 4;
  const R J = F32 ? R(a.f_J) : R(a.J);
  const R dt = F32 ? R(a.f_dt) : R(a.dt), dt4 = F32 ? R(a.f_dt4) : R(a.dt4);
  const T rsl_s = F32 ? cmake<T>(R(a.f_par[0]), R(a.f_par[1])) : cmake<T>(R(a.rsl_s[0]), R(a.rsl_s[1]));
  const T iU_s = F32 ? cmake<T>(R(a.f_par[2]), R(a.f_par[3])) : cmake<T>(R(a.iU_s[0]), R(a.iU_s[1]));
  const T iF_s = F32 ? cmake<T>(R(a.f_par[4]), R(a.f_par[5])) : cmake<T>(R(a.iF_s[0]), R(a.iF_s[1]));
  const bool timedep = !FAST && a.ft_vals != nullptr;

  const int64_t ngroups = (a.ntraj + tpc - 1) / tpc;
  const int64_t slice = N;
  int buf = 0;
  for (int64_t g = g_begin; g < ngroups; g += g_stride) {
    const int64_t traj = g * tpc + slot;
    const bool active = in_slot && traj < a.ntraj;
    const int64_t tr = active ? traj : 0;
    T* st = reinterpret_cast<T*>(a.state) + tr * N;
    const T* __restrict__ g_rsl = a.rsl ? reinterpret_cast<const T*>(a.rsl) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iU = a.iU ? reinterpret_cast<const T*>(a.iU) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iF = a.iF ? reinterpret_cast<const T*>(a.iF) + tr * a.par_stride : nullptr;
    T beta[VPT];
#pragma unroll
    for (int v = 0; v < VPT; ++v) beta[v] = active && valid_of(v) ? st[site_of(v)] : cmake<T>(R(0), R(0));
    const uint32_t seed = a.seeds[tr], id = a.ids[tr];
    const T* noise_tr = reinterpret_cast<const T*>(a.noise) + tr * a.noise_traj_stride;
    for (int64_t step = 0; step < a.nsteps; ++step) {
      const uint32_t gstep = a.step0 + uint32_t(step);
      T* sb = s_b + (a.dbuf ? buf : 0) * int64_t(tpc) * slice + int64_t(in_slot ? slot : 0) * slice;
      const uint32_t sba = smem_addr(sb);
      auto ld_site = [&](int q) -> T { return lds_c(sba + uint32_t(q) * uint32_t(sizeof(T)), T{}); };
#pragma unroll
      for (int v = 0; v < VPT; ++v) if (valid_of(v)) sts_c(sba + uint32_t(site_of(v)) * uint32_t(sizeof(T)), beta[v]);
      __syncthreads();
      // hopping term of a site, read lazily from this step's buffer (the next
      // step writes the other buffer, or waits at the second barrier)
      auto hop_table = [&](int v) -> T {
        const T b0 = ld_site(int(nb01[HOP == 0 ? v : 0] & 0xFFFFu)), b1 = ld_site(int(nb01[HOP == 0 ? v : 0] >> 16));
        const T b2 = ld_site(int(nb23[HOP == 0 ? v : 0] & 0xFFFFu)), b3 = ld_site(int(nb23[HOP == 0 ? v : 0] >> 16));
        R w[4];  // idle slots read site 0's row, as their neighbour indices do
        lds_r4(swa + uint32_t(valid_of(v) ? site_of(v) : 0) * uint32_t(4 * sizeof(R)), w);
        // (i w) b with each product rounded once, as the complex product with
        // a zero real part gives
        T acc = cmake<T>(-(w[0] * b0.y), w[0] * b0.x);
        acc = cadd(acc, cmake<T>(-(w[1] * b1.y), w[1] * b1.x));
        acc = cadd(acc, cmake<T>(-(w[2] * b2.y), w[2] * b2.x));
        return cadd(acc, cmake<T>(-(w[3] * b3.y), w[3] * b3.x));
      };
      auto hop_stencil = [&](int p, int r, int c) -> T {
        const int right = c + 1 < ny ? p + 1 : p + 1 - ny, left = c > 0 ? p - 1 : p - 1 + ny;
        const int down = r + 1 < nx ? p + ny : p + ny - N, up = r > 0 ? p - ny : p - ny + N;
        const T sy = cadd(ld_site(right), ld_site(left)), sx = cadd(ld_site(down), ld_site(up));
        const T s = cmake<T>(wy * sy.x + wx * sx.x, wy * sy.y + wx * sx.y);
        return cmake<T>(J * s.y, -J * s.x);  // -i J s
      };
      int id_t = 0, id_p = 0;
      R dtt = R(0), dtp = R(0), seg_ratio = R(0);
      if (timedep) {
        id_t = a.ft_id[gstep];
        dtt = F32 ? R(a.ft_dt_f[gstep]) : R(a.ft_dt[gstep]);
        if (!FAST && a.work != nullptr) {  // work / area: the previous step's F(t)
          id_p = gstep > 0 ? a.ft_id[gstep - 1] : id_t;
          dtp = gstep > 0 ? (F32 ? R(a.ft_dt_f[gstep - 1]) : R(a.ft_dt[gstep - 1])) : dtt;
          if (gstep > 0) seg_ratio = R((a.ft_dt[gstep] - a.ft_dt[gstep - 1]) / a.dt);
        }
      }
      int rl = rl0, cl = cl0, rh = rh0, ch = ch0;
#pragma unroll
      for (int v = 0; v < H; ++v) {
        T xi_lo, xi_hi;
        if (FAST || a.noise_mode == 0) {
          const u32x4 w = wiener_words(uint32_t(site_of(v)), gstep, seed, id);
          xi_lo = Wiener<R>::term(w.x, w.y, a);
          xi_hi = Wiener<R>::term(w.z, w.w, a);
        } else {
          const T* nz = noise_tr + int64_t(gstep) * N;
          xi_lo = Wiener<R>::buffer(valid_of(v) ? nz[site_of(v)] : cmake<T>(R(0), R(0)), dt4);
          xi_hi = Wiener<R>::buffer(valid_of(v + H) ? nz[site_of(v + H)] : cmake<T>(R(0), R(0)), dt4);
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int vv = q ? v + H : v;
          const bool ok = valid_of(vv);
          const int p = ok ? site_of(vv) : 0;
          const T r = g_rsl ? __ldg(g_rsl + p) : rsl_s;
          const T u = g_iU ? __ldg(g_iU + p) : iU_s;
          T f = g_iF ? __ldg(g_iF + p) : iF_s;
          if (timedep) {
            const T f0 = __ldg(reinterpret_cast<const T*>(a.ft_vals) + int64_t(id_t) * N + p);
            const T f1 = __ldg(reinterpret_cast<const T*>(a.ft_slopes) + int64_t(id_t) * N + p);
            f = cmake<T>(f0.x + dtt * f1.x, f0.y + dtt * f1.y);
          }
          T h;
          if constexpr (HOP == 0) h = hop_table(vv);
          else h = ok ? (q ? hop_stencil(p, rh, ch) : hop_stencil(p, rl, cl)) : cmake<T>(R(0), R(0));
          beta[vv] = local_update(beta[vv], h, r, u, f, dt, Wiener<R>::scale(dt4), q ? xi_hi : xi_lo);
          if (!FAST && a.work != nullptr && ok && active) {
            R fd = R(0);
            if (timedep && gstep > 0) {  // Re F = Im(i F); the first step of a run has F(t - dt) = F(t)
              if (id_p == id_t) {
                // same table segment: the difference is the slope times the
                // time step, free of the cancellation of F(t) - F(t - dt)
                fd = __ldg(reinterpret_cast<const T*>(a.ft_slopes) + int64_t(id_t) * N + p).y * seg_ratio;
              } else {
                const T g0 = __ldg(reinterpret_cast<const T*>(a.ft_vals) + int64_t(id_p) * N + p);
                const T g1 = __ldg(reinterpret_cast<const T*>(a.ft_slopes) + int64_t(id_p) * N + p);
                fd = (f.y - (g0.y + dtp * g1.y)) / dt;
              }
            }
            const T b = beta[vv];
            R* wk = reinterpret_cast<R*>(a.work) + tr * N + p;
            R* ar = reinterpret_cast<R*>(a.area) + tr * N + p;
            *wk += (R(2) * dt) * b.x * fd;
            *ar += (dt * fd) * (b.x * b.x + b.y * b.y - R(0.5));
          }
        }
        if constexpr (HOP == 1) {  // advance both sites by tpt
          cl += dc; rl += dr; if (cl >= ny) { cl -= ny; ++rl; }
          ch += dc; rh += dr; if (ch >= ny) { ch -= ny; ++rh; }
        }
      }
      if (a.dbuf) buf ^= 1; else __syncthreads();
    }
    if (active) {
      bool bad = false;
#pragma unroll
      for (int v = 0; v < VPT; ++v) if (valid_of(v)) { st[site_of(v)] = beta[v]; bad |= !finite_c(beta[v]); }
      set_status(a.status, traj, bad);
    }
  }
}

template <typename R, int VPT, int CTA, int HOP, bool FAST>
__global__ void __launch_bounds__(CTA) ell_kernel(const StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ell_body<R, VPT, CTA, HOP, FAST>(a, smem_raw, blockIdx.x, gridDim.x);
}

// Same, with the arguments in device memory (kept there across the frames of a
// captured graph); they are copied to shared memory first.
template <typename R, int VPT, int CTA, int HOP, bool FAST>
__global__ void __launch_bounds__(CTA) ell_kernel_dev(const StepArgs* __restrict__ ap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  for (int i = threadIdx.x; i < int(sizeof(StepArgs) / 4); i += CTA)
    reinterpret_cast<uint32_t*>(&s_a)[i] = reinterpret_cast<const uint32_t*>(ap)[i];
  __syncthreads();
  ell_body<R, VPT, CTA, HOP, FAST>(s_a, smem_raw, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------------
// Square stencil with runs of four sites along a row per thread (FP32, the
// fast run: Philox noise, no F(t), no work / area). Thread t of a trajectory
// holds sites 4t..4t+3 and their Philox partners N/2 + 4t..N/2 + 4t + 3
// (ny and N/2 multiples of 4, so a run never crosses a row end). The runs
// go to shared memory in two 16-byte stores; per run the rows above and
// below arrive in two 16-byte loads each and the left / right ends in one
// load each, while the neighbours inside the run are the thread's own
// registers -- 1.5 loads per site-update instead of 4. The sums keep the
// order of ell_body's stencil (right + left, then down + up), so results
// equal the real-space kernel's.
// ------------------------------------------------------------------------
template <int CTA>
__device__ __forceinline__ void rowrun_body(const StepArgs& a, unsigned char* smem_raw, int64_t g_begin,
                                            int64_t g_stride) {
  using T = float2;
  T* s_b = reinterpret_cast<T*>(smem_raw);
  const int N = int(a.nsites), half = N / 2, nx = int(a.nx), ny = int(a.ny);
  const int tpt = half / 4, tpc = CTA / tpt;
  const int tid = threadIdx.x, slot = tid / tpt, t = tid % tpt;
  const bool in_slot = slot < tpc;
  const float J = a.f_J, dt = a.f_dt;
  const T rsl_s = make_float2(a.f_par[0], a.f_par[1]);
  const T iU_s = make_float2(a.f_par[2], a.f_par[3]);
  const T iF_s = make_float2(a.f_par[4], a.f_par[5]);
  const float wy = ny > 1 ? 1.f : 0.f, wx = nx > 1 ? 1.f : 0.f;
  constexpr uint32_t TS = uint32_t(sizeof(T));
  // per run k: first site, and the sites of its up / down rows and of its
  // left / right ends (periodic)
  int p0[2], up[2], dn[2], lf[2], rt[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int p = k * half + 4 * t, r = p / ny, c = p % ny;
    p0[k] = p;
    up[k] = (r > 0 ? r - 1 : nx - 1) * ny + c;
    dn[k] = (r + 1 < nx ? r + 1 : 0) * ny + c;
    lf[k] = r * ny + (c > 0 ? c - 1 : ny - 1);
    rt[k] = r * ny + (c + 4 < ny ? c + 4 : 0);
  }
  const int64_t ngroups = (a.ntraj + tpc - 1) / tpc;
  int buf = 0;
  for (int64_t g = g_begin; g < ngroups; g += g_stride) {
    const int64_t traj = g * tpc + slot;
    const bool active = in_slot && traj < a.ntraj;
    const int64_t tr = active ? traj : 0;
    T* st = reinterpret_cast<T*>(a.state) + tr * N;
    const T* __restrict__ g_rsl = a.rsl ? reinterpret_cast<const T*>(a.rsl) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iU = a.iU ? reinterpret_cast<const T*>(a.iU) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iF = a.iF ? reinterpret_cast<const T*>(a.iF) + tr * a.par_stride : nullptr;
    T v[2][4];
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int j = 0; j < 4; ++j) v[k][j] = active ? st[p0[k] + j] : make_float2(0.f, 0.f);
    const uint32_t seed = a.seeds[tr], id = a.ids[tr];
    for (int64_t step = 0; step < a.nsteps; ++step) {
      const uint32_t gstep = a.step0 + uint32_t(step);
      T* sb = s_b + (a.dbuf ? buf : 0) * int64_t(tpc) * N + int64_t(in_slot ? slot : 0) * N;
      const uint32_t sba = smem_addr(sb);
      if (in_slot) {
        sts_run4(sba + uint32_t(p0[0]) * TS, v[0]);
        sts_run4(sba + uint32_t(p0[1]) * TS, v[1]);
      }
      __syncthreads();
      T h[2][4];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        T U[4], D[4];
        lds_run4(sba + uint32_t(up[k]) * TS, U);
        lds_run4(sba + uint32_t(dn[k]) * TS, D);
        const T L = lds_c(sba + uint32_t(lf[k]) * TS, T{}), Rr = lds_c(sba + uint32_t(rt[k]) * TS, T{});
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const T right = j < 3 ? v[k][j + 1] : Rr, left = j > 0 ? v[k][j - 1] : L;
          const T sy = cadd(right, left), sx = cadd(D[j], U[j]);
          const T s = make_float2(wy * sy.x + wx * sx.x, wy * sy.y + wx * sx.y);
          h[k][j] = make_float2(J * s.y, -J * s.x);  // -i J s
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const u32x4 w = wiener_words(uint32_t(p0[0] + j), gstep, seed, id);
        const T xi[2] = {Wiener<float>::term(w.x, w.y, a), Wiener<float>::term(w.z, w.w, a)};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const int p = p0[k] + j;
          const T r = g_rsl ? __ldg(g_rsl + p) : rsl_s;
          const T u = g_iU ? __ldg(g_iU + p) : iU_s;
          const T f = g_iF ? __ldg(g_iF + p) : iF_s;
          v[k][j] = local_update(v[k][j], h[k][j], r, u, f, dt, 1.0f, xi[k]);
        }
      }
      if (a.dbuf) buf ^= 1; else __syncthreads();
    }
    if (active) {
      bool bad = false;
#pragma unroll
      for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          st[p0[k] + j] = v[k][j];
          bad |= !finite_c(v[k][j]);
        }
      set_status(a.status, traj, bad);
    }
  }
}

template <int CTA>
__global__ void __launch_bounds__(CTA, 1) rowrun_kernel(const StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  rowrun_body<CTA>(a, smem_raw, blockIdx.x, gridDim.x);
}

template <int CTA>
__global__ void __launch_bounds__(CTA, 1) rowrun_kernel_dev(const StepArgs* __restrict__ ap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  for (int i = threadIdx.x; i < int(sizeof(StepArgs) / 4); i += CTA)
    reinterpret_cast<uint32_t*>(&s_a)[i] = reinterpret_cast<const uint32_t*>(ap)[i];
  __syncthreads();
  rowrun_body<CTA>(s_a, smem_raw, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------------
// 1-D Lieb lattice with whole cells per thread: thread t of a trajectory
// holds cells t and t + Nc/2 (sites 3c, 3c+1, 3c+2 = A, B, C of cell c), so
// each Philox pair (p, p + N/2) is one thread's, the couplings inside a cell
// (A-B, B-C) use registers, and only C of the previous cell and B of the next
// cell come from the other threads' shared-memory slices. The neighbour
// table of the general kernel pads every site to four entries (A has one
// coupling, B three, C two); here each site sums its own couplings in the
// table's order (ascending neighbour index), each product (-i J) b rounded
// once, so the FP32 results equal the table kernel's. Couplings of
// TWMCLiebSolver::Setup (TWMCLiebSolver.cpp:52-85): A(3i)-B(3i+1) J_AB,
// B(3i+1)-C(3i+2) J_BC, C(3i+2)-B(3(i+1)+1) J_BC, with PBC
// C(3(Nc-1)+2)-B(1). Nc even, Nc / 2 <= CTA; no work / area.
// ------------------------------------------------------------------------
template <typename R, int CTA>
__device__ __forceinline__ void lieb_cell_body(const StepArgs& a, unsigned char* smem_raw) {
  using T = c2_t<R>;
  T* s_b = reinterpret_cast<T*>(smem_raw);
  const int N = int(a.nsites), nc = N / 3, half = N / 2, tpt = nc / 2;
  const int tpc = CTA / tpt;
  const int tid = threadIdx.x, slot = tid / tpt, t = tid % tpt;
  const bool in_slot = slot < tpc;
  constexpr bool F32 = sizeof(R) == 4;
  const R jab = F32 ? R(a.f_lieb_jab) : R(a.lieb_jab), jbc = F32 ? R(a.f_lieb_jbc) : R(a.lieb_jbc);
  const R dt = F32 ? R(a.f_dt) : R(a.dt), dt4 = F32 ? R(a.f_dt4) : R(a.dt4);
  const T rsl_s = F32 ? cmake<T>(R(a.f_par[0]), R(a.f_par[1])) : cmake<T>(R(a.rsl_s[0]), R(a.rsl_s[1]));
  const T iU_s = F32 ? cmake<T>(R(a.f_par[2]), R(a.f_par[3])) : cmake<T>(R(a.iU_s[0]), R(a.iU_s[1]));
  const T iF_s = F32 ? cmake<T>(R(a.f_par[4]), R(a.f_par[5])) : cmake<T>(R(a.iF_s[0]), R(a.iF_s[1]));
  const bool pbc = a.lieb_pbc != 0;
  const bool timedep = a.ft_vals != nullptr;
  // (-i J) b, each component rounded once
  auto hj = [](R j, T b) -> T { return cmake<T>(j * b.y, -(j * b.x)); };
  const T zero = cmake<T>(R(0), R(0));
  // neighbours outside the thread's cells, per held cell k: C of the previous
  // cell and B of the next one (-1: none, open boundary)
  int prev_c[2], next_b[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int c = t + k * tpt;
    prev_c[k] = c > 0 ? 3 * c - 1 : (pbc ? N - 1 : -1);
    next_b[k] = c < nc - 1 ? 3 * c + 4 : (pbc ? 1 : -1);
  }
  const int64_t ngroups = (a.ntraj + tpc - 1) / tpc;
  int buf = 0;
  for (int64_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int64_t traj = g * tpc + slot;
    const bool active = in_slot && traj < a.ntraj;
    const int64_t tr = active ? traj : 0;
    T* st = reinterpret_cast<T*>(a.state) + tr * N;
    const T* __restrict__ g_rsl = a.rsl ? reinterpret_cast<const T*>(a.rsl) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iU = a.iU ? reinterpret_cast<const T*>(a.iU) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iF = a.iF ? reinterpret_cast<const T*>(a.iF) + tr * a.par_stride : nullptr;
    T b[6];  // cell t: A, B, C; cell t + Nc/2: A, B, C
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      b[j] = active ? st[3 * t + j] : zero;
      b[3 + j] = active ? st[half + 3 * t + j] : zero;
    }
    const uint32_t seed = a.seeds[tr], id = a.ids[tr];
    const T* noise_tr = reinterpret_cast<const T*>(a.noise) + tr * a.noise_traj_stride;
    for (int64_t step = 0; step < a.nsteps; ++step) {
      const uint32_t gstep = a.step0 + uint32_t(step);
      T* sb = s_b + (a.dbuf ? buf : 0) * int64_t(tpc) * N + int64_t(in_slot ? slot : 0) * N;
      const uint32_t sba = smem_addr(sb);
      if (in_slot) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          sts_c(sba + uint32_t(3 * t + j) * uint32_t(sizeof(T)), b[j]);
          sts_c(sba + uint32_t(half + 3 * t + j) * uint32_t(sizeof(T)), b[3 + j]);
        }
      }
      __syncthreads();
      T h[6];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int c = t + k * tpt;
        const T A = b[3 * k], B = b[3 * k + 1], C = b[3 * k + 2];
        const T cp = prev_c[k] >= 0 ? lds_c(sba + uint32_t(prev_c[k]) * uint32_t(sizeof(T)), T{}) : zero;
        const T bn = next_b[k] >= 0 ? lds_c(sba + uint32_t(next_b[k]) * uint32_t(sizeof(T)), T{}) : zero;
        h[3 * k] = hj(jab, B);
        // B: neighbours in ascending index -- C of the previous cell first,
        // except in cell 0, where it wraps to the last site
        if (c > 0) {
          h[3 * k + 1] = cadd(cadd(hj(jbc, cp), hj(jab, A)), hj(jbc, C));
        } else {
          const T s = cadd(hj(jab, A), hj(jbc, C));
          h[3 * k + 1] = prev_c[k] >= 0 ? cadd(s, hj(jbc, cp)) : s;
        }
        // C: B of its cell, then B of the next cell -- first in the last cell,
        // where the next B wraps to site 1
        if (c < nc - 1) {
          h[3 * k + 2] = cadd(hj(jbc, B), hj(jbc, bn));
        } else {
          h[3 * k + 2] = next_b[k] >= 0 ? cadd(hj(jbc, bn), hj(jbc, B)) : hj(jbc, B);
        }
      }
      int id_t = 0;
      R dtt = R(0);
      if (timedep) {
        id_t = a.ft_id[gstep];
        dtt = F32 ? R(a.ft_dt_f[gstep]) : R(a.ft_dt[gstep]);
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T xi_lo, xi_hi;
        const int plo = 3 * t + j, phi = half + plo;
        if (a.noise_mode == 0) {
          const u32x4 w = wiener_words(uint32_t(plo), gstep, seed, id);
          xi_lo = Wiener<R>::term(w.x, w.y, a);
          xi_hi = Wiener<R>::term(w.z, w.w, a);
        } else {
          const T* nz = noise_tr + int64_t(gstep) * N;
          xi_lo = Wiener<R>::buffer(nz[plo], dt4);
          xi_hi = Wiener<R>::buffer(nz[phi], dt4);
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int p = q ? phi : plo, v = q ? 3 + j : j;
          const T r = g_rsl ? __ldg(g_rsl + p) : rsl_s;
          const T u = g_iU ? __ldg(g_iU + p) : iU_s;
          T f = g_iF ? __ldg(g_iF + p) : iF_s;
          if (timedep) {
            const T f0 = __ldg(reinterpret_cast<const T*>(a.ft_vals) + int64_t(id_t) * N + p);
            const T f1 = __ldg(reinterpret_cast<const T*>(a.ft_slopes) + int64_t(id_t) * N + p);
            f = cmake<T>(f0.x + dtt * f1.x, f0.y + dtt * f1.y);
          }
          b[v] = local_update(b[v], h[v], r, u, f, dt, Wiener<R>::scale(dt4), q ? xi_hi : xi_lo);
        }
      }
      if (a.dbuf) buf ^= 1; else __syncthreads();
    }
    if (active) {
      bool bad = false;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        st[3 * t + j] = b[j];
        st[half + 3 * t + j] = b[3 + j];
        bad |= !finite_c(b[j]) || !finite_c(b[3 + j]);
      }
      set_status(a.status, traj, bad);
    }
  }
}

template <typename R, int CTA>
__global__ void __launch_bounds__(CTA) lieb_cell_kernel(const StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  lieb_cell_body<R, CTA>(a, smem_raw);
}

// ------------------------------------------------------------------------
// Square stencil on a 2-CTA thread-block cluster per trajectory, for lattices
// whose field does not fit one CTA's double-buffered shared memory with
// registers to spare (N > 8192 sites, FP32). The sites are paired as in the
// single-CTA kernel (p and p + half share a Philox call); rank 0 of the
// cluster owns the pairs with p in [0, q), rank 1 those with p in [q, half),
// q = ceil(half / 2), so each CTA holds two contiguous quarters of the
// lattice. Each CTA keeps its sites in two shared-memory buffers (slots
// [0, q) low sites, [q, 2q) their partners); a step reads the current buffer
// -- neighbours owned by the other CTA through distributed shared memory --
// and writes the next one, then the cluster synchronises once. The field is
// never held in registers, so a thread loops over its pairs without
// unrolling and 1024 threads fit 64 registers. Per-site parameters and both
// noise modes as in the single-CTA kernel; no F(t) and no work / area.
// ------------------------------------------------------------------------
// Trajectories tr_begin, tr_begin + tr_stride, ... per cluster (both CTAs
// of a cluster pass the same values).
template <typename R, int CTA>
__device__ __forceinline__ void ell_cluster_body(const StepArgs& a, unsigned char* smem_raw, int64_t tr_begin,
                                                 int64_t tr_stride) {
  namespace cg = cooperative_groups;
  using T = c2_t<R>;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = int(cl.block_rank());
  const int N = int(a.nsites), half = (N + 1) / 2, q = (half + 1) / 2;
  const int lo0 = rank == 0 ? 0 : q;
  const int npair = rank == 0 ? q : half - q;
  const int nx = int(a.nx), ny = int(a.ny);
  const R wy = ny > 1 ? R(1) : R(0), wx = nx > 1 ? R(1) : R(0);
  constexpr bool F32 = sizeof(R) == 4;
  const R J = F32 ? R(a.f_J) : R(a.J);
  const R dt = F32 ? R(a.f_dt) : R(a.dt), dt4 = F32 ? R(a.f_dt4) : R(a.dt4);
  const T rsl_s = F32 ? cmake<T>(R(a.f_par[0]), R(a.f_par[1])) : cmake<T>(R(a.rsl_s[0]), R(a.rsl_s[1]));
  const T iU_s = F32 ? cmake<T>(R(a.f_par[2]), R(a.f_par[3])) : cmake<T>(R(a.iU_s[0]), R(a.iU_s[1]));
  const T iF_s = F32 ? cmake<T>(R(a.f_par[4]), R(a.f_par[5])) : cmake<T>(R(a.iF_s[0]), R(a.iF_s[1]));
  T* const own0 = reinterpret_cast<T*>(smem_raw);
  T* const own1 = own0 + 2 * q;
  constexpr uint32_t TS = uint32_t(sizeof(T));
  const uint32_t oa0 = smem_addr(own0), oa1 = smem_addr(own1);
  const uint32_t pa0 = cluster_addr(oa0, uint32_t(rank ^ 1)), pa1 = cluster_addr(oa1, uint32_t(rank ^ 1));
  const int t = threadIdx.x;
  const int rl0 = (lo0 + t) / ny, cl0 = (lo0 + t) % ny;
  const int rh0 = (lo0 + t + half) / ny, ch0 = (lo0 + t + half) % ny;
  const int dr = CTA / ny, dc = CTA % ny;
  // field value of site p in buffer b (owner and slot from the pairing)
  auto load = [&](int b, int p) -> T {
    const bool hi = p >= half;
    const int lo = hi ? p - half : p;
    const int owner = lo < q ? 0 : 1;
    const int slot = (hi ? q : 0) + lo - (owner ? q : 0);
    return owner == rank ? lds_c((b ? oa1 : oa0) + uint32_t(slot) * TS, T{})
                         : ldc_c((b ? pa1 : pa0) + uint32_t(slot) * TS, T{});
  };
  for (int64_t tr = tr_begin; tr < a.ntraj; tr += tr_stride) {
    T* st = reinterpret_cast<T*>(a.state) + tr * N;
    const T* __restrict__ g_rsl = a.rsl ? reinterpret_cast<const T*>(a.rsl) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iU = a.iU ? reinterpret_cast<const T*>(a.iU) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iF = a.iF ? reinterpret_cast<const T*>(a.iF) + tr * a.par_stride : nullptr;
    const uint32_t seed = a.seeds[tr], id = a.ids[tr];
    const T* noise_tr = reinterpret_cast<const T*>(a.noise) + tr * a.noise_traj_stride;
    for (int j = t; j < npair; j += CTA) {
      const int pl = lo0 + j, ph = pl + half;
      own0[j] = st[pl];
      if (ph < N) own0[q + j] = st[ph];
    }
    cl.sync();
    int b = 0;
    bool bad = false;
    for (int64_t step = 0; step < a.nsteps; ++step) {
      const uint32_t gstep = a.step0 + uint32_t(step);
      int rl = rl0, cl_ = cl0, rh = rh0, ch = ch0;  // (row, column) of this thread's pair
#pragma unroll 1
      for (int j = t; j < npair; j += CTA) {
        const int pl = lo0 + j, ph = pl + half;
        T xi_lo, xi_hi;
        if (a.noise_mode == 0) {
          const u32x4 w = wiener_words(uint32_t(pl), gstep, seed, id);
          xi_lo = Wiener<R>::term(w.x, w.y, a);
          xi_hi = Wiener<R>::term(w.z, w.w, a);
        } else {
          const T* nz = noise_tr + int64_t(gstep) * N;
          xi_lo = Wiener<R>::buffer(nz[pl], dt4);
          xi_hi = Wiener<R>::buffer(ph < N ? nz[ph] : cmake<T>(R(0), R(0)), dt4);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const int p = k ? ph : pl;
          if (p >= N) continue;
          const int r = k ? rh : rl, c = k ? ch : cl_;
          const int right = c + 1 < ny ? p + 1 : p + 1 - ny, left = c > 0 ? p - 1 : p - 1 + ny;
          const int down = r + 1 < nx ? p + ny : p + ny - N, up = r > 0 ? p - ny : p - ny + N;
          const T sy = cadd(load(b, right), load(b, left)), sx = cadd(load(b, down), load(b, up));
          const T sv = cmake<T>(wy * sy.x + wx * sx.x, wy * sy.y + wx * sx.y);
          const T h = cmake<T>(J * sv.y, -J * sv.x);  // -i J s
          const T rr = g_rsl ? __ldg(g_rsl + p) : rsl_s;
          const T uu = g_iU ? __ldg(g_iU + p) : iU_s;
          const T ff = g_iF ? __ldg(g_iF + p) : iF_s;
          const int slot = (k ? q : 0) + j;
          const T cur = lds_c((b ? oa1 : oa0) + uint32_t(slot) * TS, T{});
          sts_c((b ? oa0 : oa1) + uint32_t(slot) * TS,
                local_update(cur, h, rr, uu, ff, dt, Wiener<R>::scale(dt4), k ? xi_hi : xi_lo));
        }
        cl_ += dc; rl += dr; if (cl_ >= ny) { cl_ -= ny; ++rl; }
        ch += dc; rh += dr; if (ch >= ny) { ch -= ny; ++rh; }
      }
      b ^= 1;
      cl.sync();
    }
    for (int j = t; j < npair; j += CTA) {
      const int pl = lo0 + j, ph = pl + half;
      const T* fin = b ? own1 : own0;
      const T v0 = fin[j];
      st[pl] = v0;
      bad |= !finite_c(v0);
      if (ph < N) {
        const T v1 = fin[q + j];
        st[ph] = v1;
        bad |= !finite_c(v1);
      }
    }
    set_status(a.status, tr, bad);
    __syncthreads();  // the write-back reads buffer b before the next trajectory loads buffer 0
  }
}

template <typename R, int CTA>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(CTA, 1) ell_cluster_kernel(const StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ell_cluster_body<R, CTA>(a, smem_raw, blockIdx.x / 2, gridDim.x / 2);
}

template <typename R, int CTA>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(CTA, 1) ell_cluster_kernel_dev(const StepArgs* __restrict__ ap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  for (int i = threadIdx.x; i < int(sizeof(StepArgs) / 4); i += CTA)
    reinterpret_cast<uint32_t*>(&s_a)[i] = reinterpret_cast<const uint32_t*>(ap)[i];
  __syncthreads();
  ell_cluster_body<R, CTA>(s_a, smem_raw, blockIdx.x / 2, gridDim.x / 2);
}

// ------------------------------------------------------------------------
// Power-of-two form of the cluster stencil: N = nx * ny = 2^k sites, ny a
// power of two with 2 <= ny <= N / 4, FP32. Same pairing, ownership and
// shared-memory slots
// as ell_cluster_body -- rank 0 holds the quarters ("bands") [0, q) and
// [N/2, N/2 + q), rank 1 the other two, q = N / 4 -- but the owner / slot
// arithmetic reduces to bits: a row lies inside one band and the bands
// alternate between the ranks (0, 1, 0, 1, wrapping), so left / right
// neighbours are always in the thread's own CTA, and up / down neighbours
// are in the other CTA exactly on a band's first / last row. Sums are formed
// in the same order as ell_cluster_body. FAST: Philox noise and scalar U, F
// compiled in (omega per site allowed); otherwise both noise modes and
// per-site U, F as in ell_cluster_body.
// ------------------------------------------------------------------------
// Trajectories tr_begin, tr_begin + tr_stride, ... per cluster (both CTAs
// of a cluster pass the same values).
template <int CTA, bool FAST>
__device__ __forceinline__ void ell_cluster_pow2_body(const StepArgs& a, unsigned char* smem_raw, int64_t tr_begin,
                                                      int64_t tr_stride) {
  namespace cg = cooperative_groups;
  using T = float2;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = int(cl.block_rank());
  const int N = int(a.nsites), half = N >> 1, q = N >> 2;
  const int ny = int(a.ny), m = ny - 1;
  const int lny = __ffs(ny) - 1;
  const int rb_last = (q >> lny) - 1;  // rows per band - 1
  const float J = a.f_J, dt = a.f_dt, dt4 = a.f_dt4;
  const T rsl_s = make_float2(a.f_par[0], a.f_par[1]);
  const T iU_s = make_float2(a.f_par[2], a.f_par[3]);
  const T iF_s = make_float2(a.f_par[4], a.f_par[5]);
  constexpr uint32_t TS = uint32_t(sizeof(T));
  T* const own0 = reinterpret_cast<T*>(smem_raw);
  T* const own1 = own0 + 2 * q;
  const uint32_t oa0 = smem_addr(own0), oa1 = smem_addr(own1);
  const uint32_t pa0 = cluster_addr(oa0, uint32_t(rank ^ 1)), pa1 = cluster_addr(oa1, uint32_t(rank ^ 1));
  // slots of the peer's band edges: a band's first row looks up into the
  // peer's last row (slot q - ny + c, in the peer's high band when the site's
  // band index equals the rank), its last row down into the peer's first row
  const uint32_t up_edge[2] = {uint32_t(q - ny + (rank == 0 ? q : 0)), uint32_t(q - ny + (rank == 1 ? q : 0))};
  const uint32_t dn_edge[2] = {uint32_t(rank == 0 ? 0 : q), uint32_t(rank == 1 ? 0 : q)};
  const int lo0 = rank * q;
  const int t = threadIdx.x;
  for (int64_t tr = tr_begin; tr < a.ntraj; tr += tr_stride) {
    T* st = reinterpret_cast<T*>(a.state) + tr * N;
    const T* __restrict__ g_rsl = a.rsl ? reinterpret_cast<const T*>(a.rsl) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iU = !FAST && a.iU ? reinterpret_cast<const T*>(a.iU) + tr * a.par_stride : nullptr;
    const T* __restrict__ g_iF = !FAST && a.iF ? reinterpret_cast<const T*>(a.iF) + tr * a.par_stride : nullptr;
    const uint32_t seed = a.seeds[tr], id = a.ids[tr];
    const T* noise_tr = reinterpret_cast<const T*>(a.noise) + tr * a.noise_traj_stride;
    for (int j = t; j < q; j += CTA) {
      own0[j] = st[lo0 + j];
      own0[q + j] = st[lo0 + j + half];
    }
    cl.sync();
    int b = 0;
    bool bad = false;
    for (int64_t step = 0; step < a.nsteps; ++step) {
      const uint32_t gstep = a.step0 + uint32_t(step);
      const uint32_t cur = b ? oa1 : oa0, nxt = b ? oa0 : oa1, peer = b ? pa1 : pa0;
#pragma unroll 1
      for (int j = t; j < q; j += CTA) {
        const int pl = lo0 + j;
        const int c = j & m, rb = (j >> lny) & rb_last;
        T xi_lo, xi_hi;
        if (FAST || a.noise_mode == 0) {
          const u32x4 w = wiener_words(uint32_t(pl), gstep, seed, id);
          xi_lo = Wiener<float>::term(w.x, w.y, a);
          xi_hi = Wiener<float>::term(w.z, w.w, a);
        } else {
          const T* nz = noise_tr + int64_t(gstep) * N;
          xi_lo = Wiener<float>::buffer(nz[pl], dt4);
          xi_hi = Wiener<float>::buffer(nz[pl + half], dt4);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const uint32_t sl = uint32_t(k * q + j);        // own slot of the site
          const uint32_t row0 = sl - uint32_t(c);
          const T right = lds_c(cur + (row0 + uint32_t((c + 1) & m)) * TS, T{});
          const T left = lds_c(cur + (row0 + uint32_t((c - 1) & m)) * TS, T{});
          const T down = rb == rb_last ? ldc_c(peer + (dn_edge[k] + uint32_t(c)) * TS, T{})
                                       : lds_c(cur + (sl + uint32_t(ny)) * TS, T{});
          const T up = rb == 0 ? ldc_c(peer + (up_edge[k] + uint32_t(c)) * TS, T{})
                               : lds_c(cur + (sl - uint32_t(ny)) * TS, T{});
          const T sv = cadd(cadd(right, left), cadd(down, up));
          const T h = make_float2(J * sv.y, -J * sv.x);  // -i J s
          const int p = k ? pl + half : pl;
          const T rr = g_rsl ? __ldg(g_rsl + p) : rsl_s;
          const T uu = !FAST && g_iU ? __ldg(g_iU + p) : iU_s;
          const T ff = !FAST && g_iF ? __ldg(g_iF + p) : iF_s;
          const T v = lds_c(cur + sl * TS, T{});
          sts_c(nxt + sl * TS, local_update(v, h, rr, uu, ff, dt, 1.0f, k ? xi_hi : xi_lo));
        }
      }
      b ^= 1;
      cl.sync();
    }
    const T* fin = b ? own1 : own0;
    for (int j = t; j < q; j += CTA) {
      const T v0 = fin[j], v1 = fin[q + j];
      st[lo0 + j] = v0;
      st[lo0 + j + half] = v1;
      bad |= !finite_c(v0) || !finite_c(v1);
    }
    set_status(a.status, tr, bad);
    __syncthreads();  // the write-back reads buffer b before the next trajectory loads buffer 0
  }
}

template <int CTA, bool FAST>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(CTA, 1) ell_cluster_pow2_kernel(const StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ell_cluster_pow2_body<CTA, FAST>(a, smem_raw, blockIdx.x / 2, gridDim.x / 2);
}

template <int CTA, bool FAST>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(CTA, 1) ell_cluster_pow2_kernel_dev(const StepArgs* __restrict__ ap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  for (int i = threadIdx.x; i < int(sizeof(StepArgs) / 4); i += CTA)
    reinterpret_cast<uint32_t*>(&s_a)[i] = reinterpret_cast<const uint32_t*>(ap)[i];
  __syncthreads();
  ell_cluster_pow2_body<CTA, FAST>(s_a, smem_raw, blockIdx.x / 2, gridDim.x / 2);
}

}  // namespace twmc
