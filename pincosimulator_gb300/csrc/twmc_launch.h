// twmc_launch.h -- interface between the host API and the kernel
// translation units of libtwmc_cuda.so.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace twmc {

struct StepArgs;

// Register layout of a square-lattice FFT plan, as the host needs it to lay
// out the k-space table (last pass) and the moments (natural order).
struct PlanView {
  int nbits = 0, bx = 0, by = 0, e = 0, npass = 0, nthr = 0;
  int reg_last[8] = {0};
  int thr_last[32] = {0};
};

struct LaunchInfo {
  const char* name = "";
  int cta = 0;
  int grid = 0;
  size_t smem = 0;
  int blocks_per_sm = 0;
};

// Plans compiled into the square FFT kernel (twmc_square_*.cu).
bool square_plan(int bx, int by, PlanView* out);
int square_tpt(int bx, int by);

// Launch the square-lattice FFT step kernel. Returns false (with *err set)
// when the shape is not compiled in or the launch fails.
bool square_launch_f32(int bx, int by, const StepArgs& a, int nparams, cudaStream_t s, LaunchInfo* info,
                       std::string* err);
bool square_launch_f64(int bx, int by, const StepArgs& a, int nparams, cudaStream_t s, LaunchInfo* info,
                       std::string* err);

// Real-space (neighbour list / stencil) step kernel, any N.
bool ell_launch(int prec, const StepArgs& a, cudaStream_t s, LaunchInfo* info, std::string* err);
// FP32 fast path of the real-space kernel (twmc_ell_fast.cu): variant = index
// of the (sites per thread, threads per CTA) table.
bool ell_launch_fast_f32(const StepArgs& a, cudaStream_t s, LaunchInfo* info, std::string* err);
bool ell_prepare_fast_f32(int variant, StepArgs* a, int* grid, size_t* smem, std::string* err);
void ell_launch_dev_fast_f32(int variant, int hop, const StepArgs* dev_args, int grid, size_t smem, cudaStream_t s);

// One-off kernels (twmc_misc.cu).
struct InitArgs {
  int64_t ntraj, nsites;
  int prec;                 // 0 f32 state, 1 f64 state
  void* state;              // [ntraj][N] complex (prec)
  const uint32_t* seeds;
  const uint32_t* ids;
  int ic_kind;              // per batch (twmc_ic_kind)
  const double* binit;      // [N] complex, or NULL: binit_s
  const double* bsigma;     // [N] complex, or NULL: bsigma_s
  double binit_s[2], bsigma_s[2];
  const double* given;      // [ntraj][N] complex (ic_kind = GIVEN)
  // disorder: per matrix base [N], amp [N], kind; given realisations [ntraj][N] or NULL
  const double* base[3];    // [N] complex, or NULL: base_s
  double base_s[3][2];
  const double* amp[3];
  int kind[3];
  const double* given_real[3];
  uint32_t stream[3];
  double* real_out[3];      // [ntraj][N] complex FP64 realisations, or NULL
  // derived per-site step parameters in state precision, [ntraj][N] complex or NULL
  void* rsl;
  void* iU;
  void* iF;
  int lattice;              // 0 square, 1 Lieb
  double gamma, detuning;
};
bool init_launch(const InitArgs& a, cudaStream_t s, std::string* err);
// out[k] = double(in[k]) for k < n (in: FP32 device array).
bool widen_launch(const void* in, double* out, int64_t n, cudaStream_t s, std::string* err);

struct MomentArgs {
  int64_t ntraj, nsites;
  int prec;
  const void* state;        // [ntraj][N] complex
  const void* nk;           // [ntraj][N] real or NULL
  int nblocks;
  double* out;              // [nblocks][N][3]
};
bool moments_launch(const MomentArgs& a, cudaStream_t s, std::string* err);

bool fp32_peak(double* tflops, std::string* err);

bool wiener_launch(int prec, uint32_t seed, uint32_t id, uint32_t step0, int64_t nsteps, int64_t n, double* d_out,
                   cudaStream_t s, std::string* err);
bool philox_launch(const uint32_t* d_ctr, size_t n, uint32_t k0, uint32_t k1, uint32_t* d_out, cudaStream_t s,
                   std::string* err);

}  // namespace twmc
