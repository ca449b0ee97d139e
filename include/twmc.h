/*
 * twmc.h -- C ABI of libtwmc_cuda.so, the GB300 (sm_103a) Truncated Wigner
 * Monte Carlo trajectory engine.
 *
 * It replaces the per-trajectory hot path of the reference's TWMC solvers
 * (paths relative to the PincoSimulator project root):
 *   - TWMCBaseSolver::Compute  src/TWMC/Solvers/TWMCBaseSolver.cpp:94-283
 *     (1-D chain / 2-D square lattice, FFT hopping, Euler-Maruyama step)
 *   - TWMCLiebSolver::Compute  src/TWMC/Solvers/TWMCLiebSolver.cpp:109-299
 *     (1-D Lieb lattice, real-space coupling, optional F(t))
 * behind the reference's plugin interface Solver::Setup/Compute/
 * ApproximateComputationProgress (src/Base/Solver.hpp:16-31). A C++ Solver
 * subclass (pincosimulator_gb300/host) or any FFI caller packs the reference's
 * TWMCTaskData into twmc_task_desc and calls twmc_run.
 *
 * Conventions
 *   - Complex arrays are interleaved doubles (re, im), i.e. the memory layout
 *     of std::complex<double> / the reference's complex_p.
 *   - Site order is the reference's row-major MatrixCXd order: site
 *     p = i * ny + j on an nx x ny lattice after TWMCSystemData's 1-D swap
 *     (a chain is nx = 1, ny = N; TWMCSystemData.cpp:25-37); on the Lieb
 *     lattice p = 3 * cell + {0:A, 1:B, 2:C}.
 *   - All buffers are owned by the caller. Return codes: 0 = OK, < 0 error.
 *     No C++ exception crosses this boundary.
 *   - A handle is not internally synchronised: calls on one handle must be
 *     serialised by the caller; different handles are independent.
 */
#ifndef TWMC_H
#define TWMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TWMC_ABI_VERSION 3

#if defined(__GNUC__)
#define TWMC_API __attribute__((visibility("default")))
#else
#define TWMC_API
#endif

enum twmc_status {
  TWMC_OK = 0,
  TWMC_ERR_INVALID = -1,     /* bad argument / unsupported combination */
  TWMC_ERR_CUDA = -2,        /* CUDA runtime error (message in twmc_last_error) */
  TWMC_ERR_TIMEOUT = -3,     /* a bounded device-side wait gave up */
  TWMC_ERR_NONFINITE = -4,   /* a trajectory became NaN/Inf (per-task status) */
  TWMC_ERR_NOMEM = -5,       /* device allocation failed */
  TWMC_ERR_NOT_BUILT = -6    /* the kernel variant for this shape is not compiled in */
};

enum twmc_lattice {
  TWMC_LATTICE_SQUARE = 0, /* 1-D chain or 2-D square lattice (TWMCBaseSolver) */
  TWMC_LATTICE_LIEB = 1    /* 1-D Lieb lattice, 3 sites per cell (TWMCLiebSolver) */
};

enum twmc_precision { TWMC_PREC_F32 = 0, TWMC_PREC_F64 = 1 };

enum twmc_noise_mode {
  TWMC_NOISE_PHILOX = 0, /* in-kernel Philox4x32-10: Wiener increments with a fixed key and counter
                            (site pair, step, id, seed); initial fields and disorder keyed by (seed, id),
                            counter (site pair, 0, stream, 0) */
  TWMC_NOISE_BUFFER = 1  /* caller-supplied Wiener increments (deterministic-noise mode) */
};

enum twmc_hop_mode {
  TWMC_HOP_FFT = 0,     /* square lattice: on-chip FFT, k-space multiply, inverse FFT (the reference's algorithm) */
  TWMC_HOP_STENCIL = 1  /* square lattice: the same operator applied in real space (nearest neighbours) */
};

enum twmc_integrator {
  TWMC_INTEGRATOR_EULER = 0, /* the reference's step (TWMCBaseSolver.cpp:232-266): the hopping h = IFFT(-i 2J c_k
                                FFT(beta)) / N enters the Euler-Maruyama increment with the local terms */
  TWMC_INTEGRATOR_SPLIT = 1  /* exponential split step: beta' = IFFT(exp(-i 2J c_k dt) FFT(beta)) / N (the
                                hopping integrated exactly over dt), then the Euler-Maruyama local step on beta'
                                (square lattice, FFT path only) */
};

enum twmc_ic_kind {
  TWMC_IC_SETTINGS = 0,  /* ReadFromSettings: beta = beta_init + beta_init_sigma * xi (xi from the init stream) */
  TWMC_IC_FIXED = 1,     /* FixedPoint: beta = beta_init */
  TWMC_IC_GIVEN = 2      /* ReadFromPreviousData / caller-given field: beta = init_field */
};

enum twmc_noise_kind { TWMC_DISORDER_NONE = 0, TWMC_DISORDER_GAUSSIAN = 1, TWMC_DISORDER_UNIFORM = 2 };

/* One noisy parameter matrix (NoisyMatrix, src/Base/NoisyMatrix.cpp:118-162):
 * value = base + noise, noise drawn per trajectory on its own Philox stream. */
typedef struct twmc_matrix {
  const double* base;      /* n_sites complex; NULL = all zero */
  int32_t noise_kind;      /* twmc_noise_kind */
  const double* noise_amp; /* n_sites complex amplitudes (Re scales the real draw, Im the imaginary) */
} twmc_matrix;

typedef struct twmc_system_desc {
  int32_t lattice;     /* twmc_lattice */
  int64_t nx, ny;      /* lattice (Lieb: cells = nx * ny, sites = 3 * cells) */
  int32_t pbc;         /* Lieb: periodic boundary (the square lattice is always periodic) */
  double J;            /* square lattice hopping */
  double J_AB, J_BC;   /* Lieb couplings */
  double gamma;        /* loss rate */
  double detuning;     /* Lieb: delta = detuning - E */
  double dt;           /* timestep */
  int64_t frame_steps; /* steps between saved frames (TWMCSystemData::frame_steps) */
  twmc_matrix omega;   /* square: omega; Lieb: E */
  twmc_matrix U;
  twmc_matrix F;
  twmc_matrix beta_init;
  twmc_matrix beta_init_sigma;
  /* Optional F(t) table (NoisyMatrix::SetTemporalValue): ft_nrec records at
   * ft_times (ascending), ft_values = ft_nrec x n_sites complex; NaN entries
   * are gap-filled as the reference does. Lieb lattice only. */
  int64_t ft_nrec;
  const double* ft_times;
  const double* ft_values;
  int32_t precision;   /* twmc_precision */
  int32_t noise_mode;  /* twmc_noise_mode */
  int32_t hop_mode;    /* twmc_hop_mode (square lattice) */
  int32_t n_moment_blocks; /* ensemble blocks for standard errors (0 = 32) */
  /* Square lattice: accumulate the drive's work and area per site between
   * saves (TWMCThermoSolver.cpp:203-236, the solver the reference's manager
   * selects for a periodic lattice with F(t), TWMCManager.cpp:47-58):
   *   work += 2 dt Re(b) dF/dt,  area += dt dF/dt (|b|^2 - 1/2),
   *   dF/dt = Re(F(t) - F(t - dt)) / dt (0 on a run's first step),
   * b the field after the step. Runs on the real-space kernel. */
  int32_t thermo;
  int32_t integrator;  /* twmc_integrator (TWMC_INTEGRATOR_SPLIT needs the FFT path: square lattice, hop_mode
                          FFT, power-of-two sides of a compiled plan, no F(t), no work / area) */
} twmc_system_desc;

typedef struct twmc_task_desc {
  uint64_t id;            /* TWMCTaskData::id (low 32 bits enter the Philox key / counter) */
  uint32_t seed;          /* TWMCTaskData::rngSeed (Philox key / counter word) */
  int32_t ic_kind;        /* twmc_ic_kind */
  double t_start, t_end;  /* TWMCTaskData::t_start / t_end */
  int32_t store_initial;  /* TWMCTaskData::storeInitialState */
  const double* init_field; /* TWMC_IC_GIVEN: n_sites complex */
  const double* U_realization;     /* optional given disorder realisations (n_sites complex), e.g. */
  const double* omega_realization; /* on continuation (TWMCBaseSolver.cpp:185-199); NULL = draw */
  const double* F_realization;
} twmc_task_desc;

typedef struct twmc_outputs {
  double* frames;          /* optional: n_tasks x n_frames x n_sites complex128 (the "traj" dataset) */
  double* final_field;     /* optional: n_tasks x n_sites complex */
  double* U_realization;   /* optional: n_tasks x n_sites complex (U_Realization dataset) */
  double* omega_realization; /* optional: n_tasks x n_sites complex (Omega_Realization dataset) */
  double* F_realization;   /* optional: n_tasks x n_sites complex (F_Realizatio dataset) */
  double* moments;         /* optional: n_frames x n_moment_blocks x n_sites x 3 FP64 sums of
                              |a|^2, |a|^4 and |a_k|^2 (unitary FFT; 0 on the Lieb lattice) */
  int64_t* frames_written; /* optional: n_tasks (frames actually produced) */
  double* t_final;         /* optional: n_tasks (extraDataMemory[1]) */
  int32_t* status;         /* optional: n_tasks (0 or TWMC_ERR_NONFINITE) */
  double* work;            /* optional (thermo): n_tasks x n_frames x n_sites float64 ("work" dataset),
                              accumulated since the previous saved frame (0 for an initial frame) */
  double* area;            /* optional (thermo): same layout ("area" dataset) */
} twmc_outputs;

typedef struct twmc_handle twmc_handle;

/* Version of this ABI (TWMC_ABI_VERSION). */
TWMC_API int twmc_version(void);

/* Builds a solver for one system (TWMCBaseSolver::Setup / TWMCLiebSolver::Setup,
 * TWMCBaseSolver.cpp:24-92, TWMCLiebSolver.cpp:29-104): uploads the k-space
 * table or coupling, parameters and F(t) table, selects the kernel. */
TWMC_API int twmc_create(const twmc_system_desc* desc, twmc_handle** out);

/* Runs n tasks to completion (Solver::Compute, Solver.hpp:22). Tasks are
 * grouped by (t_start, t_end, store_initial) and each group runs as one
 * batch on the GPU. Outputs are written in task order. */
TWMC_API int twmc_run(twmc_handle* h, const twmc_task_desc* tasks, size_t n, twmc_outputs* out);

/* Deterministic-noise mode: Wiener increments for the next twmc_run, laid out
 * [task][step][site] complex (the reference's randCMat draws,
 * TWMCBaseSolver.cpp:285-291). count = number of complex values. The buffer is
 * copied; steps beyond the supplied range are an error. */
TWMC_API int twmc_set_noise_buffer(twmc_handle* h, const double* xi, size_t count);

/* Fraction of the current/last twmc_run completed (ApproximateComputationProgress). */
TWMC_API int twmc_progress(const twmc_handle* h, double* fraction);

/* Message of the last error on this handle ("" if none). */
TWMC_API const char* twmc_last_error(const twmc_handle* h);

TWMC_API void twmc_destroy(twmc_handle* h);

/* ---- device-resident batch API (inputs and state stay in HBM) ---------- */

/* Allocates and initialises a device batch of n trajectories for the tasks
 * (initial fields and disorder drawn on the GPU). */
TWMC_API int twmc_batch_init(twmc_handle* h, const twmc_task_desc* tasks, size_t n);
/* Advances the batch by n_steps steps (asynchronous on the handle's stream). */
TWMC_API int twmc_batch_advance(twmc_handle* h, int64_t n_steps);
/* Reduces the current batch state into FP64 moment blocks (asynchronous). */
TWMC_API int twmc_batch_reduce(twmc_handle* h);
/* Waits for the handle's stream; *kernel_ms = summed device time of the
 * trajectory-step launches since the last call (may be NULL), including those
 * of twmc_run calls made since then. */
TWMC_API int twmc_sync(twmc_handle* h, double* kernel_ms);
/* Copies the batch state (n x n_sites complex128) and/or the last moment
 * blocks (n_moment_blocks x n_sites x 3) to host memory; NULL skips. */
TWMC_API int twmc_batch_download(twmc_handle* h, double* field, double* moments);
/* Kernel launches issued by this handle since creation (trajectory steps,
 * reductions, initialisation). */
TWMC_API int64_t twmc_launch_count(const twmc_handle* h);
/* Name of the step kernel variant the handle selected: "square_fft_kernel"
 * (register FFT; "square_fft_kernel<fast>" for its compiled-in common run:
 * FP32, Philox noise, scalar U and F; "square_fft_kernel<fast,split>" the same
 * with the split-step integrator), "ell_kernel<stencil>" / "ell_kernel<table>" (real space,
 * square stencil / Lieb neighbour table), "rowrun_kernel" (square stencil,
 * 4096 sites, FP32 Philox runs), "lieb_cell_kernel" (Lieb lattice, even
 * number of cells), "ell_cluster_pow2_kernel" / "ell_cluster_kernel" (square
 * stencil above 8192 sites on 2-CTA clusters). Kernels chosen at launch time
 * are reported after the first step. */
TWMC_API const char* twmc_kernel_name(const twmc_handle* h);
/* The CUDA stream (cudaStream_t) all of the handle's work is issued on, for
 * callers that order their own work or record events against it. */
TWMC_API void* twmc_stream(const twmc_handle* h);

/* FP32 FMA throughput of the current device in TFLOP/s, measured with a
 * register-resident FMA chain over all SMs (the CUDA-core roofline of the
 * step kernels). */
TWMC_API int twmc_measure_fp32_peak(double* tflops);

/* ---- heterogeneous batch -------------------------------------------------- */

/* One parameter point of a heterogeneous batch: a periodic square lattice
 * (nx = 1 for a chain) with uniform complex parameters, n_traj trajectories
 * with seeds seed0 + k and ids id0 + k, vacuum-style initial fields
 * beta_init + beta_init_sigma * xi (TWMC_IC_SETTINGS), FP32 state. */
typedef struct twmc_point_desc {
  int64_t nx, ny;
  double J, gamma, dt;
  double omega[2], U[2], F[2];       /* complex values (re, im) */
  double beta_init[2], beta_init_sigma[2];
  int64_t n_traj;
  uint32_t seed0;
  uint64_t id0;
  int32_t n_moment_blocks;           /* 0 = 32 (capped at n_traj) */
} twmc_point_desc;

typedef struct twmc_hbatch twmc_hbatch;

/* Builds a batch of n points advanced together frame by frame. Every point
 * takes one step variant -- "fft" (register FFT: chains of 32..1024 sites,
 * 16x16, 32x32, 64x64), "ell2" / "ell4" / "ell8" (real-space stencil with 2,
 * 4, 8 sites per thread, 256-thread CTAs, up to 512 / 1024 / 2048 sites),
 * "rowrun" (runs of four sites along a row, 512-thread CTAs, ny a multiple
 * of 4, up to 4096 sites), "ell8w" (8 sites per thread, 512-thread CTAs, up
 * to 4096 sites), "cluster_pow2" / "cluster" (2-CTA clusters, 4097..16384
 * sites; the power-of-two form for N = 2^k, ny a power of two <= N/4) --
 * and every (point, trajectory group) is a work item of a persistent
 * work-queue kernel for its CTA geometry, taken from an atomic counter,
 * longest items first. One frame (frame_steps steps of every point, FP64
 * moment blocks, counters) is captured into a CUDA graph. tune: 0 = the
 * default variant per shape (FFT where a plan exists, else row runs on
 * 4096-site lattices, the fullest real-space stencil, or the cluster form);
 * 1 = per shape, time every variant the shape admits once on a trial batch
 * and keep the fastest (cached in $TWMC_TUNE_CACHE or
 * ~/.cache/twmc_tune.json). */
TWMC_API int twmc_hbatch_create(const twmc_point_desc* points, size_t n, int64_t frame_steps, int32_t tune,
                                twmc_hbatch** out);
/* The same with the step variant of every point given by name (variants[i],
 * one of the names above); a variant the point's lattice does not admit
 * returns TWMC_ERR_INVALID. */
TWMC_API int twmc_hbatch_create_variants(const twmc_point_desc* points, size_t n, int64_t frame_steps,
                                         const char* const* variants, twmc_hbatch** out);
/* Replays the frame graph n_frames times (asynchronous). */
TWMC_API int twmc_hbatch_run(twmc_hbatch* b, int64_t n_frames);
/* Waits for the batch; *ms = device time of the last twmc_hbatch_run. */
TWMC_API int twmc_hbatch_sync(twmc_hbatch* b, double* ms);
/* Last frame's moment blocks of one point (n_blocks x sites x 3 doubles). */
TWMC_API int twmc_hbatch_moments(twmc_hbatch* b, size_t point, double* out);
/* Current field of one point (n_traj x sites complex128). */
TWMC_API int twmc_hbatch_state(twmc_hbatch* b, size_t point, double* out);
/* Redraws one point's initial fields from per-site device arrays (sites
 * complex128 each, NULL = the point's uniform value): a = beta_init +
 * beta_sigma * (xi1 + i xi2) with the same Philox draws as at creation. Only
 * before the first twmc_hbatch_run (e.g. warm starts from predicted fields). */
TWMC_API int twmc_hbatch_set_init(twmc_hbatch* b, size_t point, const double* beta_init, const double* beta_sigma);
/* Trajectory means <a> (complex128) and <|a|^2> (double) per site of every
 * point into device arrays of twmc_hbatch_total_sites entries (point i's
 * sites follow point i-1's), FP64 compensated, on the batch's stream
 * (asynchronous); accumulate != 0 adds to the arrays instead. */
TWMC_API int twmc_hbatch_field_moments(twmc_hbatch* b, double* mean, double* abs2, int32_t accumulate);
TWMC_API int64_t twmc_hbatch_total_sites(const twmc_hbatch* b);
/* Site averages of the last frame's moment blocks of every point into host
 * out [sum_i n_blocks_i][3] (point i's blocks follow point i-1's): the
 * inputs of spatially averaged n, g2 with block standard errors per frame,
 * without copying whole moment arrays. Synchronises. */
TWMC_API int twmc_hbatch_block_means(twmc_hbatch* b, double* out);
/* cudaStream_t the batch runs on. */
TWMC_API void* twmc_hbatch_stream(const twmc_hbatch* b);
/* Kernel the point runs on. */
TWMC_API const char* twmc_hbatch_plan(const twmc_hbatch* b, size_t point);
TWMC_API const char* twmc_hbatch_last_error(const twmc_hbatch* b);
TWMC_API int64_t twmc_hbatch_launch_count(const twmc_hbatch* b);
TWMC_API void twmc_hbatch_destroy(twmc_hbatch* b);

/* ---- allocation-free entry point ------------------------------------------ */

/* k-space populations and FP64 moment blocks of a caller-owned device batch,
 * without allocating any device memory. It has no counterpart in the
 * reference. It is for callers that cannot allocate device memory: a host
 * application whose own pool already owns the device, or a latency-critical
 * loop where cudaMalloc's implicit synchronisation is not acceptable. It
 * computes what twmc_batch_reduce returns after a twmc_batch_advance:
 *   moments[b][p] = sums over trajectories [b T/B, (b+1) T/B) of
 *                   (|a_p|^2, |a_p|^4, |FFT(a)_p|^2 / N)
 * state:    device pointer, n_traj x nx*ny complex64 (interleaved floats),
 *           site order as everywhere in this ABI; nx, ny powers of two of a
 *           compiled square-lattice plan (1 x 32..4096, 16x16, 32x32, 64x64)
 * moments:  device pointer, n_blocks x nx*ny x 3 doubles (fully written)
 * stream:   cudaStream_t to run on (NULL = default stream)
 * Limit: n_traj * nx * ny <= 4194304 (the 16 MiB scratch array that every
 * device loading the library holds until the process exits); larger sizes,
 * unsupported shapes and null pointers return TWMC_ERR_INVALID.
 * Calls outside stream capture look up the scratch array's device address
 * (cudaGetSymbolAddress, with the device current) and remember it; a call
 * during capture uses the remembered address, so the first call on a device
 * -- and the first after a cudaDeviceReset -- must come before any stream
 * capture (a first call under capture returns TWMC_ERR_CUDA). All calls share
 * the one scratch array: calls that overlap on the GPU (different streams, or
 * host threads without ordering) race. The call allocates nothing and does
 * not synchronise. */
TWMC_API int twmc_kspace_moments_noalloc(const void* state, int64_t n_traj, int64_t nx, int64_t ny,
                                         int32_t n_blocks, double* moments, void* stream);

/* ---- learned warm start --------------------------------------------------- */

/* A multilayer perceptron with BF16 weights and FP32 accumulation on the
 * tensor cores, GELU after every hidden layer, trained with MSE loss and
 * Adam. No counterpart in the reference. It maps a parameter point to an
 * MLP row: (Re a_k, Im a_k) of the steady-state k-mode mean field for every
 * k (natural order k = kx ny + ky, unitary DFT), then the density n.
 * Parameters form one FP32 array: for each layer l, W_l [widths[l+1]]
 * [widths[l]] row-major, then b_l [widths[l+1]]. Pointers named x, y,
 * target, weights, rows, mean, abs2, beta_* are DEVICE pointers; calls taking
 * a stream are asynchronous on it. */
typedef struct twmc_mlp twmc_mlp;

/* widths[0..n_layers]; Glorot-uniform weights from seed, zero biases;
 * max_batch = rows per backward call (forward calls are chunked). */
TWMC_API int twmc_mlp_create(int32_t n_layers, const int32_t* widths, int64_t max_batch, uint64_t seed,
                             twmc_mlp** out);
TWMC_API int64_t twmc_mlp_param_count(const twmc_mlp* m);
/* Host copies of the FP32 parameters (set also resets Adam) and gradients. */
TWMC_API int twmc_mlp_set_params(twmc_mlp* m, const float* host);
TWMC_API int twmc_mlp_get_params(twmc_mlp* m, float* host);
TWMC_API int twmc_mlp_get_grads(twmc_mlp* m, float* host);
/* y [batch][widths[n]] = net(x [batch][widths[0]]). */
TWMC_API int twmc_mlp_forward(twmc_mlp* m, const float* x, int64_t batch, float* y, void* stream);
/* Forward + gradients of L = sum_{b,o} w_o (y - target)^2 / (batch O) into
 * the gradient array (weights: [O] or NULL = 1); *loss (host, optional:
 * NULL keeps the call asynchronous) receives L. */
TWMC_API int twmc_mlp_backward(twmc_mlp* m, const float* x, const float* target, const float* weights,
                               int64_t batch, float* loss, void* stream);
/* One Adam step from the current gradients. */
TWMC_API int twmc_mlp_adam(twmc_mlp* m, float lr, float beta1, float beta2, float eps, void* stream);
/* L of the last backward (synchronises). */
TWMC_API int twmc_mlp_last_loss(twmc_mlp* m, float* loss);
TWMC_API const char* twmc_mlp_last_error(const twmc_mlp* m);
TWMC_API int64_t twmc_mlp_launch_count(const twmc_mlp* m);
TWMC_API void twmc_mlp_destroy(twmc_mlp* m);
/* Prepares training rows t [rows][cols] in place: squash each value to
 * asinh(v / squash) when squash > 0 (log-like beyond |v| ~ squash), then
 * standardise every column (mean, stdv per column; the deviation floored at
 * floor_frac x its maximum over columns). weights (optional, [cols]): loss
 * weights clamp((stdv_c / max stdv)^2, 1e-4, 1) from the unfloored
 * deviations, so columns that barely vary across points (k-modes that vanish
 * by symmetry, up to noise) do not dominate the loss. */
TWMC_API int twmc_mlp_standardize(float* t, int64_t rows, int32_t cols, double squash, float floor_frac, float* mean,
                                  float* stdv, float* weights, void* stream);
/* MLP rows [n_points][ld] (ld >= 2 nx ny + 1) from per-point sums over
 * `frames` frames of the mean field (complex128, [n_points][nx ny]) and of
 * <|a|^2> ([n_points][nx ny]), e.g. from twmc_hbatch_field_moments. */
TWMC_API int twmc_mlp_targets(const double* mean, const double* abs2, int64_t n_points, int64_t nx, int64_t ny,
                              int32_t frames, float* rows, int64_t ld, void* stream);
/* Initial fields from MLP rows (de-standardised with mean / stdv when not
 * NULL, then un-squashed with squash as above): beta_init = inverse DFT of
 * the predicted amplitudes, beta_sigma = sqrt((n_inc + 1/2) / 2) per
 * quadrature with n_inc = min(max(n - |beta_init|^2, 0), max_incoherent)
 * (complex128, [n_points][nx ny] each), the inputs of twmc_hbatch_set_init.
 * nx ny <= 4096. */
TWMC_API int twmc_mlp_fields(const float* rows, int64_t ld, int64_t n_points, const float* mean, const float* stdv,
                             double squash, double max_incoherent, int64_t nx, int64_t ny, double* beta_init,
                             double* beta_sigma, void* stream);

/* ---- self-check entry points -------------------------------------------- */

/* Philox4x32-10 evaluated on the GPU for n counters (ctr: n x 4, key: 2 words),
 * out: n x 4 words. */
TWMC_API int twmc_debug_philox(const uint32_t* ctr, size_t n, const uint32_t* key, uint32_t* out);

/* The complex Wiener normals xi of one trajectory exactly as the step kernels
 * draw them in Philox mode (twmc_system_desc.noise_mode = TWMC_NOISE_PHILOX),
 * for steps step0 .. step0 + n_steps - 1 of an n_sites lattice, in the run's
 * precision (TWMC_PREC_F32: the FP32 Box-Muller, widened exactly):
 * out[(k * n_sites + p) * 2 + {0,1}] = Re, Im of xi at step step0 + k, site p.
 * The per-step draw of randCMat (TWMCBaseSolver.cpp:285-291), as a device
 * self-check: a caller can replay a Philox-mode trajectory through any
 * deterministic-noise implementation with these values. */
TWMC_API int twmc_debug_wiener(int32_t precision, uint32_t seed, uint64_t id, uint32_t step0, int64_t n_steps,
                               int64_t n_sites, double* out);

#ifdef __cplusplus
}
#endif

#endif /* TWMC_H */
