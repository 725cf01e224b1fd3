/*
 * nlm_capi.h -- C ABI of the GB300 split-step propagation engine.
 *
 * This is the drop-in boundary for the propagation path of the `nonlinearmedium`
 * module of MultimodeNonlinearOptics.  Every entry point below replaces one method of
 * the reference's pybind11 API (src/nlmModulePy.cpp) and is what a binding of that
 * API binds to (the Python binding shipped with this library is a ctypes layer over
 * these functions).
 *
 * Conventions
 *  - Complex arrays are interleaved double pairs (re, im), i.e. numpy complex128,
 *    row-major, in FFT order exactly like the reference (src/_NonlinearMedium.cpp:121-124).
 *  - All host buffers are owned by the caller; device buffers are owned by the handle.
 *  - Every function returns an nlm_status.  On error, nlm_last_error() returns a
 *    thread-local message.  NLM_ERR_INVALID_ARGUMENT corresponds to the reference's
 *    std::invalid_argument (Python ValueError), NLM_ERR_RUNTIME to std::runtime_error
 *    (RuntimeError), NLM_ERR_INDEX to std::out_of_range (IndexError).
 *  - A handle is not thread-safe; different handles may be used from different threads.
 *  - No call falls back to a CPU implementation: a call that needs the GPU returns
 *    NLM_ERR_NO_DEVICE when no CUDA device is usable.
 */
#ifndef NLM_CAPI_H
#define NLM_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nlm_status {
  NLM_OK = 0,
  NLM_ERR_INVALID_ARGUMENT = 1, /* reference: std::invalid_argument -> ValueError        */
  NLM_ERR_RUNTIME = 2,          /* reference: std::runtime_error     -> RuntimeError      */
  NLM_ERR_INDEX = 3,            /* reference: std::out_of_range      -> IndexError        */
  NLM_ERR_CUDA = 4,             /* CUDA runtime error                                     */
  NLM_ERR_NO_DEVICE = 5,        /* no usable CUDA device: there is no CPU fallback        */
  NLM_ERR_UNSUPPORTED = 6,      /* a grid size this engine does not implement             */
  NLM_ERR_TIMEOUT = 7           /* a bounded device-side wait gave up                     */
} nlm_status;

typedef struct nlm_medium nlm_medium;   /* one solver instance (or a Cascade)            */

/* Pulse and intensity-profile enums, same values as src/_NonlinearMedium.hpp:25-34. */
enum { NLM_GAUSSIAN = 0, NLM_SECH = 1, NLM_SINC = 2 };
enum { NLM_GAUSSIAN_BEAM = 0, NLM_CONSTANT = 1, NLM_GAUSSIAN_APODIZATION = 2 };

/* Last error message of the calling thread (never NULL). */
const char* nlm_last_error(void);

/* Library version string. */
const char* nlm_version(void);

/* Number of registered solvers and their names, in the order of
 * solvers/RegisteredSolvers.hpp:1-16. */
int nlm_solver_count(void);
const char* nlm_solver_name(int index);
/* Scalar constructor arguments of a solver, in the reference's positional order with
 * the array arguments (customPump, poling) removed.  Names are separated by ',' and
 * each carries its default after '=' when it has one; "inf" denotes infinity. */
const char* nlm_solver_signature(const char* solver);

/* --- construction (solver ctors, e.g. solvers/Chi2PDC.cpp:18-24 and their py::init,
 *     solvers/Chi2PDC.cpp:51-60; base ctor src/_NonlinearMedium.cpp:8-40) ------------ */
/* args: the solver's scalar constructor arguments in nlm_solver_signature order
 * (enums and integers passed as doubles).  custom_pump: N complex values or NULL/0.
 * poling: domain lengths or NULL/0.  Host-side setup only: no device is touched. */
nlm_status nlm_create(const char* solver, const double* args, size_t nargs,
                      const double* custom_pump, size_t n_custom_pump,
                      const double* poling, size_t n_poling, nlm_medium** out);
nlm_status nlm_destroy(nlm_medium* medium);

/* Solver properties. */
nlm_status nlm_info(const nlm_medium* m, int* n_signal_modes, int* n_pump_modes,
                    int* n_freqs, int* n_z_steps, int* n_z_steps_p, int* fully_nonlinear,
                    int* is_cascade);
/* dz, dzp, z, tMax (src/_NonlinearMedium.hpp:94-100). */
nlm_status nlm_lengths(const nlm_medium* m, double* z, double* dz, double* dzp, double* t_max);

/* --- setPump overloads (src/_NonlinearMedium.cpp:180-222, 506-534) ---------------- */
nlm_status nlm_set_pump_type(nlm_medium* m, int pulse_type, double chirp, double delay,
                             unsigned pump_index);
nlm_status nlm_set_pump_custom(nlm_medium* m, const double* custom_pump, size_t n,
                               double chirp, double delay, unsigned pump_index);
nlm_status nlm_set_pump_from(nlm_medium* m, const nlm_medium* other, unsigned mode_index,
                             double delay, unsigned pump_index);

/* --- runPumpSimulation (src/_NonlinearMedium.cpp:225-250, solvers/Chi3.cpp:41-70) ---- */
nlm_status nlm_run_pump(nlm_medium* m);

/* --- runSignalSimulation (src/_NonlinearMedium.cpp:253-260) --------------------------
 * Fills the handle's signal grids (nZSteps x N per mode); read them with nlm_get_grid. */
nlm_status nlm_run_signal(nlm_medium* m, const double* input_prof, size_t n,
                          int in_time_domain, unsigned input_mode);

/* --- computeGreensFunction (src/_NonlinearMedium.cpp:263-375) ------------------------
 * use_input/use_output: 0/1 lists (may be NULL/0 for "all modes").  First call
 * nlm_green_dims to validate and obtain the matrix shape (rows x cols), then nlm_green
 * with caller buffers of rows*cols complex values each.  n_threads is accepted for API
 * parity and validated like the reference; the work runs on the GPU.                  */
nlm_status nlm_green_dims(nlm_medium* m, unsigned n_threads, const uint8_t* use_input,
                          size_t n_use_input, const uint8_t* use_output, size_t n_use_output,
                          size_t* rows, size_t* cols);
nlm_status nlm_green(nlm_medium* m, int in_time_domain, int run_pump, unsigned n_threads,
                     int normalize, const uint8_t* use_input, size_t n_use_input,
                     const uint8_t* use_output, size_t n_use_output, double* green_c,
                     double* green_s);
/* Same computation with C and S written to DEVICE memory (CUDA pointers on the
 * handle's device), for callers that keep the matrices resident in HBM. */
nlm_status nlm_green_device(nlm_medium* m, int in_time_domain, int run_pump, unsigned n_threads,
                            int normalize, const uint8_t* use_input, size_t n_use_input,
                            const uint8_t* use_output, size_t n_use_output, void* green_c_dev,
                            void* green_s_dev);

/* --- computeGreensFunction split over several GPUs ------------------------------------------
 * The 2 N nSignalModes impulse propagations of computeGreensFunction (all modes, as with empty
 * useInput/useOutput) are independent: src/_NonlinearMedium.cpp:350-353 splits them over threads in
 * contiguous ranges; nlm_green_rows computes the raw last-row outputs (nSignalModes N complex each) of
 * the range [first, first + count) on this handle's GPU, nlm_green_finish turns the gathered raw
 * rows of all propagations into C and S (src/_NonlinearMedium.cpp:329-345, 360-372). */
nlm_status nlm_green_rows(nlm_medium* m, int in_time_domain, int run_pump, size_t first, size_t count,
                          double* raw_out);
nlm_status nlm_green_finish(nlm_medium* m, const double* raw, int normalize, double* green_c,
                            double* green_s);
/* The same two steps on device memory of the handle's GPU (row-major complex128, the layouts above):
 * the rows are written, and C and S computed, in place on the device, so that a gather between the
 * GPUs (NCCL) reads and writes device buffers with no host round trip.  Both return after the work
 * on the handle's stream has finished.  No counterpart in the reference (its threads share memory). */
nlm_status nlm_green_rows_device(nlm_medium* m, int in_time_domain, int run_pump, size_t first, size_t count,
                                 void* raw_out_dev);
nlm_status nlm_green_finish_device(nlm_medium* m, const void* raw_dev, int normalize, void* green_c_dev,
                                   void* green_s_dev);

/* --- batchSignalSimulation (src/_NonlinearMedium.cpp:378-444;
 *     src/_FullyNonlinearMedium.hpp:8-11 where run_pump is ignored) -------------------
 * inputs: rows x cols complex.  Output: rows x (nOut*N) complex; nlm_batch_dims gives
 * nOut*N.                                                                              */
nlm_status nlm_batch_dims(nlm_medium* m, size_t rows, size_t cols, unsigned n_threads,
                          unsigned input_mode, const uint8_t* use_output, size_t n_use_output,
                          size_t* out_cols);
nlm_status nlm_batch(nlm_medium* m, const double* inputs, size_t rows, size_t cols,
                     int in_time_domain, int run_pump, unsigned n_threads, unsigned input_mode,
                     const uint8_t* use_output, size_t n_use_output, double* out);
/* Device-resident variant: inputs and outputs are CUDA pointers. */
nlm_status nlm_batch_device(nlm_medium* m, const void* inputs_dev, size_t rows, size_t cols,
                            int in_time_domain, int run_pump, unsigned n_threads,
                            unsigned input_mode, const uint8_t* use_output, size_t n_use_output,
                            void* out_dev);

/* --- ragged batch: several media, one seeded signal each, one call ----------------
 * No counterpart method in the reference (it would loop over media calling
 * batchSignalSimulation one row at a time, src/_NonlinearMedium.cpp:378-444).
 * inputs[k] is an N_k complex row for media[k]; outputs[k] receives the last row of all
 * signal modes (nSignalModes_k*N_k complex).  Pumps must have been run.  The call plans
 * each medium's form (one SM in a ragged launch, or a cluster of 4 or 8 SMs) for the
 * shortest makespan and runs as one CUDA graph, replayed while the plan stays the same. */
nlm_status nlm_ragged_batch(nlm_medium* const* media, size_t n_media, const double* const* inputs,
                            int in_time_domain, double* const* outputs);
/* nlm_ragged_batch's makespan planner alone, with no device work: n_media media given by their grid
 * (n_freqs), signal mode count, nZSteps, whether the RK4 propagator matrices are used (propagator),
 * ragged-launch class (media of one class share a launch: one solver and one grid) and available
 * forms (bit 0: one SM in a ragged launch, bits 1-3: clusters of 4, 8 and 16 SMs); the SMs that
 * cluster slots may use, the sixteen-SM slots that can run at once, the SMs for slots and ragged
 * launches together and the ragged CTAs' granularity, as nlm_ragged_batch measures them.  Outputs: the
 * makespan the plan was made for (microseconds; -1 when no plan fits the SMs at once, the slots then
 * queueing), per medium its form (0-3) and cluster slot (-1: a ragged launch; a slot's media run one
 * after another), the ragged launches' CTAs, and (times_us, n_media x 4) each medium's estimated
 * march time in each form (microseconds, -1 where the form is not available), from the engine's
 * GB300 per-step table.  No counterpart in the reference (scheduling support). */
nlm_status nlm_ragged_plan(size_t n_media, const unsigned* n_freqs, const unsigned* n_modes,
                           const unsigned* n_z_steps, const int* propagator, const int* launch_class,
                           const unsigned* forms, int cluster_sms, int w16_slots, int pool_sms,
                           int pool_granularity, double* makespan_us, int* form, int* slot,
                           int* ragged_ctas, double* times_us);
/* The plan of the last nlm_ragged_batch call: its estimated makespan (microseconds), the cluster
 * slots of four, eight and sixteen SMs, the CTAs of its one-SM ragged launches, the CUDA-graph
 * captures and replays of ragged calls so far, the SMs the plan could use (those clusters of four can
 * hold at once; the environment variable NLM_RAGGED_CLUSTER_SMS overrides the measured figure) and
 * the sixteen-SM slots that can run at once (NLM_RAGGED_W16_SLOTS overrides it; 0 when no medium of
 * the call has that form), and the call's device time (milliseconds, CUDA events on its stream around
 * the enqueued work).  No counterpart in the reference (measurement support). */
nlm_status nlm_ragged_last_plan(double* makespan_estimate_us, int* slots_c4, int* slots_w8, int* slots_w16,
                                int* ragged_ctas, long* graph_captures, long* graph_replays, int* sm_budget,
                                int* w16_capacity, double* gpu_ms);

/* --- gradients (no counterpart in the reference) -------------------------------------------
 * Reverse-mode gradients of a functional L of the output spectra of a Chi2PDC batch with respect to
 * the input spectra, the pump spectrum F0 = FFT(envelope) and a continuous poling profile d(z).
 * Complex gradients use the convention dL/dRe z + i dL/dIm z.
 *
 * nlm_set_poling_profile: replace the domain pattern by d(z) on the nZSteps grid (the values the
 *   reference keeps in its protected _poling array, src/_NonlinearMedium.cpp:470-503).
 * nlm_adjoint_forward: propagate rows x N input spectra (device) to rows x N output spectra (device),
 *   storing the states every checkpoint_interval steps (<= 0: every step when that fits in 40 % of the
 *   free device memory, at most 96 GB, else every ceil(sqrt(nZSteps-1)) steps, the segments
 *   being recomputed in the reverse sweep).
 *   Chi3GNLSE with checkpoint_interval <= 0 on a grid of 1024..8192 points, with rows x 4 <= SMs and
 *   the stage values of every step within a quarter of the free device memory (and 64 GB): the
 *   forward stores those stage values instead and *used_interval is 0 (nothing is recomputed).
 *   The pump must have been run.
 * nlm_adjoint_backward: given dL/dX (device, rows x N) returns dL/dX_in (device, rows x N), dL/dF0
 *   (device, N; may be NULL) and dL/dd (host, nZSteps doubles; may be NULL). */
nlm_status nlm_set_poling_profile(nlm_medium* m, const double* profile, size_t n);
nlm_status nlm_adjoint_forward(nlm_medium* m, const void* inputs_dev, size_t rows, void* out_dev,
                               int checkpoint_interval, int* used_interval);
nlm_status nlm_adjoint_backward(nlm_medium* m, const void* grad_out_dev, void* grad_in_dev,
                                void* grad_pump_dev, double* grad_poling);

/* --- allocation-free Chi3GNLSE batch ----------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory where they
 * propagate (memory owned by another allocator with a fixed budget, or loops where cudaMalloc /
 * cudaFree would synchronise the device): the same propagation as nlm_batch_device for a Chi3GNLSE
 * medium (rows x N complex inputs on the device, one N-point output row each, frequency or time
 * domain as in_time_domain), with the kernel's scratch taken from one 16 MiB file-scope device array
 * instead of an allocation.  The medium must have run one GPU call before (its device tables are
 * built there), with the same device current as now.  The array holds a slot of 2 N values per
 * resident propagation, so it bounds how many CTAs run at once, not the number of rows; grids the
 * one-CTA Chi3GNLSE kernel does not take (power of two, 8 to 4096 points) are rejected with
 * NLM_ERR_UNSUPPORTED.  The call is asynchronous on cuda_stream (a cudaStream_t; NULL is the legacy
 * default stream).  All calls share the array: calls that overlap on the GPU race.  The first call
 * on a device looks up the array's address (again on every call outside stream capture); make it
 * before any stream capture. */
nlm_status nlm_batch_gnlse_noalloc(nlm_medium* m, const void* inputs_dev, size_t rows,
                                   int in_time_domain, void* out_dev, void* cuda_stream);

/* --- getters (src/nlmModulePy.cpp:100-123) ---------------------------------------------
 * which: 0 = pumpFreq, 1 = pumpTime, 2 = signalFreq, 3 = signalTime, 4 = field.
 * Returns a pointer into a host mirror owned by the handle (refreshed from the device on
 * every call), valid until the handle is destroyed.  NLM_ERR_INDEX when index is out of
 * range, like the reference's std::vector::at.                                        */
nlm_status nlm_get_grid(nlm_medium* m, int which, unsigned index, const double** data,
                        size_t* rows, size_t* cols);
/* which: 0 = tau, 1 = omega, 2 = poling, 3 = ramanResponse (complex, Chi3GNLSE only),
 * 4 = envelope of pump `index` (complex).  Real arrays are doubles. */
nlm_status nlm_get_axis(nlm_medium* m, int which, unsigned index, const double** data, size_t* n);

/* --- Cascade (src/Cascade.cpp:3-167) --------------------------------------------------
 * connections: for each of the n_media-1 junctions a list of (input mode of next medium,
 * output mode of previous medium) pairs, flattened; conn_counts gives pairs per junction and
 * n_junctions their number (must be n_media-1, src/Cascade.cpp:21-22).
 * The cascade does not own its media: keep them alive while it exists.                 */
nlm_status nlm_cascade_create(nlm_medium* const* media, size_t n_media, const unsigned* connections,
                              const size_t* conn_counts, size_t n_junctions, int share_pump,
                              nlm_medium** out);
nlm_status nlm_cascade_add(nlm_medium* cascade, nlm_medium* medium, const unsigned* connection,
                           size_t n_pairs);
nlm_status nlm_cascade_media(const nlm_medium* cascade, size_t* n_media);

/* --- device / stream -------------------------------------------------------------------- */
/* Select the CUDA stream (a cudaStream_t) used by a handle; NULL = library stream. */
nlm_status nlm_set_stream(nlm_medium* m, void* cuda_stream);
/* Wait for all work of the handle. */
nlm_status nlm_synchronize(nlm_medium* m);
/* 1 when a CUDA device is usable by this process. */
int nlm_device_available(void);

/* --- engine controls ------------------------------------------------------------------- */
/* Schedule controls of the batched kernels.  cta_per_sm: 0 = autotuner (default: the first
 * batched launch of a shape times the kernel variants, propagations per CTA and resident CTAs per
 * SM on a few z steps and keeps the fastest for the process; NLM_AUTOTUNE=0 in the environment
 * turns it off), -1 = occupancy maximum without timing, > 0 = that many resident CTAs per SM;
 * use_propagator: 1 = precomputed RK4 propagator for linear solvers, 0 = direct DiffEq,
 * -1 = automatic; use_graph: 1 = batched launches captured into CUDA graphs and replayed
 * (default), 0 = direct launches.  No counterpart in the reference. */
nlm_status nlm_set_schedule(nlm_medium* m, int cta_per_sm, int use_propagator, int use_graph);
/* Launch shape of the last propagation of this handle: values[0..7] = points per thread R,
 * propagations per CTA, grid, block, resident CTAs per SM, 1 if chosen by the autotuner, the
 * autotuner trials this handle ran, and the registers per thread of the kernel variant.  No
 * counterpart in the reference. */
nlm_status nlm_last_schedule(const nlm_medium* m, int* values);
/* 1 (default): a launch of at most SMs/4 propagations on a grid of 1024 to 8192 points spreads
 * each propagation over a cluster of 4 CTAs (one per SM, four-step FFT through distributed
 * shared memory); so do the Chi3 pump march and the reverse sweeps of nlm_adjoint_backward (on 4
 * or, pipelined, 8 CTAs) on such grids.  On grids of 128 to 1024 points, such launches (and the
 * Chi2PDC reverse sweeps) and the Chi3 pump march use clusters with one point per thread instead;
 * full-grid propagations (runSignalSimulation) take the widest one-point-per-thread form: eight CTAs
 * at 1024 points, sixteen (a non-portable cluster size) at 2048 and 4096 points where the solver
 * has that form (single-mode solvers; multi-mode ones whose mode-fused buffers fit), eight otherwise;
 * the Chi3 pump march uses eight CTAs on 2048 and 4096 points.  On 128 to 1024 points, a Chi3
 * nlm_run_pump defers the pump march: the next nlm_run_signal runs it beside the signal on one
 * cluster of eight CTAs (four each, the signal one pump step pair behind); any other call that reads
 * the pump grids runs it alone first.
 * 3: as 1 without the widest forms (full grids on four CTAs up to 1024 points, eight above) and
 * without the deferred Chi3 pump march.
 * 2: the four-points-per-thread clusters only.  0: one CTA per propagation.  nlm_ragged_batch plans
 * each medium's form among those its mode allows (1: one, four, eight or sixteen CTAs; 3: one, four
 * or eight).  Other values: NLM_ERR_VALUE.  No counterpart in the reference. */
nlm_status nlm_set_cluster(nlm_medium* m, int enable);
/* Arithmetic of the single-mode precomputed-propagator kernel (Chi3, Chi2PDC Green's functions
 * and batches on power-of-two grids up to 4096 points): 0 = FP64 (default), 1 = double-float
 * (pairs of FP32 values, ~48-bit significand, on the FP32 units).  Other paths stay FP64, among
 * them launches of at most SMs/4 propagations on cluster grids (see nlm_set_cluster).
 * No counterpart in the reference (its arithmetic is always FP64). */
nlm_status nlm_set_precision(nlm_medium* m, int precision);
/* Run computeGreensFunction's propagations one per kernel launch (the "plain" form),
 * limited to the first max_instances impulse propagations (0 = all); the matrices of
 * the rows not propagated are left zero.  Timing helper for the plain-vs-batched ratio. */
nlm_status nlm_green_plain(nlm_medium* m, int in_time_domain, int run_pump, size_t max_instances,
                           double* green_c, double* green_s);
/* Propagation launches of this handle (and of a cascade's media) captured into CUDA graphs, and
 * replays of captured graphs, since creation.  A batched propagation (with the Green's-function
 * epilogue) is captured once per distinct set of launch arguments and replayed by later calls;
 * use_graph = 0 in nlm_set_schedule launches directly.  No counterpart in the reference. */
nlm_status nlm_graph_stats(const nlm_medium* m, long* captures, long* replays);
/* Number of kernels the last nlm_* call of this handle launched. */
nlm_status nlm_last_launch_count(const nlm_medium* m, long* launches);
/* Time the fused propagation kernel with CUDA events on the handle's stream.  enable = 1
 * resets and starts accumulating, 0 stops; total_ms/count return what was accumulated.
 * No counterpart in the reference (measurement support). */
nlm_status nlm_kernel_timing(nlm_medium* m, int enable, double* total_ms, long* count);
/* Measured FP64 FMA throughput of the current device in TFLOP/s (an FMA counts as two
 * flops): the roofline denominator of the propagation kernels.  No counterpart in the
 * reference (measurement support). */
nlm_status nlm_fp64_peak(double* tflops);
/* Measured FP64 tensor-core (DMMA, m16n8k16) throughput of the current device in TFLOP/s: what a
 * DFT-as-GEMM schedule could draw on in FP64.  No counterpart in the reference (measurement support). */
nlm_status nlm_fp64_mma_peak(double* tflops);
/* FP64 FMA throughput of the device with one CTA of warps_per_sm warps on every SM (TFLOP/s): shows
 * how many warps an SM needs to reach its FP64 rate (one per scheduler).  Measurement support. */
nlm_status nlm_fp64_warps_rate(int warps_per_sm, double* tflops);

/* --- Green's-function consumers (multimode.py:15-47) -------------------------------------------
 * Device pointers, row-major, on the given CUDA stream (NULL: the legacy default stream); the call
 * returns after the launch.  green_c / green_s: rows x cols complex128 (the (C, S) pair of
 * nlm_green*).
 * nlm_quadrature_greens: z = [[Re(C+S), -Im(C-S)], [Im(C+S), Re(C-S)]], 2 rows x 2 cols float64
 *   (calcQuadratureGreens, multimode.py:15-26).
 * nlm_abasis_greens: z = sqrt(1/2) [[C, S], [conj(S), conj(C)]], 2 rows x 2 cols complex128 (the
 *   matrix of calcCovarianceMtxABasis, multimode.py:40-47). */
nlm_status nlm_quadrature_greens(const void* green_c_dev, const void* green_s_dev, size_t rows, size_t cols,
                                 void* z_dev, void* cuda_stream);
nlm_status nlm_abasis_greens(const void* green_c_dev, const void* green_s_dev, size_t rows, size_t cols, void* z_dev,
                             void* cuda_stream);

/* --- Cascade composition (src/Cascade.cpp:128-129) --------------------------------------------
 * The Green's-function composition of two chained media, on device pointers (row-major complex128)
 * and the given CUDA stream: c_out = C2 C1 + S2 conj(S1), s_out = C2 S1 + S2 conj(C1), with C2, S2
 * rows x inner and C1, S1 inner x cols.  nlm_green of a cascade runs the same kernel between its
 * media; exported so that the composition can be timed and checked on its own.  Outputs must not
 * alias inputs. */
nlm_status nlm_cascade_compose(const void* c2_dev, const void* s2_dev, const void* c1_dev, const void* s1_dev,
                               size_t rows, size_t inner, size_t cols, void* c_out_dev, void* s_out_dev,
                               void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* NLM_CAPI_H */
