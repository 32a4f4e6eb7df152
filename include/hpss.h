/*
 * hpss.h -- C ABI of the GB300 semblance engine (libhpss_gb300.so).
 *
 * This is the drop-in boundary for the semblance hot path of
 * HighPerformanceSeismicStacking.  In the reference, the path sits behind the
 * C++ ComputeAlgorithm family (common/include/semblance/algorithm/
 * ComputeAlgorithm.hpp:29-100) whose CUDA subclasses launch the kernels
 * (cuda/src/semblance/algorithm/Cuda*Algorithm.cu).  Each entry point below
 * names the reference member it replaces.  All signatures use plain C types;
 * no exception crosses the boundary; every call returns an hpss_status
 * (0 = OK, < 0 = error, message via hpss_last_error).
 *
 * Threading: one handle per host thread (like one ComputeAlgorithm per
 * device thread in SingleHostRunner.cpp:49-106).  A handle owns all the
 * device memory it uses and one CUDA stream.
 *
 * Data conventions (as the reference):
 *  - traces are passed sorted by (midpoint, half-offset) ascending, the order
 *    Gather::readGatherFromFile leaves them in (Gather.cpp:117, Trace.cpp:63);
 *  - a result block for one midpoint is [(2 + nParams)][S] floats, SoA:
 *    semblance, stack, then the parameters (velocity, A, B | velocity, slope),
 *    exactly ComputeAlgorithm::getComputedResults (ComputeAlgorithm.hpp:84);
 *  - linear-search candidates follow buildParameterArrayFor*: the first
 *    parameter varies slowest, velocity is searched uniformly in v and stored
 *    as 4/v^2, the upper bound is excluded (step = (U - L) / G).
 */
#ifndef HPSS_H
#define HPSS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int hpss_status;

/* Status codes.  The reference throws C++ exceptions; the mapping is:
 * invalid_argument -> HPSS_ERR_INVALID_ARGUMENT, logic_error (wrong number of
 * bounds / granularities, CudaComputeAlgorithmBuilder.cu:26-31) ->
 * HPSS_ERR_LOGIC, runtime_error from CUDA_ASSERT (CudaUtils.cu:8-15) ->
 * HPSS_ERR_CUDA / HPSS_ERR_NO_DEVICE. */
#define HPSS_OK 0
#define HPSS_ERR_INVALID_ARGUMENT (-1)
#define HPSS_ERR_LOGIC (-2)
#define HPSS_ERR_CUDA (-3)
#define HPSS_ERR_NO_DEVICE (-4)
#define HPSS_ERR_OUT_OF_MEMORY (-5)
#define HPSS_ERR_NOT_READY (-6)
#define HPSS_ERR_TIMEOUT (-7)
#define HPSS_ERR_DEVICE_CHECK (-8)

/* Bits of the device error word (hpss_stats.device_error,
 * hpss_noalloc_device_error).  A synchronous call that sees TIMEOUT returns
 * HPSS_ERR_TIMEOUT, any other bit HPSS_ERR_DEVICE_CHECK; its outputs are then
 * not valid. */
#define HPSS_DEVERR_SMEM_BOUNDS 1u   /* shared-memory index out of its span
                                        (bounds-checked builds only) */
#define HPSS_DEVERR_SPAN_OVERFLOW 2u /* a trace span larger than the stage */
#define HPSS_DEVERR_TIMEOUT 4u       /* staging copies did not complete
                                        within the bounded wait */

/* traveltime_t (common/include/capability.h:3-7). */
#define HPSS_MODEL_CMP 0
#define HPSS_MODEL_ZOCRS 1
#define HPSS_MODEL_OCT 2

/* Device storage of the trace amplitudes.  FP32 is what the reference
 * stores; BF16 / FP16 halve the bytes (FP16 with a per-trace FP32 scale).
 * Interpolation and all sums stay FP32. */
#define HPSS_STORAGE_FP32 0
#define HPSS_STORAGE_BF16 1
#define HPSS_STORAGE_FP16 2

/* Kernel family: PLAIN is the one-(sample, candidate)-per-thread FP32 form of
 * the reference kernels with the argmax fused (its arithmetic is the
 * reference's, operation for operation); TUNED stages each gather's trace
 * windows in shared memory and shares them across the candidates of a CTA.
 * For CMP and ZO-CRS, TUNED takes the stack's linear sum as the sum of the
 * per-tap window sums (semblance and chosen parameters identical to PLAIN,
 * the stack within a few ulp); TUNED_EXACT accumulates it in the reference's
 * order (every output identical to PLAIN) at one more add per tap.  For OCT
 * both run the same kernel. */
#define HPSS_KERNEL_PLAIN 0
#define HPSS_KERNEL_TUNED 1
#define HPSS_KERNEL_TUNED_EXACT 2

typedef struct hpss_handle_s *hpss_handle;

/* Per-call statistics (StatisticResult, common/include/semblance/result/
 * StatisticResult.hpp:8-15, plus the evaluation count of the metric). */
typedef struct {
    double evals;             /* (m0, t0, candidate, selected trace) tuples */
    double not_used;          /* OCT traces skipped for their displaced midpoint */
    double selected_traces;   /* sum over midpoints of selected traces */
    double kernel_ms;         /* device time of the compute launches */
    double selection_ms;      /* device time of trace selection */
    uint32_t device_error;    /* device error word (0 = none) */
    int32_t kernel_variant;   /* tuned-kernel shape chosen by the autotuner
                                 (-1: plain / not applicable) */
    double near_ties;         /* linear search: (m0, t0) samples whose best
                                 semblance is > 0 and whose runner-up lies
                                 within HPSS_NEAR_TIE_REL * max(best, 1e-3)
                                 of it (the chosen index may differ from
                                 another FP32 evaluation's there); 0 for
                                 differential evolution and stretch-free */
    uint32_t candidate_parts; /* tuned linear search: candidate ranges the
                                 search of each (midpoint, 32-sample tile)
                                 was split into so that a call with few
                                 midpoints fills the GPU (1: no split) */
} hpss_stats;

#define HPSS_NEAR_TIE_REL 1e-4f

/* Device selection and handle creation.
 * Replaces CudaDeviceContext(devId) + activate()
 * (cuda/src/semblance/data/CudaDeviceContext.cu:10-17). */
hpss_status hpss_create(int device, hpss_handle *out);
hpss_status hpss_destroy(hpss_handle h);

/* Message of the last failed call on this handle (thread-local if h is
 * NULL: errors of hpss_create). */
const char *hpss_last_error(hpss_handle h);

/* Library version string. */
const char *hpss_version(void);

/* Number of visible CUDA devices (CudaSingleHostRunner::getNumOfDevices,
 * cuda/src/execution/CudaSingleHostRunner.cu:18-29). */
hpss_status hpss_device_count(int *count);

/* Upload the whole line once: amplitudes [nTraces][S] (row-major, FP32),
 * midpoints and half-offsets [nTraces].  Replaces
 * ComputeAlgorithm::copyGatherDataToDevice (ComputeAlgorithm.cpp:31-61) and
 * the per-midpoint copyOnlySelectedTracesToDevice (ComputeAlgorithm.cpp
 * :107-153): traces stay resident and are selected on the device.
 * `storage` is one of HPSS_STORAGE_*.  Host pointers; page-locked memory is
 * copied asynchronously, pageable memory synchronously. */
hpss_status hpss_upload_gather(hpss_handle h, const float *samples,
                               const float *midpoints,
                               const float *halfoffsets, uint32_t nTraces,
                               uint32_t samplesPerTrace, float dtInSeconds,
                               int storage);

/* Traveltime model and its parameter bounds (Traveltime::update*BoundFor
 * Parameter, common/src/traveltime/Traveltime.cpp:39-53, built by
 * TraveltimeBuilder, TraveltimeBuilder.cpp:24-106).  nParams must be 1
 * (CMP), 3 (ZO-CRS: velocity, A, B -- A and B bounds as the builder derived
 * them) or 2 (OCT: velocity, slope).  apm is Gather::getApm (used by ZO-CRS
 * and OCT selection, OCT evaluation); h0 is the OCT reference half-offset. */
hpss_status hpss_set_traveltime(hpss_handle h, int model, uint32_t nParams,
                                const float *lower, const float *upper,
                                float apm, float h0);

/* Candidate grid of the linear search.  REFERENCE is
 * buildParameterArrayFor* with setupDiscretizationSteps
 * (LinearSearchAlgorithm.cpp:129-141): uniform in velocity, step (U - L) / G,
 * U never reached.  INCLUSIVE includes both bounds: the velocity parameter is
 * uniform in c = 4/v^2 from 4/L^2 (index 0, lowest velocity) to 4/U^2, the
 * others uniform from L to U, G values each.  No reference counterpart for
 * INCLUSIVE (the grids of the ZO-CRS workloads are stated inclusive in C).
 * Default REFERENCE; applies to hpss_linear_search*. */
#define HPSS_GRID_REFERENCE 0
#define HPSS_GRID_INCLUSIVE 1
hpss_status hpss_set_grid_mode(hpss_handle h, int mode);

/* Precision modes of the linear search (no reference counterpart; the
 * default 0 is the reference's FP32 arithmetic).  FP64_TRAVELTIME forms the
 * ZO-CRS / OCT traveltime in FP64 (square-root arguments, divisions, the
 * displaced midpoint) and rounds it to FP32 once (CMP: no effect);
 * COMPENSATED compensates the window sums when window x selected traces
 * exceeds 4096 terms.  Both run in the tuned kernels: CMP / ZO-CRS in one
 * fixed shape (no autotuning; FP64 traveltime bit-identical to the plain
 * kernel's), summing each staging round (at most 256 traces) in FP32 and
 * adding the rounds with Knuth's two-sum; OCT with the FP64 traveltime in
 * the OCT kernel (bit-identical to the plain kernel's).  The plain kernel,
 * and OCT with COMPENSATED, compensate every term (Neumaier).
 * Interpolation stays FP32. */
#define HPSS_PREC_FP64_TRAVELTIME 1
#define HPSS_PREC_COMPENSATED 2
/* Every step in FP64 -- traveltime, window index and fraction,
 * interpolation, sums, semblance, argmax -- rounded to FP32 once at the end:
 * the FP64 reference the other modes are judged against (at a small
 * fraction of the FP32 throughput; overrides the other flags). */
#define HPSS_PREC_FP64 4
hpss_status hpss_set_precision(hpss_handle h, int flags);

/* OCT over several target half-offsets in one call (no reference
 * counterpart: the reference holds one h0 per OffsetContinuationTrajectory,
 * common/src/traveltime/OffsetContinuationTrajectory.cpp:5-25, and runs a
 * whole job per h0).  With nH0 >= 1 values, every OCT linear search,
 * differential evolution, stretch-free and trace-selection call over nM0
 * midpoints computes nH0 x nM0 results in one launch: result blocks (and
 * stretch-free parameter blocks, selection counts) are laid out
 * [nH0][nM0][...], block (b, i) being midpoint i at h0s[b] -- exactly what
 * a call with hpss_set_traveltime(..., h0s[b]) would give, the DE random
 * stream included.  The h0 of hpss_set_traveltime is then not used; nH0 = 0
 * restores it.  At most 64 values; CMP and ZO-CRS calls are unaffected;
 * hpss_linear_search_line rejects OCT lists. */
hpss_status hpss_set_oct_half_offsets(hpss_handle h, const float *h0s, uint32_t nH0);

/* Semblance window: tauIndexDisplacement = (int)(tau / dt), window
 * w = 2 * tau + 1 (Gather.cpp:75-76).  w must be <= 31
 * (MAX_WINDOW_SIZE, common/include/gpu/interface.h:10). */
hpss_status hpss_set_window(hpss_handle h, int tauIndexDisplacement);

/* Linear search over nM0 midpoints in one call.
 * Replaces LinearSearchAlgorithm::computeSemblanceAndParametersForMidpoint
 * (LinearSearchAlgorithm.cpp:26-57) with the CUDA steps of
 * CudaLinearSearchAlgorithm (selectTracesToBeUsedForMidpoint :225-324,
 * computeSemblanceAtGpuForMidpoint :35-163, initializeParameters :165-223),
 * batched over midpoints.  granularity[nParams] as the --granularity flag.
 * out (host): [nM0][2 + nParams][S].  Synchronous. */
hpss_status hpss_linear_search(hpss_handle h, const float *m0s, uint32_t nM0,
                               const uint32_t *granularity, int kernel,
                               float *out, hpss_stats *stats);

/* Upload a line and search it in one call, the upload overlapped with the
 * search: the amplitudes go to the device in 8 trace ranges on a second
 * stream while the midpoints are searched in 8 contiguous groups, each group
 * starting as soon as the traces it can select have arrived, and each
 * group's results are copied back while the next group runs.  The line
 * replaces the resident one as hpss_upload_gather would (same arguments and
 * checks); the traveltime and the window must be set before.  Results,
 * statistics and errors are those of hpss_upload_gather followed by
 * hpss_linear_search, except stats->kernel_ms (device time from the first
 * group's start to the last group's end, copies overlapped) and
 * stats->selection_ms (0).  Host arrays must stay unchanged until it
 * returns.  The reference copies the selected traces of every midpoint
 * before its search (ComputeAlgorithm::copyOnlySelectedTracesToDevice,
 * common/src/semblance/algorithm/ComputeAlgorithm.cpp:107-153); this call
 * replaces that per-midpoint copy for a whole line. */
hpss_status hpss_linear_search_line(hpss_handle h, const float *samples,
                                    const float *midpoints, const float *halfoffsets,
                                    uint32_t nTraces, uint32_t samplesPerTrace,
                                    float dtInSeconds, int storage, const float *m0s,
                                    uint32_t nM0, const uint32_t *granularity, int kernel,
                                    float *out, hpss_stats *stats);

/* Same computation with device-resident midpoints and output (d_m0s,
 * d_out are device pointers).  Enqueued on the handle's stream; returns
 * without synchronising.  stats may be NULL (its timing fields are then not
 * filled). */
hpss_status hpss_linear_search_device(hpss_handle h, const float *d_m0s,
                                      uint32_t nM0,
                                      const uint32_t *granularity, int kernel,
                                      float *d_out, hpss_stats *stats);

/* Differential evolution (DE/rand/1/bin) per (m0, t0) sample.
 * Replaces DifferentialEvolutionAlgorithm::computeSemblanceAndParametersFor
 * Midpoint (DifferentialEvolutionAlgorithm.cpp:21-81) and the kernels of
 * cuda/src/semblance/kernel/common/differential_evolution.cu.  F and CR are
 * runtime values (the reference compiles F = 0.85, CR = 0.5,
 * interface.h:5-6); `generations` counts the initial evaluation as the
 * reference does.  The random stream is a counter-based generator keyed by
 * `seed` and by each midpoint's value (the reference's curand stream is
 * seeded from time(NULL)): a midpoint's result does not depend on the other
 * midpoints, half-offsets or shards of the call.
 * out (host): [nM0][2 + nParams][S] with RAW parameters (velocity, not 4/v^2),
 * as selectBestIndividualsFor* write them. */
hpss_status hpss_differential_evolution(hpss_handle h, const float *m0s,
                                        uint32_t nM0, uint32_t population,
                                        uint32_t generations, float F,
                                        float CR, uint64_t seed, float *out,
                                        hpss_stats *stats);

/* Device-pointer variant of hpss_differential_evolution (async). */
hpss_status hpss_differential_evolution_device(
    hpss_handle h, const float *d_m0s, uint32_t nM0, uint32_t population,
    uint32_t generations, float F, float CR, uint64_t seed, float *d_out,
    hpss_stats *stats);

/* Stretch-free stack: for n in [-nmax, nmax] the model parameters chosen at
 * sample s - n by a previous search (params: host [nM0][nParams][S], RAW
 * parameters, velocity first -- the layout of the reference's result files
 * read by StretchFreeAlgorithm::readNonStretchedFreeParameterFromFile,
 * StretchFreeAlgorithm.cpp:101-125) are applied with a time shift n*dt.
 * Replaces StretchFreeAlgorithm::computeSemblanceAndParametersForMidpoint
 * (StretchFreeAlgorithm.cpp:23-50) and CudaStretchFreeAlgorithm
 * (CudaStretchFreeAlgorithm.cu:28-200).  out: [nM0][3][S] = semblance,
 * stack, best n. */
hpss_status hpss_stretch_free(hpss_handle h, const float *m0s, uint32_t nM0,
                              const float *params, int nmax, float *out,
                              hpss_stats *stats);

/* Selected-trace count per midpoint, as selectTracesToBeUsedForMidpoint
 * computes it (filteredTracesCount).  For OCT the selection uses the
 * linear-search sampling rule (oct/linear_search.cu:155-192). */
hpss_status hpss_select_traces(hpss_handle h, const float *m0s, uint32_t nM0,
                               uint32_t *counts);

/* The CUDA stream the handle launches on (cudaStream_t), for callers that
 * order their own work or record events against it. */
void *hpss_stream(hpss_handle h);

/* Bytes of device memory currently held by the handle. */
size_t hpss_device_bytes(hpss_handle h);

/* Result files from a result slab [nM0][rows][S] (the layout of every
 * search's output): one SU file per row r, paths[r] (NULL: row skipped),
 * holding for every midpoint i in order the 240-byte trace header
 * headers[i] (trace_info_t, the CDP's header) followed by slab[i][r][0..S).
 * Replaces Dumper::dumpResult (common/src/output/Dumper.cpp:77-114), which
 * writes one header and one trace per CDP from the ResultSet's per-CDP
 * vectors: here each file image is assembled in one buffer -- from device
 * memory (slabOnDevice != 0) by one strided copy per file -- and written at
 * once.  Errors via hpss_last_error(NULL). */
hpss_status hpss_write_result_files(const float *slab, int slabOnDevice, uint32_t nM0,
                                    uint32_t rows, uint32_t S, const void *headers,
                                    const char *const *paths);

/* Linear search that allocates nothing -- no counterpart in the reference.
 * For callers that may not call cudaMalloc (a plug-in inside another
 * framework's memory pool, a process with a fixed device-memory budget): the
 * caller passes device buffers for the line (samples [nTraces][stride] FP32,
 * stride >= S and a multiple of 4, 16-byte aligned; midpoints, half-offsets),
 * the midpoints d_m0s and the output d_out [nM0][2+nParams][S]; the scratch
 * lives in a fixed __device__ array of the library (about 5.3 MB, held on
 * every device that loads the library).  CMP and ZO-CRS only; limits:
 * candidates <= 65536, midpoints <= 16384, traces <= 1048576 (larger sizes are
 * rejected with HPSS_ERR_INVALID_ARGUMENT).  The first call on a device looks
 * the scratch up (make it before any stream capture).  Calls share the
 * scratch: calls that overlap on the GPU race.  Enqueued on `stream`
 * (cudaStream_t; NULL = default stream); errors found on the host via
 * hpss_last_error(NULL); errors found by the kernels (the device error word,
 * hpss_stats.device_error of the allocating calls) via
 * hpss_noalloc_device_error.  The scratch address is looked up once per
 * device and kept: do not call it on a device after cudaDeviceReset.
 * Same results as hpss_linear_search with the tuned kernel. */
hpss_status hpss_linear_search_noalloc(
    int model, const float *d_samples, uint32_t stride, const float *d_midpoints,
    const float *d_halfoffsets, uint32_t nTraces, uint32_t samplesPerTrace,
    float dtInSeconds, int tauIndexDisplacement, const float *lower,
    const float *upper, const uint32_t *granularity, float apm,
    const float *d_m0s, uint32_t nM0, float *d_out, void *stream);

/* Device error word of the last hpss_linear_search_noalloc call on the
 * current device (no counterpart in the reference): waits for `stream` and
 * copies the word into *word (0 = none; bits as hpss_stats.device_error).
 * The word is cleared at the start of every call, so read it before the next
 * call.  Allocates nothing. */
hpss_status hpss_noalloc_device_error(void *stream, uint32_t *word);

#ifdef __cplusplus
}
#endif
#endif /* HPSS_H */
