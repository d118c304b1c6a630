/*
 * hpxfft_gb300 -- C ABI of the GB300 (sm_103a) 2D real-to-complex FFT.
 *
 * This is the boundary the C++ drop-in headers (hpxfft::shared::loop and
 * friends) and any FFI (ctypes, cgo, JNI) bind.  Plain pointers and sizes
 * only; every function returns an hpxfft_status (0 = success).
 *
 * Data layout (the reference's, core/include/hpxfft/util/vector_2d.hpp:9-86
 * and examples/hpxfft/shared_loop_2d.cpp:27-40): a row-major buffer of
 * n_row x n_col reals, n_col = 2 * (ny/2 + 1).  The first ny reals of a row
 * are input data, the last two are padding.  The forward transform overwrites
 * row kx with the n_col/2 complex values X[kx][ky] = sum_{x,y} v[x][y]
 * exp(-2 pi i (kx x / n_row + ky y / ny)), unnormalised (numpy.fft.rfft2
 * orientation: the reference transposes back at the end,
 * core/src/shared/loop.cpp:94-102).
 *
 * Precision: HPXFFT_PREC_F64 stores doubles and computes in float-float on
 * the FP32 pipes (about 48 significant bits; relative L2 error vs FP64 FFTW
 * is ~1e-14); HPXFFT_PREC_F64_NATIVE computes with DFMA (slow on GB300,
 * kept as a cross-check); HPXFFT_PREC_F32 stores and computes float;
 * HPXFFT_PREC_BF16X3 stores float and runs the first radix-16 stage of each
 * column DFT and of each row DFT (compiled row lengths 128..8192) as a dense
 * complex matmul on the tensor cores (tcgen05, BF16 operands split three
 * ways, FP32 accumulation), the other stages in FP32.
 */
#ifndef HPXFFT_GB300_H
#define HPXFFT_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define HPXFFT_API __attribute__((visibility("default")))
#else
#define HPXFFT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    HPXFFT_OK = 0,
    HPXFFT_ERR_INVALID_ARG = 1,      /* std::invalid_argument in the reference (bad plan flag) */
    HPXFFT_ERR_UNSUPPORTED_SIZE = 2, /* odd ny, or a size outside the limits of hpxfft_plan_create */
    HPXFFT_ERR_ALLOC = 3,            /* device or pinned allocation failed */
    HPXFFT_ERR_CUDA = 4,             /* a CUDA runtime call failed */
    HPXFFT_ERR_TIMEOUT = 5,          /* a bounded device-side wait gave up */
    HPXFFT_ERR_STATE = 6,            /* call out of order (e.g. execute on a destroyed plan) */
    HPXFFT_ERR_IO = 7                /* std::runtime_error in the reference (file open) */
} hpxfft_status;

typedef enum {
    HPXFFT_PREC_F64 = 0,        /* FP64 in HBM, float-float arithmetic */
    HPXFFT_PREC_F64_NATIVE = 1, /* FP64 in HBM, DFMA arithmetic */
    HPXFFT_PREC_F32 = 2,        /* FP32 in HBM and arithmetic */
    HPXFFT_PREC_BF16X3 = 3      /* FP32 in HBM; split-BF16 tensor-core column stage; n_row a power of two, 1024..65536 */
} hpxfft_precision;

typedef struct hpxfft_plan_s *hpxfft_plan;
typedef struct hpxfft_plan3d_s *hpxfft_plan3d;

/* Plan a 2D r2c of `batch` equally sized arrays of n_row x n_col reals
 * (n_col = 2*(ny/2+1), so ny = n_col - 2).  plan_flag is one of
 * "estimate", "measure", "patient", "exhaustive"; anything else returns
 * HPXFFT_ERR_INVALID_ARG.  "estimate" plans by fixed rules set by
 * measurements on GB300.  "measure", "patient" and "exhaustive" run trial
 * transforms of every distinct candidate plan (column strategy: cluster
 * kernel or two-kernel four-step pass; float-float pair exchange between the
 * kernels; split-BF16 vectors per CTA and tensor-core rows) on two scratch
 * arrays of the plan's size (allocated and freed during the call), best of
 * 3, 5 or 10 runs, and keep the fastest.  The choice is cached per shape,
 * batch, precision and device architecture, so a later plan of the same kind
 * runs no trials; hpxfft_wisdom_export / _import save and restore the cache.
 * Measurements "cached_plan", "autotune_candidates", "autotune_ms_<i>",
 * "autotune_best_ms" and "choice_*" describe the search.
 * Allocates the twiddle tables and no data buffer.
 * Sizes: ny even, any n_row (as FFTW takes them); batch <= 65535.  The
 * direct kernels take ny/2 (the row's complex length) and n_row without a
 * prime factor above 13: a row on a cluster of C in {1, 2, 4} CTAs of at
 * most 8192 complex values each, a column on C in {1, 2, 4, 8, 16} CTAs of
 * at most 4096 (FP64) or 8192 (FP32) each, C > 1 needing the length
 * divisible by C^2, and power-of-two n_row up to 2^24 (FP64) or 2^25
 * (FP32) through the two-kernel column pass.  Other lengths take
 * Bluestein's convolution through power-of-two column plans, and rows
 * outside the direct kernels run as a column pass on a transposed copy
 * (n_row <= 2^21 there); measurements "bluestein_rows", "bluestein_columns"
 * (the convolution length, 0 when unused) and "transposed_rows" say which.
 * Split-BF16 (n_row a power of two in [1024, 65536]) keeps the direct
 * kernels' sizes.  Sizes outside all of these return
 * HPXFFT_ERR_UNSUPPORTED_SIZE before any device call.
 * Replaces: hpxfft::shared::loop::initialize (core/src/shared/loop.cpp:158-189)
 * and fftw_adapter::{r2c_1d,c2c_1d}::plan (core/src/util/adapter_fftw.cpp:6-10,24-30),
 * string_to_fftw_plan_flag (core/include/hpxfft/util/adapter_fftw.hpp:22-44). */
HPXFFT_API int hpxfft_plan_create(hpxfft_plan *plan, size_t n_row, size_t n_col, size_t batch, int precision,
                       const char *plan_flag);

/* Free the plan's device memory, events and owned stream.
 * Replaces: ~loop / fftw_adapter::cleanup (core/include/hpxfft/shared/loop.hpp:30). */
HPXFFT_API int hpxfft_plan_destroy(hpxfft_plan plan);

/* Run on a caller-owned cudaStream_t, taken verbatim (NULL is the legacy
 * default stream).  A new plan runs on a non-blocking stream of its own,
 * whose handle hpxfft_plan_get_stream returns before any set_stream. */
HPXFFT_API int hpxfft_plan_set_stream(hpxfft_plan plan, void *cuda_stream);
HPXFFT_API int hpxfft_plan_get_stream(hpxfft_plan plan, void **cuda_stream);

/* Bytes of one array in HBM (n_row * n_col * sizeof(real)) times batch. */
HPXFFT_API int hpxfft_plan_buffer_bytes(hpxfft_plan plan, size_t *bytes);

/* In-place forward transform of a device buffer in the padded layout,
 * stream-ordered, asynchronous.  Replaces the four phases of
 * loop::fft_2d_r2c_par (core/src/shared/loop.cpp:56-113) and the per-locality
 * compute of distributed::loop::fft_2d_r2c at one locality
 * (core/src/distributed/loop.cpp:130-272). */
HPXFFT_API int hpxfft_execute_r2c(hpxfft_plan plan, void *device_values);

/* Out-of-place forward transform: d_in (padded real layout, read only) to
 * d_out (same layout, receives the spectrum).  d_in may equal d_out. */
HPXFFT_API int hpxfft_execute_r2c_oop(hpxfft_plan plan, const void *d_in, void *d_out);

/* Host buffer in, host buffer out (in place): copies to a plan-owned device
 * buffer, transforms, copies back, synchronises.  The drop-in path of
 * loop::initialize + loop::fft_2d_r2c_par. */
HPXFFT_API int hpxfft_execute_r2c_host(hpxfft_plan plan, void *host_values);

/* Unnormalised inverse (c2r) of a half spectrum in the padded layout, in
 * place: nx*ny * original.  No reference counterpart (the FFTW backward
 * direction exists in core/include/hpxfft/util/adapter_fftw.hpp:11 but is
 * never planned). */
HPXFFT_API int hpxfft_execute_c2r(hpxfft_plan plan, void *device_values);

/* Adjoint of the forward transform, in place: the buffer holds G =
 * dL/dRe X + i dL/dIm X over the half spectrum and receives dL/dx (pads 0).
 * No reference counterpart (gradient for fft_2d_r2c_backward). */
HPXFFT_API int hpxfft_execute_r2c_backward(hpxfft_plan plan, void *device_values);

/* The adjoint on a host buffer, in place: copies to the plan-owned device
 * buffer, transforms, copies back, synchronises (the host-side
 * fft_2d_r2c_backward of the C++ classes).  No reference counterpart. */
HPXFFT_API int hpxfft_execute_r2c_backward_host(hpxfft_plan plan, void *host_values);

/* Wait for every transform issued on the plan's stream; HPXFFT_ERR_TIMEOUT
 * if a bounded device-side wait of a tensor-core kernel gave up (the flag is
 * cleared by the call).  No reference counterpart (FFTW calls return when
 * done). */
HPXFFT_API int hpxfft_plan_synchronize(hpxfft_plan plan);

/* Measurement by key, seconds unless stated: "total", "first_fftw" (row
 * kernel), "first_trans" (0: fused), "second_fftw" (column kernel),
 * "second_trans" (0: fused), "plan", "plan_flops", "h2d", "d2h", "e2e"
 * (host buffer in to host buffer out of the last hpxfft_execute_r2c_host),
 * "gbps" (4 S / total, GB/s), "gflops" (2.5 N log2 N per array, N = nx ny,
 * times batch, / total), "roofline" (gbps over the device's nominal DRAM
 * bandwidth from its memory clock and bus width, 0 if unknown).
 * Unknown keys give 0, like loop::get_measurement (core/src/shared/loop.cpp:192). */
HPXFFT_API int hpxfft_get_measurement(hpxfft_plan plan, const char *name, double *value);

/* Mean kernel durations (seconds) over every transform executed since the
 * last hpxfft_timing_reset: first = row kernel, second = column kernel (the
 * inverse runs them in the opposite order), total = both.  Blocks until the
 * transforms are done.  No reference counterpart (the reference keeps the
 * last run only, core/src/shared/loop.cpp:106-110). */
HPXFFT_API int hpxfft_timing_stats(hpxfft_plan plan, double *first_mean, double *second_mean, double *total_mean,
                                   long long *count);
HPXFFT_API int hpxfft_timing_reset(hpxfft_plan plan);

/* Append the chosen GPU plan to a text file.  HPXFFT_ERR_IO if the file
 * cannot be opened.  Replaces loop::write_plans_to_file
 * (core/src/shared/loop.cpp:194-212). */
HPXFFT_API int hpxfft_write_plan(hpxfft_plan plan, const char *file_path);

/* 1 if plan_flag is a valid plan flag string, else 0. */
HPXFFT_API int hpxfft_plan_flag_valid(const char *plan_flag);

/* 3D r2c of `batch` arrays of n0 x n1 x n2 reals, the last axis padded to
 * n_col = 2*(n2/2+1) (the 2D layout with one more leading axis); in place,
 * output X[k0][k1][k2], k2 <= n2/2, unnormalised (numpy.fft.rfftn).  A
 * batched 2D r2c over the n0 slabs, then the column pass along axis 0.
 * n0 * batch <= 65535.  No reference counterpart (the reference is 2D
 * only; "multidimensional" in its title). */
HPXFFT_API int hpxfft_plan3d_create(hpxfft_plan3d *plan, size_t n0, size_t n1, size_t n_col, size_t batch,
                                    int precision, const char *plan_flag);
HPXFFT_API int hpxfft_plan3d_destroy(hpxfft_plan3d plan);
HPXFFT_API int hpxfft_plan3d_set_stream(hpxfft_plan3d plan, void *cuda_stream);
HPXFFT_API int hpxfft_plan3d_buffer_bytes(hpxfft_plan3d plan, size_t *bytes);
HPXFFT_API int hpxfft_execute3d_r2c(hpxfft_plan3d plan, void *device_values);
/* "total", "first_fftw" (axis 2), "second_fftw" (axis 1), "third_fftw"
 * (axis 0) of the last transform, seconds; other keys as the 2D plan. */
HPXFFT_API int hpxfft_plan3d_get_measurement(hpxfft_plan3d plan, const char *name, double *value);

/* ---- slab decomposition over P ranks -----------------------------------
 * The per-locality compute of hpxfft::distributed::loop::fft_2d_r2c
 * (core/src/distributed/loop.cpp:130-272) for P localities, one GPU each,
 * with index maps that are right for every P (the reference's transposes,
 * core/src/distributed/loop.cpp:87-127, interleave the slabs cyclically and
 * are right only for P = 1).  Rank r holds global rows r*n_row_local .. of
 * the padded n_row x n_col input (n_row = P * n_row_local).  The dcy =
 * n_col/2 complex columns split into P tiles of w = ceil(dcy / P) columns
 * (zero padded), so dcy need not be a multiple of P.  A send or receive
 * buffer is P tiles of hpxfft_slab_tile_bytes each, tile d for rank d.
 * The exchanges are the caller's (an all_to_all of equal tiles, or P
 * scatters); the library runs the local phases, stream-ordered:
 *   1. hpxfft_slab_rows(values, send): row r2c of the local rows (in place)
 *      and the pack (core/src/distributed/loop.cpp:19-27 split_vec);
 *   2. exchange send -> recv (tile d to rank d);
 *   3. hpxfft_slab_columns(recv): the received tiles are the column slab
 *      [n_row][w] of this rank's columns; column c2c in place; afterwards
 *      tile d holds the rows of rank d and is sent back as it is;
 *   4. exchange recv -> recv2;
 *   5. hpxfft_slab_finish(recv2, values): the local rows of the spectrum,
 *      X[r*n_row_local + x][ky], in the padded layout.
 * Measurements (seconds, last run): "first_fftw", "first_split",
 * "second_fftw", "second_trans", "plan"; "first_trans" and "second_split"
 * are 0 (no separate transposes); "first_comm" / "second_comm" belong to
 * the caller.  Split-BF16 runs FP32 rows and tensor-core columns (n_row a
 * power of two in [1024, 65536]). */
typedef struct hpxfft_slab_s *hpxfft_slab;
HPXFFT_API int hpxfft_slab_create(hpxfft_slab *slab, size_t n_row_local, size_t n_col, size_t n_ranks, size_t rank,
                                  int precision, const char *plan_flag);
HPXFFT_API int hpxfft_slab_destroy(hpxfft_slab slab);
HPXFFT_API int hpxfft_slab_set_stream(hpxfft_slab slab, void *cuda_stream);
HPXFFT_API int hpxfft_slab_tile_bytes(hpxfft_slab slab, size_t *bytes);
HPXFFT_API int hpxfft_slab_rows(hpxfft_slab slab, void *device_values, void *device_send);
HPXFFT_API int hpxfft_slab_columns(hpxfft_slab slab, void *device_recv);
HPXFFT_API int hpxfft_slab_finish(hpxfft_slab slab, const void *device_recv, void *device_values);
HPXFFT_API int hpxfft_slab_synchronize(hpxfft_slab slab);
HPXFFT_API int hpxfft_slab_get_measurement(hpxfft_slab slab, const char *name, double *value);

/* Static description of a status code; message of the calling thread's
 * most recent failure. */
HPXFFT_API const char *hpxfft_status_string(int status);
HPXFFT_API const char *hpxfft_last_error(void);

/* ---- batches of uneven sizes -------------------------------------------
 * Many independent forward 2D r2c transforms of different shapes in one
 * persistent work-queue launch, captured in a CUDA graph and replayed.
 * Instance i is an n_rows[i] x n_cols[i] padded array placed at byte offset
 * offsets[i] of one device arena (hpxfft_batch_offsets); every row and every
 * column must fit one CTA (at most 8192 FP32 or 4096 FP64 complex values).
 * plan_flag "estimate" uses the default queue order; "measure", "patient"
 * and "exhaustive" time candidate orders on a scratch arena once and cache
 * the winner for this mix of shapes (see hpxfft_wisdom_*).
 * No reference counterpart (the reference transforms one array at a time). */
typedef struct hpxfft_batch_s *hpxfft_batch;
HPXFFT_API int hpxfft_batch_create(hpxfft_batch *batch, size_t count, const size_t *n_rows, const size_t *n_cols,
                                   int precision, const char *plan_flag);
HPXFFT_API int hpxfft_batch_destroy(hpxfft_batch batch);
HPXFFT_API int hpxfft_batch_arena_bytes(hpxfft_batch batch, size_t *bytes);
HPXFFT_API int hpxfft_batch_offsets(hpxfft_batch batch, size_t *offsets);
HPXFFT_API int hpxfft_batch_set_stream(hpxfft_batch batch, void *cuda_stream);
/* In place on the arena, asynchronous (graph launch on the batch's stream). */
HPXFFT_API int hpxfft_batch_execute(hpxfft_batch batch, void *d_arena);
/* Wait for the last execute; HPXFFT_ERR_TIMEOUT if a bounded device wait gave up. */
HPXFFT_API int hpxfft_batch_synchronize(hpxfft_batch batch);
/* "total" (s, last execute), "plan" (s), "items", "lag", "ctas_per_sm",
 * "algorithmic_bytes", "cached_plan". */
HPXFFT_API int hpxfft_batch_get_measurement(hpxfft_batch batch, const char *name, double *value);

/* Tuned plans, process-wide (batch queue configurations and 2D plan
 * choices): write them to / read them from a text file (the analogue of
 * FFTW wisdom), or drop them.  Import rejects a malformed file whole. */
HPXFFT_API int hpxfft_wisdom_export(const char *path);
HPXFFT_API int hpxfft_wisdom_import(const char *path);
HPXFFT_API int hpxfft_wisdom_forget(void);

/* Forward FP64 transform that allocates nothing, for callers that cannot
 * allocate device memory: an application whose pool allocator already holds
 * all device memory (cudaMalloc would fail or fragment it), or a pipeline
 * that must not call cudaMalloc / cudaFree because they can synchronise the
 * whole device.  d_in and d_out are caller-owned device buffers in the padded
 * layout (they may be equal); the transform is queued on `stream` (NULL is
 * the legacy default stream) and nothing is synchronised.
 * Limits: n_row <= 16384 and ny = n_col - 2 <= 16384, FP64 only; larger
 * sizes return HPXFFT_ERR_UNSUPPORTED_SIZE.  The twiddle tables live in one
 * 1 MiB static __device__ array that each GPU loading the library keeps
 * until the process exits; every call rewrites it, so calls that overlap on
 * the GPU (other streams, other threads) race and must be serialised by the
 * caller.  The first call on a device does a one-time set-up (it looks up
 * the array's device address and sets kernel attributes); make that first
 * call before any stream capture.  "Allocates nothing" holds for this
 * library's own calls: under CUDA's lazy module loading (the default) the
 * driver loads the library's kernels on that first call and may reserve
 * device memory for their code then.  Make the first call on each device
 * before the caller's pool reserves its memory, or run with
 * CUDA_MODULE_LOADING=EAGER.  Later calls, of any supported shape, load no
 * further code.  Shapes whose lengths are not powers of two run kernels
 * with per-thread local memory, for which the driver may enlarge its local
 * memory reservation the first time such a shape runs.  The device-address
 * cache has one slot per device index below 64.  No counterpart in the
 * reference. */
HPXFFT_API int hpxfft_execute_r2c_noalloc(const void *d_in, void *d_out, size_t n_row, size_t n_col, void *stream);

/* Measured FP32 and FP64 FMA throughput of the current device, TFLOP/s
 * (2 flops per FMA; about 40 ms of kernels, allocates a small buffer).  The
 * FP64 drop-in's float-float arithmetic rests on the ratio of the two.  No
 * reference counterpart. */
HPXFFT_API int hpxfft_measure_pipe_peaks(double *fp32_tflops, double *fp64_tflops);

/* Pinned host memory for fast host<->device copies (cudaHostAlloc). */
HPXFFT_API int hpxfft_host_alloc(void **ptr, size_t bytes);
HPXFFT_API int hpxfft_host_free(void *ptr);

#ifdef __cplusplus
}
#endif
#endif
