/*
 * pencilfft_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * PencilFFTs.jl transform path (one GPU, proc_dims all ones, no MPI).
 *
 * All entry points are plain C: integers, sizes and untyped pointers.  Device
 * buffers are raw CUDA device pointers owned by the caller; `stream` is a
 * cudaStream_t passed as `void*` (NULL = legacy default stream).  Every
 * function returns PFGB_OK (0) or a negative status; the message of the last
 * failure on the calling thread is available from pfgb_last_error().
 *
 * Array conventions follow the reference (column-major, Julia indexing):
 *   - input arrays are stored in natural memory order, dimension 1 fastest,
 *     extra (untransformed) dimensions slowest;
 *   - output arrays are stored with the transformed dimensions in reversed
 *     memory order (dimension N fastest) when permute_dims != 0, otherwise in
 *     natural order (reference src/plans.jl:503-521);
 *   - in-place real-to-complex plans (RFFT!) use one buffer whose real view is
 *     padded to 2*(n1/2+1) reals along dimension 1 (reference
 *     src/multiarrays_r2c.jl:69-79).
 */
#ifndef PENCILFFT_GB300_H
#define PENCILFFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFGB_MAX_DIMS 8  /* transformed dimensions */
#define PFGB_MAX_EXTRA 4 /* extra (untransformed, batch) dimensions */

/* Status codes.  The ArgumentError cases of the reference map to
 * PFGB_ERR_ARGUMENT. */
enum {
  PFGB_OK = 0,
  PFGB_ERR_ARGUMENT = -1,    /* invalid descriptor / arrays (ArgumentError) */
  PFGB_ERR_UNSUPPORTED = -2, /* valid request that this build cannot run */
  PFGB_ERR_CUDA = -3,        /* a CUDA runtime call failed */
  PFGB_ERR_ALLOC = -4        /* device or host allocation failed */
};

/* Transform kinds: one per dimension (reference src/Transforms/*.jl). */
enum {
  PFGB_FFT = 0,         /* Transforms.FFT / FFT!   (c2c, sign -1) */
  PFGB_BFFT = 1,        /* Transforms.BFFT / BFFT! (c2c, sign +1, unnormalised) */
  PFGB_RFFT = 2,        /* Transforms.RFFT / RFFT! (r2c, n -> n/2+1) */
  PFGB_BRFFT = 3,       /* Transforms.BRFFT(d) / BRFFT!(d) (c2r); see brfft_even */
  PFGB_R2R = 4,         /* Transforms.R2R(kind) / R2R!(kind); see r2r_kind */
  PFGB_NOTRANSFORM = 5  /* Transforms.NoTransform / NoTransform! */
};

/* FFTW's r2r kind codes (fftw3.h), accepted unchanged in r2r_kind.  R2HC and
 * HC2R are rejected, as in the reference (src/Transforms/r2r.jl:42-45). */
enum {
  PFGB_R2HC = 0, PFGB_HC2R = 1, PFGB_DHT = 2,
  PFGB_REDFT00 = 3, PFGB_REDFT01 = 4, PFGB_REDFT10 = 5, PFGB_REDFT11 = 6,
  PFGB_RODFT00 = 7, PFGB_RODFT01 = 8, PFGB_RODFT10 = 9, PFGB_RODFT11 = 10
};

/* Plan descriptor: the arguments of
 *   PencilFFTPlan(dims_global, transforms, proc_dims, comm, real_type;
 *                 extra_dims, permute_dims)      (reference src/plans.jl:306-320)
 * with proc_dims all ones.  A single transform expanded over all dimensions
 * (reference Transforms.expand_dims) is given here already expanded. */
typedef struct pfgb_plan_desc {
  int32_t ndims;                      /* N >= 1 */
  int64_t dims[PFGB_MAX_DIMS];        /* global input sizes (logical order) */
  int32_t kind[PFGB_MAX_DIMS];        /* PFGB_FFT ... PFGB_NOTRANSFORM */
  int32_t inplace[PFGB_MAX_DIMS];     /* 1 for the "!" variants */
  int32_t r2r_kind[PFGB_MAX_DIMS];    /* FFTW kind code when kind == PFGB_R2R */
  int32_t brfft_even[PFGB_MAX_DIMS];  /* BRFFT.even_output when kind == PFGB_BRFFT */
  int32_t real_bytes;                 /* 4 (Float32) or 8 (Float64) */
  int32_t permute_dims;               /* 1 = Val(true) (default), 0 = Val(false) */
  int32_t n_extra;                    /* number of extra_dims */
  int64_t extra_dims[PFGB_MAX_EXTRA];
  int32_t precision_mode;             /* PFGB_PRECISION_* */
  int32_t autotune;                   /* 0 = off; 1 = measure at plan creation: time
                                         the alternative kernels of each pass on
                                         temporary buffers and keep the faster
                                         (the reference's fftw_flags = FFTW.MEASURE,
                                         src/plans.jl:241-320) */
} pfgb_plan_desc;

/* Arithmetic of the transform kernels.
 *   DEFAULT:  Float32 plans compute in FP32; Float64 plans compute in
 *             double-float (two FP32 values, 48-bit significand, on the FP32
 *             pipes) the c2c / r2c / c2r lines of up to 4096 points (power of
 *             two), 3 * 2^k and 5 * 2^k points, and any other length up to
 *             2048 (Bluestein), REDFT00 / RODFT00 lines of 2^k +- 1 points
 *             and REDFT10 / REDFT01 / RODFT10 / RODFT01 / DHT / REDFT11 /
 *             RODFT11 lines of 2^k points, and every line beyond one pass
 *             (c2c lines split in two passes, r2c / c2r lines as two real
 *             lines packed in one c2c line, lines without a split as a
 *             Bluestein convolution, R2R lines through their extension:
 *             double-float transforms between element maps in FP64), and
 *             the other R2R lines whose extension is a one-pass length
 *             (a double-float c2c pass of the extension between element
 *             maps); the remaining lines (R2R extensions and c2c / r2c / c2r
 *             lines of 2049 .. 8192 points that are neither a power of two,
 *             3 * 2^k nor 5 * 2^k and have no split) in native FP64.  Both
 *             meet a relative L2 error of 1e-13.
 *   NATIVE:   Float64 plans compute every line in native FP64 (GB300's FP64
 *             rate is about 1/70 of its FP32 rate).
 *   TC_SPLIT: Float32 plans only: c2c lines of 256, 512 and 1024 points run
 *             as two DFT-matrix products on the tensor cores (tf32 hi/lo
 *             split, three products, FP32 accumulation); other lines as in
 *             DEFAULT.  Relative L2 error about 1e-6 for a 3D round trip.
 *             FFTW has no such mode.
 *   BLOCK_FLOAT: Float64 plans only: power-of-two c2c/r2c/c2r lines in block
 *             floating point (64-bit integer components, one power-of-two
 *             scale per line, 50 bits below each line's largest component
 *             for 512-point lines, 47 at 4096; exact integer sums); executions
 *             with a fused derivative use double-float.  Relative L2 error
 *             about 2e-14 for a 512^3 round trip; on GB300 about 8% slower
 *             than DEFAULT (the integer pipes run at half the FP32 rate). */
enum {
  PFGB_PRECISION_DEFAULT = 0,
  PFGB_PRECISION_NATIVE = 1,
  PFGB_PRECISION_TC_SPLIT = 2,
  PFGB_PRECISION_BLOCK_FLOAT = 3
};

typedef struct pfgb_plan pfgb_plan;

/* Information about a plan (reference: size(plan), size_global of the input
 * and output pencils, eltype_input/eltype_output, scale_factor, is_inplace). */
typedef struct pfgb_plan_info {
  int32_t ndims;
  int64_t dims_in[PFGB_MAX_DIMS];   /* logical global sizes of the input */
  int64_t dims_out[PFGB_MAX_DIMS];  /* logical global sizes of the output */
  int32_t perm_out[PFGB_MAX_DIMS];  /* memory order of the output: perm_out[0]
                                       is the fastest logical dim (0-based) */
  int32_t eltype_in_complex;        /* 1 if the input element is complex */
  int32_t eltype_out_complex;
  int32_t real_bytes;
  int32_t inplace;
  double scale_factor;              /* product of the per-dimension scales */
  int64_t input_bytes;              /* bytes of the input array (out-of-place) */
  int64_t output_bytes;             /* bytes of the output array (out-of-place) */
  int64_t inplace_bytes;            /* bytes of the aliased buffer (in-place) */
  int64_t scratch_bytes;            /* device scratch the plan holds */
  int32_t n_passes_forward;         /* kernel passes per forward transform */
  int32_t n_passes_backward;
} pfgb_plan_info;

/* Creates a plan (reference PencilFFTPlan constructor, src/plans.jl:241-320,
 * and the 1D plans of src/plans.jl:523-553).  Allocates the device tables and
 * scratch on the current CUDA device. */
int pfgb_plan_create(const pfgb_plan_desc* desc, pfgb_plan** plan);

/* Validates a descriptor and fills `info` as pfgb_plan_create would, on the
 * host only: no device memory is allocated and no CUDA call is made. */
int pfgb_plan_query(const pfgb_plan_desc* desc, pfgb_plan_info* info);

/* Releases a plan and its device memory. */
int pfgb_plan_destroy(pfgb_plan* plan);

/* Fills `info` (reference size(p), scale_factor(p), is_inplace(p),
 * eltype_input/output(p), pencil_output(p) permutation). */
int pfgb_plan_info_get(const pfgb_plan* plan, pfgb_plan_info* info);

/* Forward transform: reference LinearAlgebra.mul!(dst, p, src)
 * (src/operations.jl:24-31).  Out-of-place plans require non-aliased buffers
 * and leave src unchanged; in-place plans require dst == src. */
int pfgb_forward(pfgb_plan* plan, void* dst, const void* src, void* stream);

/* Backward transform: reference ldiv!(dst, p, src) when normalise != 0
 * (src/operations.jl:44-52, scaling fused into the last pass) and
 * bmul!(dst, p, src) when normalise == 0 (src/operations.jl:34-41). */
int pfgb_backward(pfgb_plan* plan, void* dst, const void* src, void* stream,
                  int normalise);

/* Spectral derivative fused into the transform (the callers of the reference's
 * examples/gradient.jl and test/include/FourierOperations.jl, which multiply
 * the spectrum by i k before ldiv!).  pfgb_forward_deriv computes
 * i k_dim * (plan * src); pfgb_backward_deriv computes plan \ (i k_dim * src)
 * (bmul! when normalise == 0) without modifying src.  k = 2 pi f / length with
 * f the fftfreq / rfftfreq frequency of the index along logical dimension
 * `dim` (0-based), which must carry FFT, BFFT, RFFT or BRFFT.  The multiply is
 * applied in the last forward / first backward pass, so it costs no extra
 * sweep; that pass must be complex-to-complex (PFGB_ERR_UNSUPPORTED if not,
 * e.g. for 1D r2c plans). */
int pfgb_forward_deriv(pfgb_plan* plan, void* dst, const void* src, void* stream, int dim,
                       double length);
int pfgb_backward_deriv(pfgb_plan* plan, void* dst, const void* src, void* stream, int normalise,
                        int dim, double length);

/* Sum of spectral derivatives of several fields in one backward transform:
 *   dst = plan \ (sum_t coef[t] * i k_{dim[t]} * src[t]),  1 <= nterm <= 3,
 * with k as in pfgb_backward_deriv (length[t]: domain length along dim[t]);
 * bmul! when normalise == 0.  Replaces the reference's vector calculus in
 * Fourier space followed by one ldiv! per result (divergence and curl!,
 * test/include/FourierOperations.jl:18-86; examples/gradient.jl:48-318): the
 * divergence of u is the three terms (u1, 0, 1), (u2, 1, 1), (u3, 2, 1), and
 * curl component 1 is (u3, 1, 1), (u2, 2, -1).  The sources, which have the
 * plan's output layout, are read once by the first backward pass (a
 * complex-to-complex pass, as for pfgb_backward_deriv) and not modified; the
 * other passes are those of pfgb_backward.  Out-of-place plans only. */
int pfgb_backward_deriv_sum(pfgb_plan* plan, void* dst, const void* const* src, int nterm,
                            const int* dim, const double* coef, const double* length,
                            void* stream, int normalise);

/* Applies one plan to a collection of arrays (reference mul!/ldiv!/bmul!
 * broadcast over tuples or arrays of PencilArrays, src/operations.jl:129-152).
 * direction: +1 forward, -1 backward; normalise as in pfgb_backward. */
int pfgb_execute_many(pfgb_plan* plan, int direction, int normalise,
                      void* const* dst, const void* const* src, int n,
                      void* stream);

/* Batched form: records the launches of n transforms (plans[i] applied in
 * direction[i], +1 forward / -1 backward with normalise[i] as in
 * pfgb_backward, from src[i] to dst[i]) into one CUDA graph, replayed with a
 * single pfgb_batch_launch.  Covers the reference's collections of fields
 * (mul!/ldiv! over tuples and arrays, src/operations.jl:129-152) and any mix
 * of plans and sizes.  The graph has one branch per plan, so transforms of
 * different plans (independent fields) run concurrently; a transform waits
 * for earlier ones of other plans whose buffers overlap its own (written
 * then read, or read or written then written).  The buffers are fixed at
 * creation; plans must outlive the batch and must not run concurrently with
 * it (they share scratch). */
typedef struct pfgb_batch pfgb_batch;
int pfgb_batch_create(pfgb_plan* const* plans, const int* direction, const int* normalise,
                      void* const* dst, const void* const* src, int n, pfgb_batch** batch);
int pfgb_batch_launch(pfgb_batch* batch, void* stream);
int pfgb_batch_destroy(pfgb_batch* batch);

/* One transform of pfgb_batch_create_ex: plan applied in `direction` (+1
 * forward, -1 backward with `normalise` as in pfgb_backward) from src to dst;
 * deriv_dim >= 0 fuses the spectral derivative along that (0-based) logical
 * dimension of a domain of length deriv_length, as pfgb_forward_deriv (on the
 * forward output) and pfgb_backward_deriv (on the backward input) do. */
typedef struct pfgb_batch_op {
  pfgb_plan* plan;
  int32_t direction;
  int32_t normalise;
  void* dst;
  const void* src;
  int32_t deriv_dim;
  int32_t reserved;
  double deriv_length;
} pfgb_batch_op;

/* Forms of a batch.  GRAPH: the launches of every transform recorded into a
 * CUDA graph, one branch per plan (pfgb_batch_create).  PERSISTENT: one
 * launch of a persistent kernel (in a graph with the reset of its counters)
 * that walks a device work list of every tile of every pass of every
 * transform; its CTAs take tiles from a global counter in dependency order
 * and wait, bounded, for the passes each tile depends on (the previous pass
 * of its transform; for a transform's first pass, the last pass of every
 * earlier transform on the same plan or with overlapping buffers).  The
 * list is ordered by dependency level plus a rank that grows by one every
 * 32 MB of data of the earlier transforms, so that the transforms in flight
 * keep their data in L2 between passes.  Float32
 * plans whose passes all have a tile form: c2c / r2c / c2r lines of 2 .. 1024
 * points (powers of two up to 512 on the register tile, 3 * 2^k with
 * 2^k = 128 .. 512 on the mixed-radix tile, the others on the Bluestein
 * tile), with fused single derivatives; otherwise PFGB_ERR_UNSUPPORTED.
 * AUTO: PERSISTENT where possible, else GRAPH.  MEASURE: times the
 * persistent form with waves of 8, 32 and 128 MB and in pure level order,
 * and the graph form, at creation (launching the batch, which overwrites the
 * destination arrays, and in-place sources, as FFTW's MEASURE planning does),
 * and keeps the fastest.  Measured on GB300 (64 Float32 r2c + c2r round
 * trips of 48..192 points per axis: graph 4.8 ms, persistent 6.7 ms; 256 of
 * 16^3: 0.37 and 0.38 ms, against 7.9 ms launched one by one): the graph
 * form's per-pass kernels read their arguments from the constant bank and
 * run each tile at its own kernel's occupancy, the persistent kernel reads
 * them from the work list and runs every tile at two 512-thread CTAs per SM. */
#define PFGB_BATCH_GRAPH 0
#define PFGB_BATCH_PERSISTENT 1
#define PFGB_BATCH_AUTO 2
#define PFGB_BATCH_MEASURE 3
int pfgb_batch_create_ex(const pfgb_batch_op* ops, int n, int form, pfgb_batch** batch);

/* The form a batch was recorded in, and for the persistent form its work
 * list (passes, tiles), grid, dynamic shared memory per CTA and the wave size
 * of the list's order (bytes; 0 for pure dependency-level order); graph_ms
 * and persistent_ms are the times measured by PFGB_BATCH_MEASURE (the best
 * persistent order; 0 otherwise). */
typedef struct pfgb_batch_info {
  int32_t form;
  int32_t transforms;
  int32_t items;
  int32_t grid;
  int64_t tiles;
  int64_t smem;
  double graph_ms;
  double persistent_ms;
  int64_t wave_bytes;
} pfgb_batch_info;
int pfgb_batch_get_info(pfgb_batch* batch, pfgb_batch_info* info);

/* Device-side status of a persistent batch: synchronises `stream`, then
 * returns in *flags, and clears, bit 8 if a dependency wait of the kernel gave
 * up since the last call (every CTA then stopped taking tiles: the outputs of
 * that launch are incomplete; later launches run normally).  0 for the graph
 * form. */
int pfgb_batch_status(pfgb_batch* batch, void* stream, int32_t* flags);

/* Test hook for the give-up path of those waits: polls > 0 bounds every
 * dependency wait of later launches at `polls` polls; 0 restores the default
 * bound (of the order of a second).  PFGB_ERR_ARGUMENT for the graph form. */
int pfgb_batch_set_wait_test(pfgb_batch* batch, int polls);

/* Per-pass timing (replaces the reference's opt-in TimerOutputs sections
 * "PencilFFTs mul!", "FFT", ..., src/operations.jl:27,37,47,250,288,299).
 * When enabled, every kernel launch of the plan is bracketed by CUDA events
 * recorded on the launch stream. */
typedef struct pfgb_pass_timing {
  int32_t direction;      /* +1 forward, -1 backward */
  int32_t pass;           /* index of the pass within its direction */
  int32_t axis;           /* transformed logical dim (0-based), -1 for copies */
  int32_t op;             /* internal operation code */
  int32_t launches;       /* launches recorded since the last reset */
  double total_ms;        /* summed event time of those launches */
  int64_t bytes_per_launch; /* algorithmic bytes: one read of the input plus
                               one write of the output of the pass */
  char kernel[48];        /* kernel name */
} pfgb_pass_timing;

/* Enables (on != 0) or disables per-launch event timing and clears the record. */
int pfgb_plan_set_timing(pfgb_plan* plan, int on);

/* Synchronises on the recorded events and writes up to `max` per-pass entries
 * into `out`; `*n` receives the number of entries. Clears the record. */
int pfgb_plan_get_timing(pfgb_plan* plan, pfgb_pass_timing* out, int max, int* n);

/* Batched 1D Float64 complex FFT that allocates no device memory.
 *
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a memory manager that owns the device budget, a latency-critical path that
 * cannot take cudaMalloc's implicit synchronisation, a host callback where
 * CUDA allocation is not allowed): transforms `howmany` contiguous lines of
 * `n` complex doubles (interleaved re, im) from `in` to `out` (in == out
 * allowed), sign -1 (FFT) or +1 (BFFT, unnormalised), on `stream`, computing
 * in double-float like the Float64 plans.  Its only scratch is a fixed
 * 130,816-byte static device array (exponent word + twiddle tables), so n
 * must be a power of two in [32, 4096]; other sizes return PFGB_ERR_ARGUMENT.
 * Each line is scaled by its own largest exponent, so lines of very
 * different magnitude in one batch keep their accuracy.  The first call on a
 * device (with it current) resolves the array's address and fills the tables
 * with a synchronous copy: make it before any stream capture.  All calls
 * share the array: calls that overlap on the GPU race.  A device reset
 * (cudaDeviceReset) is not supported: the per-device set-up is kept for the
 * life of the process. */
int pfgb_fft1d_noalloc(int sign, int64_t n, int64_t howmany, void* out, const void* in,
                       void* stream);

/* Device-side status of the plan's persistent kernels: synchronises `stream`,
 * then returns in *flags, and clears, the bits set by bounded device waits
 * that gave up since the last call (1: a TMA tile copy of fast_pass_tma,
 * 2: a tensor-core product of tc_pass; the kernel then skipped the rest of
 * its tiles after waiting, again bounded, for the copies and products it had
 * issued; 4: one of those waits gave up too, so the kernel may have released
 * shared or tensor memory that a copy or product still wrote).  The output
 * of an execution that set a bit is incomplete.  No counterpart in the
 * reference: FFTW calls cannot stall on a device. */
int pfgb_device_status(pfgb_plan* plan, void* stream, int32_t* flags);

/* Test hook for the give-up path of those waits; no counterpart in the
 * reference.  polls > 0: in later executions, the first data wait of every
 * CTA of fast_pass_tma and tc_pass polls, `polls` times, an mbarrier that
 * nothing signals, so it gives up and the kernel takes its failure path
 * (status bit 1 or 2) without any wait that could hang.  tma != 0 also runs
 * eligible c2r passes in the TMA-fed form.  polls = 0, tma = 0 restore
 * normal execution. */
int pfgb_plan_set_wait_test(pfgb_plan* plan, int polls, int tma);

/* Planner wisdom (the counterpart of FFTW's wisdom, which the reference's
 * FFTW planner accumulates and FFTW.jl exports and imports): plans created
 * with autotune != 0 first look up the kernel choice of each measured pass
 * (keyed by device, arithmetic and pass geometry) and measure only passes
 * without an entry; every measurement is added.  pfgb_wisdom_export writes
 * the entries to a text file, pfgb_wisdom_import merges a file written by
 * it (PFGB_ERR_ARGUMENT for another format), pfgb_wisdom_forget clears them,
 * pfgb_wisdom_stats reports the number of entries and of lookups answered
 * since the last forget.  None of them needs a GPU. */
int pfgb_wisdom_export(const char* path);
int pfgb_wisdom_import(const char* path);
int pfgb_wisdom_forget(void);
int pfgb_wisdom_stats(int32_t* entries, int32_t* hits);

/* Copies the message of the last failure on this thread into buf. Returns the
 * message length. */
int pfgb_last_error(char* buf, size_t n);

/* Library version string. */
const char* pfgb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PENCILFFT_GB300_H */
