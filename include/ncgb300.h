/*
 * ncgb300.h -- C ABI of the GB300 (sm_103a) device path for ncarray arrays.
 *
 * Every entry point takes plain pointers, sizes and an explicit CUDA stream
 * (a cudaStream_t passed as void*; NULL = legacy default stream). No call
 * synchronises the device or throws: each returns an nca_status and, on
 * failure, nca_last_error() returns a message for the calling thread.
 *
 * The entry points replace the device seam of ncarray v0.7.8:
 *   - ncarray::GPUEngine static functions   src/lib/ncarray/engines/gpuengine.hh:64-638
 *   - device::RuntimeCompiler (NVRTC JIT)   src/lib/ncarray/jit/device/rtcompiler.hh:94-161
 *   - ncarray::Stencil<NDIM>                src/lib/ncarray/expression/stencil.hh:58-255
 *   - device scatter_add (histogram seed)   src/lib/ncarray/device/kernels.cuh:660-680
 * Each declaration below names the reference function it stands in for.
 */
#ifndef NCGB300_H
#define NCGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NCA_MAX_NDIM 10   /* NCARRAY_MAX_NDIM, src/lib/ncarray/custom_types.hh:65-67 */
#define NCA_MAX_OPERANDS 64
#define NCA_MAX_SCALARS 32
#define NCA_MAX_INSTRS 128
#define NCA_MAX_REDUCTIONS 4

/* ---- status codes -------------------------------------------------------- */
typedef enum nca_status {
  NCA_OK = 0,
  NCA_ERR_INVALID = 1,      /* null pointer, bad descriptor, bad tape            */
  NCA_ERR_DTYPE = 2,        /* dtype not supported by this operation             */
  NCA_ERR_SHAPE = 3,        /* shapes do not broadcast / reduce as requested     */
  NCA_ERR_COMPILE = 4,      /* NVRTC failed; nca_last_error() holds the log head */
  NCA_ERR_CUDA = 5,         /* a CUDA runtime/driver call failed                 */
  NCA_ERR_OOM = 6,          /* device scratch allocation failed                  */
  NCA_ERR_TIMEOUT = 7,      /* a bounded device wait gave up (status word set)   */
  NCA_ERR_UNSUPPORTED = 8,  /* valid request the library does not implement     */
  NCA_ERR_LIMIT = 9         /* a size limit of this ABI was exceeded             */
} nca_status;

/* ---- dtypes: numbering of ncarray::DType (src/lib/ncarray/dtype.hh:56-80),
 *      plus two 16-bit float storage types the reference does not have. ---- */
typedef enum nca_dtype {
  NCA_BOOL = 0, NCA_CHAR = 1, NCA_UINT8 = 2, NCA_UINT16 = 3, NCA_UINT32 = 4,
  NCA_UINT64 = 5, NCA_INT8 = 6, NCA_INT16 = 7, NCA_INT32 = 8, NCA_INT64 = 9,
  NCA_FLOAT32 = 10, NCA_FLOAT64 = 11,
  /* 12..21: float128, complex and vector dtypes -- not on the device path */
  NCA_BFLOAT16 = 22, NCA_FLOAT16 = 23
} nca_dtype;

/* ---- opcodes: numbering of ncarray::OpCode (src/lib/ncarray/op_code.hh:47-84),
 *      with ABS and SQRT appended after RSHFT. Instructions are packed as in
 *      pack_instruction (op_code.hh:164-168): (op << 24) | (operand index). -- */
typedef enum nca_opcode {
  NCA_OP_NOOP = 0, NCA_OP_IDX = 1, NCA_OP_LOAD_NCARR = 2, NCA_OP_LOAD_SOARR = 3,
  NCA_OP_LOAD_CONST = 4, NCA_OP_NEG = 5, NCA_OP_INC = 6, NCA_OP_DEC = 7,
  NCA_OP_SZOF = 8, NCA_OP_ADDR = 9, NCA_OP_INDR = 10, NCA_OP_CAST = 11,
  NCA_OP_LNOT = 12, NCA_OP_BNOT = 13, NCA_OP_ADD = 14, NCA_OP_SUB = 15,
  NCA_OP_MUL = 16, NCA_OP_DIV = 17, NCA_OP_MOD = 18, NCA_OP_FDIV = 19,
  NCA_OP_EQ = 20, NCA_OP_NE = 21, NCA_OP_LT = 22, NCA_OP_LE = 23, NCA_OP_GT = 24,
  NCA_OP_GE = 25, NCA_OP_LAND = 26, NCA_OP_LOR = 27, NCA_OP_BAND = 28,
  NCA_OP_BOR = 29, NCA_OP_XOR = 30, NCA_OP_LSHFT = 31, NCA_OP_RSHFT = 32,
  NCA_OP_ABS = 34, NCA_OP_SQRT = 35
} nca_opcode;

/* ---- reductions: SumTraits..MeanTraits (src/lib/ncarray/reductions.hh:109-381) */
typedef enum nca_reduce_op {
  NCA_RED_SUM = 0,     /* out dtype = op_traits<T>::sum_type (bf16/fp16 -> f32)  */
  NCA_RED_MEAN = 1,    /* out dtype = float64 (sum / count)                      */
  NCA_RED_MAX = 2,     /* out dtype = T                                          */
  NCA_RED_MIN = 3,     /* out dtype = T                                          */
  NCA_RED_ARGMAX = 4,  /* out dtype = int64, index along the reduced axes        */
  NCA_RED_ARGMIN = 5   /* out dtype = int64                                      */
} nca_reduce_op;

/*
 * An N-d view: NCOffsetsPolicy semantics (src/lib/ncarray/layout.hh:451-535).
 * Element address = data + sum_k (idx_k * strides[k] + offsets[k]) over the
 * axes k, walked in order, except that on `pointer_axis` (if >= 0) the running
 * pointer p is read as a void* table: p = ((void* const*)p)[idx + offsets[axis]]
 * (offsets[pointer_axis] is an index offset), so axes before the pointer axis
 * move the table pointer and later axes move the panel pointer.
 * With flags = NCA_VIEW_SUBOFFSETS the pointer axis has PEP 3118 suboffset
 * semantics instead (SOArrayPolicy, layout.hh:677-778): p += idx * strides[axis],
 * then p = *(void**)p + offsets[axis].
 * Pointer axes are accepted on operands (expressions, reductions, copies), not
 * on results. Strides and offsets are in BYTES; stride 0 broadcasts an axis.
 */
#define NCA_VIEW_SUBOFFSETS 1
typedef struct nca_view {
  void* data;
  int32_t dtype;
  int32_t ndim;
  int64_t shape[NCA_MAX_NDIM];
  int64_t strides[NCA_MAX_NDIM];
  int64_t offsets[NCA_MAX_NDIM];
  int32_t pointer_axis;
  int32_t flags;            /* 0, or NCA_VIEW_SUBOFFSETS with a pointer axis */
} nca_view;

/*
 * An expression tape: the RPN program of ncarray::ExprMVNode
 * (src/lib/ncarray/expression/mvnode.hh:82-459). LOAD_NCARR/LOAD_SOARR index
 * the operand views, LOAD_CONST the scalars. Every value of the tape is
 * evaluated in `compute_dtype` (the reference's WorkT: the result dtype, or
 * the promoted work dtype when the result is bool -- dynamicmvnode.hh:146-251)
 * and the result is cast to the output view's dtype.
 * Scalars are passed as 8-byte slots: scalar i has dtype scalar_dtypes[i] and
 * its value in the first itemsize bytes of scalar_slots[i].
 */
typedef struct nca_tape {
  const uint32_t* instrs;
  int32_t n_instrs;
  int32_t n_scalars;
  const int32_t* scalar_dtypes;
  const uint64_t* scalar_slots;
  int32_t compute_dtype;
  int32_t result_dtype;     /* dtype of the expression value fed to reductions */
} nca_tape;

/* One reduction of an expression (or of a single view). */
typedef struct nca_reduction {
  int32_t op;               /* nca_reduce_op                                    */
  uint32_t axes_mask;       /* bit k = reduce logical axis k; all bits = full   */
  nca_view out;             /* result: shape = kept axes in order (0-d if full) */
} nca_reduction;

/* ---- library ------------------------------------------------------------- */
const char* nca_last_error(void);
int32_t nca_version(void);
/* Number of kernels launched by this library in this process (all entry points). */
int64_t nca_launch_count(void);
/* Reads and clears the status word that bounded device waits set when they
 * give up (0 = none gave up, NCA_ERR_TIMEOUT otherwise); synchronises `stream`.
 * The reference has no device-side failure reporting (it exits or throws on
 * launch errors only: rtcompiler.hh:68-88, gpuengine.hh:156-158). */
int32_t nca_device_status(int32_t* status, void* stream);
/* Diagnostic: one thread waits on an mbarrier that nothing completes, through
 * the bounded-wait helper of every pipeline kernel, for limit_s seconds
 * (0.001 .. 2); the wait gives up, records NCA_ERR_TIMEOUT in the status word
 * nca_device_status reads, and the kernel returns. Shows that a stuck wait ends
 * with a status and leaves the context usable. No reference counterpart (the
 * reference has no device-side failure reporting). */
int32_t nca_wait_probe(double limit_s, void* stream);
/* Number of JIT kernels compiled / loaded from the disk cache / found in memory. */
int32_t nca_jit_stats(int64_t* compiled, int64_t* disk_hits, int64_t* mem_hits);
/* Directory of the on-disk cubin cache (NULL resets to the default). Replaces
 * the ~/.cache/ncarray lookup of src/lib/ncarray/jit/path_utils.cc:31-50. */
int32_t nca_jit_set_cache_dir(const char* dir);
/* Diagnostic: generates one kernel of every JIT class and compiles it with
 * NVRTC for `arch` (e.g. "sm_103a") without touching a device. No reference
 * counterpart (the reference only compiles on first use, rtcompiler.cc:445-510). */
int32_t nca_jit_selftest(const char* arch, int32_t* n_compiled);

/* ---- launch-schedule autotuner ------------------------------------------- */
/* Schedules (stencil tile shape and z-march depth; threads per block, vector
 * groups per thread and grid cap of the elementwise kernels; thread-team size
 * of row reductions) come from a cache keyed by (op class, dtypes, shape
 * class), stored as `tune.txt` lines "<key> <values...>" in the JIT cache
 * directory. mode 0: built-in heuristics only; 1: cached choices where present
 * (default; NCA_TUNE overrides); 2: a call whose key has no entry first times
 * every candidate on its stream (it synchronises the stream; skipped while the
 * stream is being captured and when an output overlaps an operand) and stores
 * the fastest. The reference launches with a fixed 256-thread block
 * (engines/gpuengine.hh:93-95) and has no tuner. */
int32_t nca_tune_set_mode(int32_t mode);
/* Values cached for `key` (up to cap of them; *n = how many there are, 0 if none). */
int32_t nca_tune_get(const char* key, int32_t* values, int32_t cap, int32_t* n);
/* Forgets every cached choice (memory and file). */
int32_t nca_tune_clear(void);

/* ---- elementwise --------------------------------------------------------- */
/* out[...] = tape(operands...) over the broadcast of the operands to out's shape.
 * Replaces GPUEngine::execute_binary_expression (gpuengine.hh:90-195) with
 * device::RuntimeCompiler::get_expr_kernel / get_dynamic_vm_kernel
 * (rtcompiler.cc:49-89, :341-366). */
int32_t nca_expr_eval(const nca_tape* tape, const nca_view* operands, int32_t n_operands,
                      const nca_view* out, void* stream);

/* One pass that evaluates the tape and (optionally) stores it to `expr_out`
 * while computing up to NCA_MAX_REDUCTIONS reductions of its value over the
 * same axes. The reference materialises the expression and then runs
 * GPUEngine::execute_reduce_axes / execute_full_reduce on it
 * (array_operations.hh:42-63,512-551,904-921); this fuses both. expr_out may
 * be NULL. All reductions must share one axes_mask. The logical shape is the
 * broadcast shape of the operands (or expr_out's shape when given). */
int32_t nca_expr_reduce(const nca_tape* tape, const nca_view* operands, int32_t n_operands,
                        const nca_view* expr_out, const nca_reduction* reds,
                        int32_t n_reds, void* stream);

/* Several expressions over the same operands in one pass. tapes[0] is
 * evaluated, stored to outs[0] and reduced by reds (as nca_expr_reduce;
 * n_reds may be 0), and each further tape i over the same operands is stored
 * elementwise to outs[i] (outs[0]'s shape), with the results of running
 * nca_expr_reduce and then nca_expr_eval for each further tape in order.
 * The pass reads every operand once when the views allow it (transposed
 * operands staged by TMA, 4-byte outputs) and no output overlaps an operand or
 * another output; otherwise the calls run one after another. No reference
 * counterpart: ncarray evaluates each expression in a GPUEngine call of its
 * own (engines/gpuengine.hh:90-195). */
#define NCA_MAX_EXTRA_OUTS 3
int32_t nca_expr_multi(const nca_tape* tapes, int32_t n_tapes, const nca_view* operands, int32_t n_operands,
                       const nca_view* outs, const nca_reduction* reds, int32_t n_reds, void* stream);

/* Reduction of one view: GPUEngine::execute_reduce_axes (gpuengine.hh:222-288)
 * when axes_mask is partial, GPUEngine::execute_full_reduce (:301-333) when it
 * covers every axis. */
int32_t nca_reduce(const nca_view* src, int32_t op, uint32_t axes_mask,
                   const nca_view* out, void* stream);

/* Full reduction of a C-contiguous float32/float64/int32/int64 view that
 * allocates no device memory: for callers that cannot call cudaMalloc or
 * cudaMallocAsync (stream capture that forbids memory nodes, pre-planned
 * real-time loops, hosts that give the library no allocator). No counterpart
 * in the reference. Its per-CTA partials live in a fixed 64 KiB device array
 * inside the library; inputs above 2^31 elements return NCA_ERR_LIMIT. The
 * first call on a device takes that array's address (make it before any
 * stream capture). Calls share the array: calls that overlap on the GPU race.
 * `out` is one element of the dtype nca_reduce would write. */
int32_t nca_reduce_noalloc(const nca_view* src, int32_t op, const nca_view* out, void* stream);

/* dst = cast(src) view to view: GPUEngine::execute_assign / execute_copy_into
 * (gpuengine.hh:377-637; kernels.cuh:613-644). */
int32_t nca_copy(const nca_view* src, const nca_view* dst, void* stream);

/* Host <-> device copy of two views of equal shape and dtype (either may be the
 * host side; pinned host memory makes it asynchronous on `stream`), each
 * contiguous along its innermost axis with positive strides: the outer axes
 * become 2-D copies, no staging kernel. Replaces the host/device transfers of
 * GPUEngine::execute_copy_into (gpuengine.hh:378-510; to_host / to_device,
 * binding_builder.hh:543-591), which copy synchronously and pack strided
 * views through a kernel first. */
int32_t nca_copy_host(const nca_view* src, const nca_view* dst, void* stream);

/* dst[...] = cast(scalar): GPUEngine::execute_fill (gpuengine.hh:338-376). */
int32_t nca_fill(const nca_view* dst, int32_t scalar_dtype, const void* scalar, void* stream);

/* ---- 3-D stencils ---------------------------------------------------------- */
/* dst[c] = src[c] + dt * sum_{o in 3x3x3} w[o] * src[c + o] with zero halo
 * (out-of-grid neighbours read 0). weights[27] is indexed (dz+1)*9+(dy+1)*3+(dx+1);
 * a 7-point stencil sets the 20 edge/corner weights to 0. src and dst are
 * C-contiguous (nz, ny, nx) float32 or float64 grids, distinct buffers.
 * Replaces the device-only Stencil<3>::create/apply of a sum of shifted views
 * (stencil.hh:76-243; rtcompiler.hh:187-385). */
int32_t nca_stencil3d(const nca_view* src, const nca_view* dst, const double* weights27,
                      double dt, void* stream);
/* `iters` Jacobi steps ping-ponging between a and b; the result ends in a if
 * iters is even, else in b. */
int32_t nca_stencil3d_iterate(const nca_view* a, const nca_view* b, const double* weights27,
                              double dt, int32_t iters, void* stream);

/* General stencil of shifted views: for every coordinate c of dest,
 *   dest[c] = tape(src[c*step + o_0], ..., src[c*step + o_{n-1}]),
 *   step[d] = src->shape[d] / dest->shape[d] (integer division, >= 1),
 * where o_i = offsets[i*ndim .. i*ndim+ndim-1] and tape operand i (LOAD_NCARR i)
 * reads offset i. src and dest have the same ndim; src may have a pointer axis
 * (NC or SO), dest may not. Every read must lie inside src (checked:
 * NCA_ERR_SHAPE). At most NCA_MAX_OPERANDS offsets. Does not synchronise, so
 * it can be captured in a CUDA graph. Replaces Stencil<NDIM>::create/apply
 * (expression/stencil.hh:76-243) and its kernel generator
 * (jit/device/rtcompiler.hh:187-385); pro/epilogue code strings
 * (jit/device/extensions.hh:68-72) have no counterpart. */
int32_t nca_stencil(const nca_view* src, const nca_view* dest, const int64_t* offsets, int32_t n_offsets,
                    const nca_tape* tape, void* stream);

/* ---- 2-D histogram ---------------------------------------------------------- */
/* For each point i with x_i, y_i finite: ix = floor((x_i - x_lo) * sx),
 * iy = floor((y_i - y_lo) * sy) evaluated in float32 with sx = (float)(nbx/(x_hi-x_lo)),
 * sy likewise; points with ix or iy outside [0, nb) are dropped.
 * counts[iy*nbx + ix] += 1 (uint64, exact) and, when w != NULL,
 * wsum[iy*nbx + ix] += w_i (float32 output; compensated float32 partial sums,
 * their rounding errors collected exactly, combined in float64).
 * counts/wsum are ACCUMULATED into (zero them first for a fresh histogram).
 * Stands in for the scatter_add primitive (kernels.cuh:660-680;
 * host/elementwise.hh:482-505), which has no public API in the reference. */
int32_t nca_hist2d(const float* x, const float* y, const float* w, int64_t n,
                   int32_t nbx, int32_t nby, double x_lo, double x_hi, double y_lo,
                   double y_hi, uint64_t* counts, float* wsum, void* stream);

/* ---- scatter-add ----------------------------------------------------------- */
/* For every element i of src, in any order: t = indices[i]; when
 * 0 <= t < dest->shape[0], dest[t] += (dest dtype) src[i]. dest is a 1-D view
 * (any byte stride) of int32, uint32, int64, uint64, float32 or float64;
 * indices (int32, uint32, int64 or uint64) and src (any device dtype) are N-d
 * views of one shape. Integer sums wrap; float sums round in the order the
 * additions land (not fixed). No pointer axes. The reference's scatter
 * primitive: host::scatter_add_recursive (host/elementwise.hh:482-505) and
 * scatter_add_kernel (device/kernels.cuh:660-680); its Python binding
 * (pyncarray/binding_builder.hh:708-775) is commented out. */
int32_t nca_scatter_add(const nca_view* dest, const nca_view* indices, const nca_view* src, void* stream);

/* ---- batched uneven reductions -------------------------------------------- */
/* One array of a batch: data pointer, length, dtype (float32/bfloat16/float16). */
typedef struct nca_batch_item {
  const void* data;
  int64_t length;
  int32_t dtype;
  int32_t reserved;
} nca_batch_item;

/* Per-array results of nca_batch_reduce (float64, one row per array). */
typedef struct nca_batch_result {
  double sum;        /* sum(x)          */
  double mean;       /* sum(x) / length */
  double max;        /* max(x)          */
  double sum_sq_m;   /* sum(x*x - x)    */
} nca_batch_result;

/* A prepared batch: device-side work-descriptor table, schedule and (after the
 * first launch) an instantiated CUDA graph for the persistent kernel. */
typedef struct nca_batch nca_batch;

/* Builds the descriptor table for `items` (copied to the device on `stream`).
 * The schedule (chunk size, block size, items per thread) comes from the
 * autotuner cache when present, else from defaults. There is no reference
 * counterpart: ncarray has no batched API (pyncarray/utilities.hh:271-314). */
int32_t nca_batch_create(const nca_batch_item* items, int32_t n_items, nca_batch** out,
                         void* stream);
/* Runs the persistent batched kernel: results[i] for items[i] (device memory). */
int32_t nca_batch_reduce(nca_batch* batch, nca_batch_result* results, void* stream);
/* Same as nca_batch_reduce, replayed through a CUDA graph captured on first use. */
int32_t nca_batch_reduce_graph(nca_batch* batch, nca_batch_result* results, void* stream);
/* The plain form: per array, one launch per op with float64 accumulation. */
int32_t nca_batch_reduce_plain(nca_batch* batch, nca_batch_result* results, void* stream);
/* Times candidate schedules on `stream` and stores the best for this batch's
 * shape class in the autotuner cache (file under the JIT cache directory). */
int32_t nca_batch_autotune(nca_batch* batch, nca_batch_result* results, void* stream);
/* Reports the schedule in use: chunk bytes, consumer threads per block, 16-byte
 * vectors per thread per slab, CTAs. */
int32_t nca_batch_schedule(const nca_batch* batch, int64_t* chunk, int32_t* threads,
                           int32_t* items_per_thread, int32_t* ctas);
/* Status word of the last launch (0 = ok, nonzero = a bounded wait gave up). */
int32_t nca_batch_status(nca_batch* batch, int32_t* status, void* stream);
void nca_batch_destroy(nca_batch* batch);

/* ---- general batched reductions ------------------------------------------- */
/* Items of a general batch: a 1-D array (float32, float64, bfloat16, float16,
 * int32 or int64) and up to NCA_BATCH_MAX_OUTS outputs, each a tape (an index
 * into the tapes given to nca_batch_expr_create; a tape over one operand,
 * LOAD_NCARR 0, with a float32 or float64 result) reduced by an nca_reduce_op.
 * No reference counterpart: ncarray has no batched API
 * (pyncarray/utilities.hh:271-314) and runs one synchronous GPUEngine launch
 * per reduction of each array (engines/gpuengine.hh:222-333). */
#define NCA_BATCH_MAX_OUTS 4
typedef struct nca_batch_expr_item {
  const void* data;
  int64_t length;
  int32_t dtype;
  int32_t n_outs;
  int32_t tape[NCA_BATCH_MAX_OUTS];
  int32_t op[NCA_BATCH_MAX_OUTS];
} nca_batch_expr_item;

/* One result: value (sum, mean, max, min; for argmax/argmin the extreme, or
 * lowest()/max() of the result dtype when no element beats it) and index
 * (argmax/argmin: first index of the extreme, 0 when none; else 0). Results
 * are rows of NCA_BATCH_MAX_OUTS per item, in item order. */
typedef struct nca_batch_value {
  double value;
  int64_t index;
} nca_batch_value;

typedef struct nca_batch_expr nca_batch_expr;

/* Groups the items by (dtype, outputs), splits the arrays into chunks, uploads
 * the tables on `stream` and compiles one persistent kernel for the batch
 * (NVRTC; cached like every JIT kernel). Synchronises `stream`. */
int32_t nca_batch_expr_create(const nca_batch_expr_item* items, int32_t n_items, const nca_tape* tapes,
                              int32_t n_tapes, nca_batch_expr** out, void* stream);
/* One persistent launch for the whole batch; results: device memory, n_items
 * rows of NCA_BATCH_MAX_OUTS. */
int32_t nca_batch_expr_run(nca_batch_expr* batch, nca_batch_value* results, void* stream);
/* The same replayed from a CUDA graph captured on first use (per results
 * pointer and stream). */
int32_t nca_batch_expr_run_graph(nca_batch_expr* batch, nca_batch_value* results, void* stream);
/* The plain form: per item and output one reduction launch of the tape in
 * float64 (float64 accumulation). */
int32_t nca_batch_expr_run_plain(nca_batch_expr* batch, nca_batch_value* results, void* stream);
/* Chunks, distinct programs and CTAs of the persistent launch. */
int32_t nca_batch_expr_info(const nca_batch_expr* batch, int64_t* n_chunks, int32_t* n_programs, int32_t* ctas);
void nca_batch_expr_destroy(nca_batch_expr* batch);

#ifdef __cplusplus
}
#endif

#endif /* NCGB300_H */
