// extern "C" entry points of libncgb300 for the expression and reduction path
// (declared in include/ncgb300.h). Each converts internal exceptions to a
// status code; none synchronises the device.
#include <cstring>

#include "common.hpp"
#include "jit.hpp"

using namespace nca;

namespace nca {
int stencil_read_status(cudaStream_t s);
int hist_read_status(cudaStream_t s);
int jit_read_status(cudaStream_t s);
}

extern "C" {

const char* nca_last_error(void) { return last_error().c_str(); }

int32_t nca_version(void) { return 1000; }

int64_t nca_launch_count(void) { return launch_count(); }

int32_t nca_device_status(int32_t* status, void* stream) {
  return guarded([&] {
    if (!status) fail(NCA_ERR_INVALID, "null status");
    const int st = stencil_read_status((cudaStream_t)stream);
    const int hs = hist_read_status((cudaStream_t)stream);
    const int js = jit_read_status((cudaStream_t)stream);
    *status = st != 0 ? st : hs != 0 ? hs : js;
  });
}

int32_t nca_jit_stats(int64_t* compiled, int64_t* disk_hits, int64_t* mem_hits) {
  return guarded([&] { jit_stats(compiled, disk_hits, mem_hits); });
}

int32_t nca_jit_set_cache_dir(const char* dir) {
  return guarded([&] { jit_set_cache_dir(dir); });
}

// Compile-only check of every JIT kernel class for `arch` (no device needed);
// writes the number of kernels compiled to *n_compiled.
int32_t nca_jit_selftest(const char* arch, int32_t* n_compiled) {
  return guarded([&] {
    const int n = jit_selftest(arch);
    if (n_compiled) *n_compiled = n;
  });
}

int32_t nca_expr_eval(const nca_tape* tape, const nca_view* operands, int32_t n_operands,
                      const nca_view* out, void* stream) {
  return guarded([&] {
    if (!out) fail(NCA_ERR_INVALID, "null out view");
    if (n_operands > 0 && !operands) fail(NCA_ERR_INVALID, "null operands");
    Tape t = make_tape(tape, n_operands);
    expr_eval(t, operands, n_operands, *out, (cudaStream_t)stream);
  });
}

int32_t nca_expr_reduce(const nca_tape* tape, const nca_view* operands, int32_t n_operands,
                        const nca_view* expr_out, const nca_reduction* reds, int32_t n_reds,
                        void* stream) {
  return guarded([&] {
    if (!reds) fail(NCA_ERR_INVALID, "null reductions");
    if (n_operands > 0 && !operands) fail(NCA_ERR_INVALID, "null operands");
    Tape t = make_tape(tape, n_operands);
    expr_reduce(t, operands, n_operands, expr_out, reds, n_reds, (cudaStream_t)stream);
  });
}

int32_t nca_expr_multi(const nca_tape* tapes, int32_t n_tapes, const nca_view* operands, int32_t n_operands,
                       const nca_view* outs, const nca_reduction* reds, int32_t n_reds, void* stream) {
  return guarded([&] {
    if (!tapes || !outs) fail(NCA_ERR_INVALID, "null tapes or outputs");
    if (n_tapes < 1) fail(NCA_ERR_INVALID, "at least one tape");
    if (n_reds > 0 && !reds) fail(NCA_ERR_INVALID, "null reductions");
    if (n_operands > 0 && !operands) fail(NCA_ERR_INVALID, "null operands");
    std::vector<Tape> ts;
    for (int i = 0; i < n_tapes; ++i) ts.push_back(make_tape(&tapes[i], n_operands));
    expr_multi(ts, operands, n_operands, outs, reds, n_reds, (cudaStream_t)stream);
  });
}

// identity tape over one view: LOAD_NCARR 0
static nca_tape identity_tape(int dt, uint32_t* instr) {
  nca_tape t;
  memset(&t, 0, sizeof(t));
  *instr = (uint32_t)NCA_OP_LOAD_NCARR << 24;
  t.instrs = instr;
  t.n_instrs = 1;
  t.compute_dtype = arith_dtype(dt);
  t.result_dtype = dt;
  return t;
}

int32_t nca_reduce(const nca_view* src, int32_t op, uint32_t axes_mask, const nca_view* out,
                   void* stream) {
  return guarded([&] {
    if (!src || !out) fail(NCA_ERR_INVALID, "null view");
    if (!dtype_valid(src->dtype)) fail(NCA_ERR_DTYPE, "dtype %d not supported on the device", src->dtype);
    uint32_t ins;
    nca_tape tp = identity_tape(src->dtype, &ins);
    Tape t = make_tape(&tp, 1);
    nca_reduction r;
    r.op = op;
    r.axes_mask = axes_mask;
    r.out = *out;
    expr_reduce(t, src, 1, nullptr, &r, 1, (cudaStream_t)stream);
  });
}

int32_t nca_copy(const nca_view* src, const nca_view* dst, void* stream) {
  return guarded([&] {
    if (!src || !dst) fail(NCA_ERR_INVALID, "null view");
    if (!dtype_valid(dst->dtype)) fail(NCA_ERR_DTYPE, "dtype %d not supported on the device", dst->dtype);
    uint32_t ins;
    nca_tape tp = identity_tape(dst->dtype, &ins);
    tp.result_dtype = dst->dtype;
    Tape t = make_tape(&tp, 1);
    expr_eval(t, src, 1, *dst, (cudaStream_t)stream);
  });
}

int32_t nca_fill(const nca_view* dst, int32_t scalar_dtype, const void* scalar, void* stream) {
  return guarded([&] {
    if (!dst || !scalar) fail(NCA_ERR_INVALID, "null argument");
    if (!dtype_valid(scalar_dtype)) fail(NCA_ERR_DTYPE, "scalar dtype %d unsupported", scalar_dtype);
    if (!dtype_valid(dst->dtype)) fail(NCA_ERR_DTYPE, "dtype %d not supported on the device", dst->dtype);
    uint64_t slot = 0;
    memcpy(&slot, scalar, dtinfo(scalar_dtype).size);
    const uint32_t ins = (uint32_t)NCA_OP_LOAD_CONST << 24;
    nca_tape tp;
    memset(&tp, 0, sizeof(tp));
    tp.instrs = &ins;
    tp.n_instrs = 1;
    tp.n_scalars = 1;
    tp.scalar_dtypes = &scalar_dtype;
    tp.scalar_slots = &slot;
    tp.compute_dtype = arith_dtype(dst->dtype);
    tp.result_dtype = dst->dtype;
    Tape t = make_tape(&tp, 0);
    expr_eval(t, nullptr, 0, *dst, (cudaStream_t)stream);
  });
}

}  // extern "C"
