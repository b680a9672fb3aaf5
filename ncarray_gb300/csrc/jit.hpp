// Expression/reduction engine of libncgb300: tape validation, canonical
// iteration space, source generation, NVRTC compilation with an in-memory and
// on-disk cubin cache, and kernel launch.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "common.hpp"

namespace nca {

// Tape after validation, with the reference's evaluation types resolved.
struct Tape {
  std::vector<uint32_t> instrs;
  std::vector<int> scalar_dtypes;
  std::vector<uint64_t> scalar_slots;
  int compute_dtype = NCA_FLOAT64;
  int result_dtype = NCA_FLOAT64;
  bool uses_idx = false;
  int n_arrays = 0;  // 1 + highest LOAD_NCARR/LOAD_SOARR index
};

Tape make_tape(const nca_tape* t, int n_operands);

// The device int that kernels with bounded waits set when a wait gives up
// (read and cleared by nca_device_status).
int* jit_status_word();

// out = tape(operands)
void expr_eval(const Tape& tape, const nca_view* ops, int nops, const nca_view& out,
               cudaStream_t stream);

// one pass: optional out, reductions sharing one axes mask. With nx extra
// tapes (same operands, each stored to xouts[i] of out's shape) the call runs
// only when all of them fuse into the one pass and returns false, launching
// nothing, when they do not; without extras it always runs and returns true.
bool expr_reduce(const Tape& tape, const nca_view* ops, int nops, const nca_view* out,
                 const nca_reduction* reds, int nred, cudaStream_t stream, const Tape* xtapes = nullptr,
                 const nca_view* xouts = nullptr, int nx = 0);

// tapes[0] stored to outs[0] and reduced by reds (nred may be 0), tapes[1..]
// stored to outs[1..]; one pass when it can (see nca_expr_multi)
void expr_multi(const std::vector<Tape>& tapes, const nca_view* ops, int nops, const nca_view* outs,
                const nca_reduction* reds, int nred, cudaStream_t stream);

// expected output dtype of a reduction op over values of dtype `in_dt`
int reduce_out_dtype(int op, int in_dt);

// JIT statistics and cache directory
void jit_stats(int64_t* compiled, int64_t* disk_hits, int64_t* mem_hits);
void jit_set_cache_dir(const char* dir);
std::string jit_cache_dir();

// Compiles (or fetches) a kernel named `name` from CUDA source for the current
// device. Used by the JIT engine and available to other modules.
CUfunction jit_get(const std::string& source, const char* name);

// The device prelude of every JIT kernel (types, 16-bit float conversions,
// the tape operations), and the statements of a tape over the compute type
// `nca_w` ending in `return` (operand k loaded as prefix + k + suffix).
const char* jit_prelude();
std::string jit_gen_eval(const Tape& t, const std::string& load_prefix, const std::string& load_suffix);
// the same over the type named W (its operations specialised by the caller)
std::string jit_gen_eval_w(const Tape& t, const std::string& load_prefix, const std::string& load_suffix,
                           const std::string& W);
// A tape scalar as the 64-bit argument word of compute dtype `compute_dtype`.
uint64_t jit_scalar_word(int compute_dtype, int scalar_dtype, uint64_t slot);
// C type name of an arithmetic dtype in generated device code.
const char* jit_ctype(int dtype);
// Generated-code expressions: the value of `dtype` held as raw bits in the
// integer expression `bits`; the raw bits (u32, or u64 for 8 bytes) of
// `value` stored as `dtype`; the unsigned integer type of `size` bytes.
std::string jit_from_bits(int dtype, const std::string& bits);
std::string jit_to_bits(int dtype, const std::string& value);
std::string jit_storage_uint(int size);

}  // namespace nca

namespace nca {
int jit_selftest(const char* arch);
// NVRTC compile of `source` for `arch` without loading it (fails on errors)
void jit_compile_only(const std::string& source, const std::string& arch);
int batch_expr_selftest(const char* arch);
int stencil_tile_selftest(const char* arch);
}
