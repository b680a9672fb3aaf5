// nca_stencil: the general stencil of ncarray's Stencil<NDIM>
// (src/lib/ncarray/expression/stencil.hh:58-255, kernel source generated by
// device::RuntimeCompiler::get_stencil_expr_kernel_str,
// src/lib/ncarray/jit/device/rtcompiler.hh:187-385):
//
//   dest[c] = tape(src[c * step + o_0], ..., src[c * step + o_{k-1}], scalars)
//   step[d] = src.shape[d] / dest.shape[d]   (integer division)
//
// for every coordinate c of dest, with any number of offsets o_i (one per
// tape operand). Each offset becomes one strided view of src (strides scaled
// by step, the offset folded into the view's constant part), so the stencil
// runs through the fused-expression kernels: every operand shares one stride
// set, so the kernels compute one offset per element and add a constant per
// operand; 16-byte vector loads and the stride-2 window loads apply as for
// any expression.
//
// Pointer axes of src: an NC table (layout.hh:468-535) is rewritten as the
// equivalent suboffset view (the table stride becomes step * sizeof(void*),
// the index offset moves into the table base), so a stepped, shifted pointer
// axis needs no new kernel path; SO views (layout.hh:677-778) keep their form.
//
// Differences from the reference, each by design:
//   - every read is checked against src's extents on the host (the reference
//     reads out of bounds when an offset leaves the array); violations return
//     NCA_ERR_SHAPE before anything runs;
//   - the tape is evaluated with the expression engine's rules (the operator
//     set is the full opcode set, not only ADD/SUB/MUL/DIV/GT), in the
//     tape's compute dtype;
//   - the reference's pro/epilogue code strings (StencilJITExtensions,
//     jit/device/extensions.hh:68-72) inject arbitrary CUDA into its kernel;
//     there is no counterpart.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "common.hpp"
#include "jit.hpp"

namespace nca {
namespace {

void check_stencil_view(const nca_view& v, const char* what) {
  if (v.ndim < 1 || v.ndim > NCA_MAX_NDIM) fail(NCA_ERR_LIMIT, "%s: ndim %d (1..%d)", what, v.ndim, NCA_MAX_NDIM);
  for (int d = 0; d < v.ndim; ++d)
    if (v.shape[d] < 0) fail(NCA_ERR_SHAPE, "%s: negative extent", what);
}

// ---------------------------------------------------------------------------
// Tiled form (step 1 on every axis, plain source and destination views, up to
// three dims). The view form (stencil_operand below) reads every operand from
// global memory, one load per offset per point; with a zero-padded source the
// rows are not on the 16-byte grid, so a 27-offset stencil issues 27 scalar
// loads per point. The tiled form reads every source element about once:
//
//   * a CTA of 32 x BY threads owns an output tile of TX = 32*VX columns by
//     TY = BY*VY rows and marches ZC planes along z (the outermost axis);
//   * the source planes it needs (TY + SY - 1 rows of TX + SX - 1 elements,
//     SX/SY/SZ the extents of the offset set) stream by cp.async into a ring
//     of PD + 1 + BACK stages in shared memory, PD planes ahead of the newest
//     one in use, BACK planes kept behind it;
//   * each thread owns VY adjacent output rows (and VX columns 32 apart); a
//     cell is one (row of its strip + dy, dx) position the offsets read. A
//     cell read at several z offsets (every cell of a 3x3x3 set, the centre
//     column of the 7-point one) has a register window: the last SZ planes'
//     values, converted to the compute type once, so a plane step reads each
//     such cell once for all the outputs that share it; the z loop is
//     unrolled SZ times so the window rotates by renaming, not by moves;
//   * a cell read at one z offset only (the faces of the 7-point set) is read
//     from the ring when the outputs need it, up to BACK planes behind;
//   * VY is the tallest strip (4, 2, 1) whose window fits 64 registers: a
//     3x3x3 set reads 18 cells per 4 outputs, the 7-point set 14 per 4;
//   * the tape is then evaluated per output exactly as the expression kernels
//     evaluate it (same operand conversion, same operations in the same
//     order), so both forms give the same bits.
//
// Plans are generated per (tape, offsets, dtypes, tile) and cached.
// NCA_STENCIL_TILE=0 selects the view form, =2 makes a stencil that does not
// fit the tiled form an error (tests); NCA_STENCIL_TILE_CFG="vx,vy,by,pd,zc[,minb]"
// overrides the tile (measurements).
// ---------------------------------------------------------------------------
struct TilePlan {
  int sz = 1, sy = 1, sx = 1;             // extents of the normalised offset set
  int vx = 1, vy = 2, by = 8, pd = 3, zc = 1;   // pd: planes in flight ahead of the one in use
  bool cpa = true;                        // cp.async staging (4- and 8-byte elements)
  bool off32 = false;                     // in-plane byte offsets fit 32 bits
  int minb = 0;                           // __launch_bounds__ minimum CTAs per SM (0: none)
  bool pk = false;                        // float32 tape on column pairs (i, i + 1) in f32x2 instructions
  std::vector<int> dz, dy, dx;            // per operand: its normalised offset
  // a cell: one (row of the thread's VY-row strip plus dy, dx) position, with
  // the z offsets read there; read at several, it has a register window
  struct Cell { int r, x; std::vector<int> zs; bool win; };
  std::vector<Cell> cells;
  std::vector<int> cell_of;               // [k * vy + jj]: the cell operand k of output row jj reads
  int back = 0;                           // planes behind the newest that direct reads reach
  int stages() const { return pd + 1 + back; }
  int window_regs(int wsize) const {      // 32-bit registers of the window
    int n = 0;
    for (const Cell& c : cells) n += c.win ? sz * vx * std::max(1, wsize / 4) : 0;
    return n;
  }
};

// The cells of plan P for its vy.
void plan_cells(TilePlan& P) {
  P.cells.clear();
  P.cell_of.assign(P.dz.size() * (size_t)P.vy, 0);
  P.back = 0;
  for (size_t k = 0; k < P.dz.size(); ++k)
    for (int jj = 0; jj < P.vy; ++jj) {
      const int r = jj + P.dy[k], x = P.dx[k];
      size_t c = 0;
      while (c < P.cells.size() && !(P.cells[c].r == r && P.cells[c].x == x)) ++c;
      if (c == P.cells.size()) P.cells.push_back({r, x, {}, false});
      auto& zs = P.cells[c].zs;
      if (std::find(zs.begin(), zs.end(), P.dz[k]) == zs.end()) zs.push_back(P.dz[k]);
      P.cell_of[k * (size_t)P.vy + (size_t)jj] = (int)c;
    }
  for (auto& c : P.cells) {
    c.win = c.zs.size() > 1;
    if (!c.win) P.back = std::max(P.back, P.sz - 1 - c.zs[0]);
  }
}

int tile_mode() {
  const char* e = getenv("NCA_STENCIL_TILE");
  return e && *e ? atoi(e) : 1;
}

std::string tile_source(const TilePlan& P, const Tape& t, int src_dt, int dst_dt, int nscal) {
  std::ostringstream os;
  const int es = dtinfo(src_dt).size, ds = dtinfo(dst_dt).size;
  const int tx = 32 * P.vx, ty = P.by * P.vy, nt = 32 * P.by;
  const int pc = tx + P.sx - 1, pr = ty + P.sy - 1, pe = pc * pr;
  const int ke = (pe + nt - 1) / nt;   // staging copies per thread per plane
  const std::string S = jit_storage_uint(es), D = jit_storage_uint(ds);
  const char* OT = P.off32 ? "int" : "i64";   // type of the in-plane offsets
  os << jit_prelude();
  os << "typedef " << jit_ctype(t.compute_dtype) << " nca_w;\ntypedef " << S << " nca_s;\n";
  os << "struct NcaStArgs { u64 w[" << 14 + std::max(nscal, 1) << "]; };\n";
  os << "__device__ __forceinline__ nca_w nca_sv(const nca_w* v, const u64* s) {\n  (void)s; const i64 lin = 0; (void)lin;\n"
     << jit_gen_eval(t, "v[", "]") << "}\n";
  if (P.pk) {
    // two float32 lanes per instruction: add, sub and multiply each as one
    // packed fused multiply-add (a + b = fma(a, 1, b), a - b = fma(b, -1, a),
    // a * b = fma(a, b, -0): one rounding, signed zeros as IEEE add, sub and
    // mul; a separate packed mul and add could be contracted into one fma),
    // division, negation and absolute value lane by lane
    os << "struct nca_f2 { u64 v; };   // lanes x (low word) and y\n"
       << "__device__ __forceinline__ u64 nca_pk2(float x, float y) { u64 r; asm(\"mov.b64 %0, {%1, %2};\" : \"=l\"(r) : \"f\"(x), \"f\"(y)); return r; }\n"
       << "__device__ __forceinline__ float nca_lo2(u64 r) { float x, y; asm(\"mov.b64 {%0, %1}, %2;\" : \"=f\"(x), \"=f\"(y) : \"l\"(r)); return x; }\n"
       << "__device__ __forceinline__ float nca_hi2(u64 r) { float x, y; asm(\"mov.b64 {%0, %1}, %2;\" : \"=f\"(x), \"=f\"(y) : \"l\"(r)); return y; }\n"
       << "template <> __device__ __forceinline__ nca_f2 nca_word<nca_f2>(u64 b) { const float f = __uint_as_float((u32)b); return {nca_pk2(f, f)}; }\n";
    // the constant pairs (1, 1), (-1, -1), (-0, -0) are read from device
    // memory so that the assembler cannot see them and turn the fma back into
    // a mul or an add
    os << "__device__ u64 nca_f2c[3] = {0x3f8000003f800000ull, 0xbf800000bf800000ull, 0x8000000080000000ull};\n"
       << "__device__ __forceinline__ nca_f2 nca_f2fma(u64 a, u64 b, u64 c) { u64 d; asm(\"fma.rn.f32x2 %0, %1, %2, %3;\" "
          ": \"=l\"(d) : \"l\"(a), \"l\"(b), \"l\"(c)); return {d}; }\n";
    const char* pops[][2] = {{"nca_add", "nca_f2fma(a.v, nca_f2c[0], b.v)"},
                             {"nca_sub", "nca_f2fma(b.v, nca_f2c[1], a.v)"},
                             {"nca_mul", "nca_f2fma(a.v, b.v, nca_f2c[2])"},
                             {"nca_mulc", "nca_f2fma(a.v, b.v, nca_f2c[2])"}};
    for (auto& o : pops)
      os << "template <> __device__ __forceinline__ nca_f2 " << o[0] << "<nca_f2>(nca_f2 a, nca_f2 b) { return " << o[1]
         << "; }\n";
    os << "template <> __device__ __forceinline__ nca_f2 nca_div<nca_f2>(nca_f2 a, nca_f2 b) { return {nca_pk2(nca_div<float>(nca_lo2(a.v), nca_lo2(b.v)), nca_div<float>(nca_hi2(a.v), nca_hi2(b.v)))}; }\n"
       << "template <> __device__ __forceinline__ nca_f2 nca_neg<nca_f2>(nca_f2 a) { return {nca_pk2(nca_neg<float>(nca_lo2(a.v)), nca_neg<float>(nca_hi2(a.v)))}; }\n"
       << "template <> __device__ __forceinline__ nca_f2 nca_abs<nca_f2>(nca_f2 a) { return {nca_pk2(nca_abs<float>(nca_lo2(a.v)), nca_abs<float>(nca_hi2(a.v)))}; }\n";
    os << "__device__ __forceinline__ nca_f2 nca_sv2(const nca_f2* v, const u64* s) {\n  (void)s;\n"
       << jit_gen_eval_w(t, "v[", "]", "nca_f2") << "}\n";
  }
  os << "__device__ __forceinline__ nca_w nca_sl(nca_s b) { return (nca_w)(" << jit_from_bits(src_dt, "b") << "); }\n";
  os << "__device__ __forceinline__ void nca_sput(char* p, nca_w e) { *(" << D << "*)p = (" << D << ")"
     << jit_to_bits(dst_dt, "e") << "; }\n";
  os << "extern \"C\" __global__ void __launch_bounds__(" << nt;
  if (P.minb > 0) os << ", " << P.minb;
  os << ") nca_stencil_tile(const NcaStArgs A) {\n"
     << "  __shared__ __align__(16) nca_s buf[" << P.stages() * pe << "];\n"
     << "  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;\n"
     << "  const i64 x0 = (i64)blockIdx.x * " << tx << ", y0 = (i64)blockIdx.y * " << ty
     << ", z0 = (i64)blockIdx.z * " << P.zc << ";\n"
     << "  const char* const sb = (const char*)A.w[0];\n  char* const db = (char*)A.w[1];\n"
     << "  const i64 ssz = (i64)A.w[2], ssy = (i64)A.w[3], ssx = (i64)A.w[4];\n"
     << "  const i64 dsz = (i64)A.w[5], dsy = (i64)A.w[6], dsx = (i64)A.w[7];\n"
     << "  const i64 nz = (i64)A.w[8], ny = (i64)A.w[9], nx = (i64)A.w[10];\n"
     << "  const i64 sny = (i64)A.w[12], snx = (i64)A.w[13];\n"
     << "  const u64* const s = A.w + 14;\n"
     << "  const int J = (int)(nz - z0 < " << P.zc << " ? nz - z0 : " << P.zc << ") + " << P.sz - 1 << ";\n";
  // per-thread staging offsets (the same in every plane)
  for (int k = 0; k < ke; ++k) {
    os << "  " << OT << " go" << k << " = 0; bool gv" << k << " = false;\n"
       << "  { const int e = tid + " << k * nt << "; const int r = e / " << pc << ", c = e - r * " << pc << ";\n"
       << "    const i64 ys = y0 + r, xs = x0 + c;\n"
       << "    gv" << k << " = e < " << pe << " && ys < sny && xs < snx; go" << k << " = (" << OT
       << ")(ys * ssy + xs * ssx); }\n";
  }
  // the next plane to issue: its index, stage (shared address) and source row
  os << "  int jiss = 0, ist = 0, rst = 0;\n"
     << "  const u32 sm0 = (u32)__cvta_generic_to_shared(buf) + (u32)tid * " << es << "u;\n"
     << "  u32 sdst = sm0;\n  i64 gzo = z0 * ssz;\n";
  // one plane into stage ist, then a commit (an empty group past the last plane)
  os << "#define NCA_ST_ISSUE() do { \\\n    if (jiss < J) { \\\n";
  for (int k = 0; k < ke; ++k) {
    if (P.cpa)
      os << "      if (gv" << k << ") asm volatile(\"cp.async.ca.shared.global [%0+" << k * nt * es << "], [%1], " << es
         << ";\\n\" :: \"r\"(sdst), \"l\"(sb + gzo + go" << k << ") : \"memory\"); \\\n";
    else
      os << "      if (gv" << k << ") buf[ist * " << pe << " + tid + " << k * nt << "] = *(const nca_s*)(sb + gzo + go" << k
         << "); \\\n";
  }
  os << "    } \\\n    asm volatile(\"cp.async.commit_group;\\n\" ::: \"memory\"); \\\n"
     << "    ++jiss; gzo += ssz; \\\n"
     << "    if (++ist == " << P.stages() << ") { ist = 0; sdst = sm0; } else sdst += " << pe * es << "u; \\\n"
     << "  } while (0)\n";
  // per output (column i, row jj of the thread's strip): its offset in a
  // destination plane and whether it exists
  for (int i = 0; i < P.vx; ++i)
    for (int jj = 0; jj < P.vy; ++jj)
      os << "  const i64 ox" << i << "_" << jj << " = x0 + tx + " << 32 * i << ", oy" << i << "_" << jj << " = y0 + ty * "
         << P.vy << " + " << jj << ";\n  const bool ok" << i << "_" << jj << " = ox" << i << "_" << jj << " < nx && oy" << i
         << "_" << jj << " < ny;\n  const " << OT << " oo" << i << "_" << jj << " = (" << OT << ")(oy" << i << "_" << jj
         << " * dsy + ox" << i << "_" << jj << " * dsx);\n";
  os << "  i64 dzo = (z0 - " << P.sz - 1 << ") * dsz;\n";
  const int ncell = (int)P.cells.size();
  const int nst = P.stages();
  for (int c = 0; c < ncell; ++c)
    if (P.cells[(size_t)c].win)
      for (int m = 0; m < P.sz; ++m)
        for (int i = 0; i < P.vx; i += P.pk ? 2 : 1)
          os << "  " << (P.pk ? "u64" : "nca_w") << " w" << c << "_" << m << "_" << i << " = 0;\n";
  os << "  for (int k = 0; k < " << P.pd << "; ++k) NCA_ST_ISSUE();\n";
  os << "  const int lb = ty * " << P.vy * pc << " + tx;\n";
  os << "  for (int jb = 0; jb < J; jb += " << P.sz << ") {\n";
  auto at = [&](int c, int i) { return P.cells[(size_t)c].r * pc + P.cells[(size_t)c].x + 32 * i; };
  // direct reads: plane j - (SZ - 1) + dz sits SZ - 1 - dz stages behind the newest
  std::vector<bool> back_used((size_t)P.sz, false);
  for (const auto& c : P.cells)
    if (!c.win) back_used[(size_t)(P.sz - 1 - c.zs[0])] = true;
  for (int u = 0; u < P.sz; ++u) {
    os << "    if (jb + " << u << " < J) {\n"
       << "      const int j = jb + " << u << ";\n"
       << "      asm volatile(\"cp.async.wait_group " << P.pd - 1 << ";\\n\" ::: \"memory\");\n"
       << "      __syncthreads();\n"
       << "      NCA_ST_ISSUE();\n"
       << "      const nca_s* const pl = buf + rst * " << pe << " + lb;\n";
    for (int c = 0; c < ncell; ++c)
      if (P.cells[(size_t)c].win)
        for (int i = 0; i < P.vx; ++i)
          if (!P.pk) os << "      w" << c << "_" << u << "_" << i << " = nca_sl(pl[" << at(c, i) << "]);\n";
          else if (i % 2 == 0)
            os << "      w" << c << "_" << u << "_" << i << " = nca_pk2(nca_sl(pl[" << at(c, i) << "]), nca_sl(pl["
               << at(c, i + 1) << "]));\n";
    os << "      if (j >= " << P.sz - 1 << ") {\n";
    for (int b = 0; b < P.sz; ++b)
      if (back_used[(size_t)b])
        os << "        const nca_s* const pb" << b << " = buf + (rst >= " << b << " ? rst - " << b << " : rst + "
           << nst - b << ") * " << pe << " + lb;\n";
    for (int c = 0; c < ncell; ++c)
      if (!P.cells[(size_t)c].win)
        for (int i = 0; i < P.vx; ++i)
          if (!P.pk)
            os << "        const nca_w d" << c << "_" << i << " = nca_sl(pb" << P.sz - 1 - P.cells[(size_t)c].zs[0] << "["
               << at(c, i) << "]);\n";
          else if (i % 2 == 0)
            os << "        const u64 d" << c << "_" << i << " = nca_pk2(nca_sl(pb" << P.sz - 1 - P.cells[(size_t)c].zs[0]
               << "[" << at(c, i) << "]), nca_sl(pb" << P.sz - 1 - P.cells[(size_t)c].zs[0] << "[" << at(c, i + 1) << "]));\n";
    auto operand = [&](int k, int i, int jj) {
      const int c = P.cell_of[(size_t)k * (size_t)P.vy + (size_t)jj];
      if (P.cells[(size_t)c].win) return "w" + std::to_string(c) + "_" + std::to_string((u + 1 + P.dz[(size_t)k]) % P.sz) +
                                        "_" + std::to_string(i);
      return "d" + std::to_string(c) + "_" + std::to_string(i);
    };
    for (int i = 0; i < P.vx; i += P.pk ? 2 : 1)
      for (int jj = 0; jj < P.vy; ++jj) {
        const std::string a = std::to_string(i) + "_" + std::to_string(jj), b = std::to_string(i + 1) + "_" + std::to_string(jj);
        if (P.pk) {
          os << "        if (ok" << a << " || ok" << b << ") {\n          const nca_f2 v[" << P.dz.size() << "] = {";
          for (size_t k = 0; k < P.dz.size(); ++k)
            os << (k ? ", " : "") << "{" << operand((int)k, i, jj) << "}";
          os << "};\n          const u64 r = nca_sv2(v, s).v;\n"
             << "          if (ok" << a << ") nca_sput(db + dzo + oo" << a << ", nca_lo2(r));\n"
             << "          if (ok" << b << ") nca_sput(db + dzo + oo" << b << ", nca_hi2(r));\n        }\n";
          continue;
        }
        os << "        if (ok" << a << ") {\n          const nca_w v[" << P.dz.size() << "] = {";
        for (size_t k = 0; k < P.dz.size(); ++k) os << (k ? ", " : "") << operand((int)k, i, jj);
        os << "};\n          nca_sput(db + dzo + oo" << a << ", nca_sv(v, s));\n        }\n";
      }
    os << "      }\n      dzo += dsz;\n      rst = rst + 1 == " << nst << " ? 0 : rst + 1;\n    }\n";
  }
  os << "  }\n  asm volatile(\"cp.async.wait_group 0;\\n\" ::: \"memory\");\n}\n";
  return os.str();
}

// NCA_STENCIL_TILE_PK=1 and a tape that reads only operands and constants and
// applies only add, sub, mul, div, neg and abs (the operations of the
// column-pair evaluator). Opt-in: measured on GB300 (512^3 float32, padded
// source) the 27-point Laplacian at 2830 GB/s against 3417 one column at a
// time, the 7-point at 4824 against 5055 (the pairs need more registers and
// the packed fma issues no faster than two float32 instructions here).
bool pk_tape(const Tape& t) {
  const char* e = getenv("NCA_STENCIL_TILE_PK");
  if (!(e && e[0] == '1')) return false;
  for (uint32_t ins : t.instrs) {
    switch ((int)(ins >> 24)) {
      case NCA_OP_NOOP: case NCA_OP_LOAD_NCARR: case NCA_OP_LOAD_SOARR: case NCA_OP_LOAD_CONST: case NCA_OP_ADD:
      case NCA_OP_SUB: case NCA_OP_MUL: case NCA_OP_DIV: case NCA_OP_NEG: case NCA_OP_ABS: break;
      default: return false;
    }
  }
  return true;
}

// The offset set and tape as a tile plan (host only); null when they fit,
// else the reason.
const char* plan_tile(const int64_t* offsets, int n, int nd, const Tape& t, TilePlan& P, int64_t* mn) {
  if (nd > 3) return "more than 3 dims";
  if (t.uses_idx) return "the tape reads the element index";
  int64_t mx[3] = {0, 0, 0};
  mn[0] = mn[1] = mn[2] = 0;
  const int lead = 3 - nd;
  for (int d = 0; d < nd; ++d) {
    mn[lead + d] = mx[lead + d] = offsets[d];
    for (int k = 1; k < n; ++k) {
      mn[lead + d] = std::min(mn[lead + d], offsets[(int64_t)k * nd + d]);
      mx[lead + d] = std::max(mx[lead + d], offsets[(int64_t)k * nd + d]);
    }
  }
  P.sz = (int)(mx[0] - mn[0] + 1); P.sy = (int)(mx[1] - mn[1] + 1); P.sx = (int)(mx[2] - mn[2] + 1);
  if (P.sz > 5 || P.sy > 9 || P.sx > 9) return "an offset set wider than 5 x 9 x 9";
  for (int k = 0; k < n; ++k) {
    int o[3] = {0, 0, 0};
    for (int d = 0; d < nd; ++d) o[lead + d] = (int)(offsets[(int64_t)k * nd + d] - mn[lead + d]);
    P.dz.push_back(o[0]); P.dy.push_back(o[1]); P.dx.push_back(o[2]);
  }
  // float32 tapes of add, sub, mul, div, neg and abs, when asked for: column
  // pairs in f32x2 instructions (two columns per thread, 32 apart)
  P.pk = arith_dtype(t.compute_dtype) == NCA_FLOAT32 && pk_tape(t);
  // the tallest strip (4, 2 or 1 rows per thread) whose register window
  // stays within 64 registers (80 for column pairs); a wide window (over 32
  // registers) in CTAs of 4 warps, at least 4 per SM, else CTAs of 8 warps,
  // at least 2 per SM
  const int wsize = dtinfo(t.compute_dtype).size;
  P.vx = P.pk ? 2 : 1;
  for (int vy : {4, 2, 1}) {
    P.vy = vy;
    plan_cells(P);
    if (P.window_regs(wsize) <= (P.pk ? 80 : 64)) break;
  }
  const int wregs = P.window_regs(wsize) / P.vx;
  if (wregs > 96) return "a register window over 96 registers";
  P.by = wregs > 32 ? 4 : 8;
  P.minb = wregs > 32 ? 4 : 2;
  return nullptr;
}

// byte range [lo, hi) a plain view can touch
void view_span(const nca_view& v, uintptr_t& lo, uintptr_t& hi) {
  intptr_t a = (intptr_t)v.data, b = (intptr_t)v.data;
  for (int d = 0; d < v.ndim; ++d) {
    a += v.offsets[d]; b += v.offsets[d];
    const intptr_t e = (intptr_t)(v.shape[d] - 1) * v.strides[d];
    if (e < 0) a += e; else b += e;
  }
  lo = (uintptr_t)a;
  hi = (uintptr_t)b + (uintptr_t)dtinfo(v.dtype).size;
}

// The tiled form, when it applies (returns false, launching nothing, when not).
bool stencil_tile(const nca_view& src, const nca_view& dest, const int64_t* step, const int64_t* offsets, int n,
                  const Tape& t, cudaStream_t stream) {
  const int mode = tile_mode();
  if (mode == 0) return false;
  const int nd = src.ndim;
  auto refuse = [&](const char* why) {
    if (mode == 2) fail(NCA_ERR_UNSUPPORTED, "tiled stencil: %s", why);
    return false;
  };
  if (src.pointer_axis >= 0) return refuse("pointer-axis source");
  for (int d = 0; d < nd; ++d)
    if (step[d] != 1) return refuse("a source/destination ratio other than 1");
  {
    uintptr_t slo, shi, dlo, dhi;
    view_span(src, slo, shi);
    view_span(dest, dlo, dhi);
    if (slo < dhi && dlo < shi) return refuse("the destination overlaps the source");
  }
  TilePlan P;
  int64_t mn[3];
  if (const char* why = plan_tile(offsets, n, nd, t, P, mn)) return refuse(why);
  const int lead = 3 - nd;
  const int es = dtinfo(src.dtype).size;
  int64_t sh[3] = {1, 1, 1}, ss[3] = {0, 0, 0}, dsh[3] = {1, 1, 1}, dst[3] = {0, 0, 0};
  for (int d = 0; d < nd; ++d) {
    sh[lead + d] = src.shape[d]; ss[lead + d] = src.strides[d];
    dsh[lead + d] = dest.shape[d]; dst[lead + d] = dest.strides[d];
  }
  const char* base = static_cast<const char*>(src.data);
  for (int d = 0; d < nd; ++d) base += src.offsets[d];
  for (int a = 0; a < 3; ++a) base += mn[a] * ss[a];
  char* dbase = static_cast<char*>(dest.data);
  for (int d = 0; d < nd; ++d) dbase += dest.offsets[d];
  P.cpa = (es == 4 || es == 8) && (uintptr_t)base % (uintptr_t)es == 0;
  for (int a = 0; a < 3; ++a) if (ss[a] % es) P.cpa = false;
  const int dev = current_device();
  const int sms = sm_count(dev);
  bool zc_set = false;
  if (const char* e = getenv("NCA_STENCIL_TILE_CFG")) {
    int v[6] = {0, 0, 0, 0, 0, 0};
    if (sscanf(e, "%d,%d,%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]) >= 5 && v[0] >= 1 && v[0] <= 4 &&
        v[1] >= 1 && v[1] <= 8 && (v[2] == 2 || v[2] == 4 || v[2] == 8 || v[2] == 16) && v[3] >= 1 && v[3] <= 8 &&
        v[4] >= 1 && v[5] >= 0 && v[5] <= 16) {
      P.vx = v[0]; P.vy = v[1]; P.by = v[2]; P.pd = v[3]; P.zc = v[4]; P.minb = v[5];
      if (P.vx % 2) P.pk = false;
      zc_set = true;
      plan_cells(P);
    }
  }
  {
    // in-plane byte offsets of the staged source rows and of the outputs
    const int64_t lim = 0x7fffffffLL;
    int64_t so = 0, dof = 0;
    so += std::llabs(ss[1]) * (sh[1] - mn[1]) + std::llabs(ss[2]) * (sh[2] - mn[2]);
    dof += std::llabs(dst[1]) * (dsh[1] + 64) + std::llabs(dst[2]) * (dsh[2] + 128);
    P.off32 = so < lim && dof < lim;
  }
  // the ring within 48 KiB: fewer planes in flight, then shorter strips
  auto ring_bytes = [&] {
    return (int64_t)P.stages() * (32 * P.vx + P.sx - 1) * (P.by * P.vy + P.sy - 1) * es;
  };
  for (;;) {
    while (P.pd > 1 && ring_bytes() > 48 * 1024) --P.pd;
    if (ring_bytes() <= 48 * 1024 || P.vy == 1) break;
    P.vy /= 2;
    P.pd = 3;
    plan_cells(P);
  }
  if (ring_bytes() > 48 * 1024) return refuse("a tile over 48 KiB of shared memory");
  const int tx = 32 * P.vx, ty = P.by * P.vy;
  const int64_t gx = (dsh[2] + tx - 1) / tx, gy = (dsh[1] + ty - 1) / ty;
  if (!zc_set) {
    // about 16 CTAs per SM over the grid, 16..32 planes per CTA
    const int64_t want = (int64_t)sms * 16;
    int64_t zc = (dsh[0] * gx * gy + want - 1) / want;
    zc = std::max<int64_t>(16, std::min<int64_t>(32, zc));
    P.zc = (int)std::min<int64_t>(zc, dsh[0]);
  }
  const int64_t gz = (dsh[0] + P.zc - 1) / P.zc;
  if (gy > 65535 || gz > 65535 || gx > 0x7fffffff) return refuse("a grid over the launch limits");
  const int nscal = (int)t.scalar_dtypes.size();
  // the plan: compiled source per (tape, offsets, dtypes, tile)
  std::ostringstream key;
  key << dev << '|' << src.dtype << '|' << dest.dtype << '|' << t.compute_dtype << '|' << P.vx << P.vy << ',' << P.by
      << ',' << P.pd << ',' << P.zc << ',' << P.cpa << P.off32 << P.pk << ',' << P.minb << '|' << P.sz << P.sy << P.sx << '|';
  for (int k = 0; k < n; ++k) key << P.dz[(size_t)k] << ',' << P.dy[(size_t)k] << ',' << P.dx[(size_t)k] << ';';
  key << '|';
  for (uint32_t ins : t.instrs) key << ins << ',';
  key << '|';
  for (int k = 0; k < nscal; ++k) key << t.scalar_dtypes[(size_t)k] << ':' << t.scalar_slots[(size_t)k] << ',';
  static std::mutex m;
  static std::map<std::string, CUfunction> plans;
  CUfunction fn = nullptr;
  {
    std::lock_guard<std::mutex> lk(m);
    auto it = plans.find(key.str());
    if (it != plans.end()) fn = it->second;
  }
  if (!fn) {
    fn = jit_get(tile_source(P, t, src.dtype, dest.dtype, nscal), "nca_stencil_tile");
    std::lock_guard<std::mutex> lk(m);
    if (plans.size() > 512) plans.clear();
    plans[key.str()] = fn;
  }
  std::vector<uint64_t> w((size_t)14 + (size_t)std::max(nscal, 1), 0);
  w[0] = (uint64_t)(uintptr_t)base; w[1] = (uint64_t)(uintptr_t)dbase;
  for (int a = 0; a < 3; ++a) {
    w[(size_t)2 + a] = (uint64_t)ss[a];
    w[(size_t)5 + a] = (uint64_t)dst[a];
    w[(size_t)8 + a] = (uint64_t)dsh[a];
    w[(size_t)11 + a] = (uint64_t)(sh[a] - mn[a]);
  }
  for (int k = 0; k < nscal; ++k)
    w[(size_t)14 + k] = jit_scalar_word(t.compute_dtype, t.scalar_dtypes[(size_t)k], t.scalar_slots[(size_t)k]);
  void* params[] = {w.data()};
  count_launch();
  check_cu(drv().cuLaunchKernel(fn, (unsigned)gx, (unsigned)gy, (unsigned)gz, 32u * (unsigned)P.by, 1, 1, 0,
                                (CUstream)stream, params, nullptr),
           "cuLaunchKernel(tiled stencil)");
  return true;
}

}  // namespace

// Compile-only check of tiled stencil plans for `arch`: the 7- and 27-point
// float32 Laplacians (the latter on column pairs), a float64 3x3x3 set, an
// int32 tape over asymmetric offsets, bfloat16 staged by plain loads, and a
// 2-D 5-point set.
int stencil_tile_selftest(const char* arch) {
  auto I = [](int op, int idx) { return (uint32_t)(op << 24) | (uint32_t)idx; };
  // sum of c * v_k over n operands, then + v_0
  auto lin = [&](int n, int w) {
    Tape t;
    for (int k = 0; k < n; ++k) {
      t.instrs.push_back(I(NCA_OP_LOAD_NCARR, k));
      t.instrs.push_back(I(NCA_OP_LOAD_CONST, 0));
      t.instrs.push_back(I(NCA_OP_MUL, 0));
      if (k) t.instrs.push_back(I(NCA_OP_ADD, 0));
    }
    t.instrs.push_back(I(NCA_OP_LOAD_NCARR, 0));
    t.instrs.push_back(I(NCA_OP_ADD, 0));
    t.scalar_dtypes = {w};
    t.scalar_slots = {0};
    t.compute_dtype = t.result_dtype = w;
    t.n_arrays = n;
    return t;
  };
  std::vector<int64_t> o7 = {1, 1, 1, 0, 1, 1, 2, 1, 1, 1, 0, 1, 1, 2, 1, 1, 1, 0, 1, 1, 2};
  std::vector<int64_t> o27;
  for (int z = 0; z < 3; ++z) for (int y = 0; y < 3; ++y) for (int x = 0; x < 3; ++x) o27.insert(o27.end(), {z, y, x});
  std::vector<int64_t> oa = {0, 0, 0, 1, 2, 3, 2, 0, 1, 0, 3, 2, 1, 1, 0};
  std::vector<int64_t> o2 = {1, 1, 0, 1, 2, 1, 1, 0, 1, 2};
  struct Case { const std::vector<int64_t>* off; int nd, src, dst, w; bool cpa; };
  const Case cases[] = {{&o7, 3, NCA_FLOAT32, NCA_FLOAT32, NCA_FLOAT32, true},
                        {&o27, 3, NCA_FLOAT32, NCA_FLOAT32, NCA_FLOAT32, true},
                        {&o27, 3, NCA_FLOAT64, NCA_FLOAT64, NCA_FLOAT64, true},
                        {&oa, 3, NCA_INT32, NCA_INT32, NCA_INT32, true},
                        {&o7, 3, NCA_BFLOAT16, NCA_BFLOAT16, NCA_FLOAT32, false},
                        {&o2, 2, NCA_FLOAT32, NCA_FLOAT32, NCA_FLOAT32, true}};
  int n = 0;
  for (const Case& c : cases) {
    const int nops = (int)c.off->size() / c.nd;
    Tape t = lin(nops, c.w);
    TilePlan P;
    int64_t mn[3];
    if (const char* why = plan_tile(c.off->data(), nops, c.nd, t, P, mn)) fail(NCA_ERR_INVALID, "selftest plan: %s", why);
    P.cpa = c.cpa;
    P.zc = 64;
    P.off32 = n % 2 == 0;
    if (n == 1) {   // the 27-point set on column pairs
      P.pk = true;
      P.vx = 2;
      plan_cells(P);
    }
    jit_compile_only(tile_source(P, t, c.src, c.dst, 1), arch);
    ++n;
  }
  return n;
}

// Builds the operand view of offset `o` (ndim values) of src for dest.
nca_view stencil_operand(const nca_view& src, const int64_t* step, const int64_t* o, const nca_view& dest) {
  nca_view v = src;
  const int pa = src.pointer_axis;
  const bool so = (src.flags & NCA_VIEW_SUBOFFSETS) != 0;
  char* data = static_cast<char*>(src.data);
  for (int d = 0; d < src.ndim; ++d) {
    v.shape[d] = dest.shape[d];
    if (d == pa) {
      // the pointer axis: strides the table before the read
      const int64_t tstride = so ? src.strides[d] : (int64_t)sizeof(void*);
      v.strides[d] = tstride * step[d];
      data += so ? o[d] * src.strides[d] : (src.offsets[d] + o[d]) * (int64_t)sizeof(void*);
      v.offsets[d] = so ? src.offsets[d] : 0;   // suboffset after the read
    } else {
      v.strides[d] = src.strides[d] * step[d];
      v.offsets[d] = src.offsets[d] + o[d] * src.strides[d];
    }
  }
  if (pa >= 0) v.flags = NCA_VIEW_SUBOFFSETS;
  v.data = data;
  return v;
}

}  // namespace nca

extern "C" int32_t nca_stencil(const nca_view* src, const nca_view* dest, const int64_t* offsets,
                               int32_t n_offsets, const nca_tape* tape, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!src || !dest || !tape) fail(NCA_ERR_INVALID, "null argument");
    if (n_offsets < 1 || !offsets) fail(NCA_ERR_INVALID, "a stencil needs at least one offset");
    if (n_offsets > NCA_MAX_OPERANDS)
      fail(NCA_ERR_LIMIT, "%d offsets: at most %d (one operand each)", n_offsets, NCA_MAX_OPERANDS);
    check_stencil_view(*src, "stencil source");
    check_stencil_view(*dest, "stencil destination");
    if (dest->ndim != src->ndim)
      fail(NCA_ERR_SHAPE, "source has %d dims, destination %d", src->ndim, dest->ndim);
    if (dest->pointer_axis >= 0) fail(NCA_ERR_UNSUPPORTED, "the destination cannot have a pointer axis");
    const int nd = src->ndim;
    int64_t step[NCA_MAX_NDIM];
    int64_t dn = 1;
    for (int d = 0; d < nd; ++d) {
      dn *= dest->shape[d];
      if (dest->shape[d] == 0) { step[d] = 1; continue; }
      step[d] = src->shape[d] / dest->shape[d];
      if (step[d] < 1)
        fail(NCA_ERR_SHAPE, "dim %d: destination extent %lld exceeds the source's %lld", d,
             (long long)dest->shape[d], (long long)src->shape[d]);
    }
    // every read src[c * step + o] must be inside src
    for (int i = 0; i < n_offsets; ++i) {
      const int64_t* o = offsets + (int64_t)i * nd;
      for (int d = 0; d < nd && dn > 0; ++d) {
        const int64_t last = (dest->shape[d] - 1) * step[d] + o[d];
        if (o[d] < 0 || last >= src->shape[d])
          fail(NCA_ERR_SHAPE, "offset %d leaves the source on dim %d (reads %lld..%lld of %lld)", i, d,
               (long long)o[d], (long long)last, (long long)src->shape[d]);
      }
    }
    Tape t = make_tape(tape, n_offsets);
    if (dn == 0) return;
    if (stencil_tile(*src, *dest, step, offsets, n_offsets, t, (cudaStream_t)stream)) return;
    std::vector<nca_view> ops((size_t)n_offsets);
    for (int i = 0; i < n_offsets; ++i) ops[(size_t)i] = stencil_operand(*src, step, offsets + (int64_t)i * nd, *dest);
    expr_eval(t, ops.data(), n_offsets, *dest, (cudaStream_t)stream);
  });
}
