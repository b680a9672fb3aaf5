// Compiled by tests/test_dropin_cpu.py with nvcc against ncarray's own headers,
// with include/ncarray_dropin ahead of them on the include path and linked
// against libncgb300: proves that ncarray's C++ API (ArrayImpl operators,
// reductions, copies, fills, Stencil<NDIM>) builds on the GB300 engine without
// a change to ncarray's sources. Run without a GPU, main() only converts
// expressions and stencils that ncarray's own code builds into the C-ABI
// descriptors (nca_tape, nca_view) and prints them as JSON; the GPU test
// replays those descriptors through the C ABI (tests/test_dropin_gpu.py).
#include "ncarray/array_impl.hh"
#include "ncarray/array_operations.hh"
#include "ncarray/expression/stencil.hh"

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

using namespace ncarray;
using DevView = NCViewFor<DevTag>;
using DevArray = NCOwnerFor<DevTag>;

static_assert(GPUEngine::is_gb300_engine, "ncarray picked up its own GPUEngine, not the drop-in");

// Every engine path ncarray's device API takes, instantiated and linked
// (never run here).
void api_paths(DevArray& a, DevArray& b, float* host) {
  DevArray c(a.ndim(), a.shape(), a.dtype());
  c = a * b + a - 2.0f;                        // execute_binary_expression
  Scalar s = a.sum();                           // execute_full_reduce
  s = a.mean(); s = a.max(); s = a.min(); s = a.argmax(); s = a.argmin();
  DevArray r = a.sum(std::vector<ssize_t>{0});  // execute_reduce_axes
  r = a.max(std::vector<ssize_t>{0}); r = a.argmin(std::vector<ssize_t>{0}); r = a.mean(std::vector<ssize_t>{0});
  a.fill(Scalar(1.5f));                         // execute_fill
  a.copy_into_astype<float>(host);              // execute_copy_into
  b.view().assign(a.view());                    // execute_assign
  auto st = Stencil<2>::create<float>({{0, 0}, {1, 1}}, {0, 0},
                                      [](auto v) { return ExprMVNode<DevTag>(v[0]) + v[1] * 0.5f; });
  DevArray d(a.ndim(), a.shape(), a.dtype());
  st.apply(a.view(), d);
}
void (*volatile keep_api_paths)(DevArray&, DevArray&, float*) = &api_paths;

static std::string view_json(const nca_view& v, uintptr_t base) {
  std::string s = "{\"buffer\": " + std::to_string((uintptr_t)v.data >= base ? ((uintptr_t)v.data - base) >> 32 : 0) +
                  ", \"byte_offset\": " + std::to_string((uintptr_t)v.data & 0xffffffffu) +
                  ", \"dtype\": " + std::to_string(v.dtype) + ", \"pointer_axis\": " + std::to_string(v.pointer_axis) +
                  ", \"flags\": " + std::to_string(v.flags);
  const char* names[3] = {"shape", "strides", "offsets"};
  const int64_t* arrs[3] = {v.shape, v.strides, v.offsets};
  for (int k = 0; k < 3; ++k) {
    s += std::string(", \"") + names[k] + "\": [";
    for (int d = 0; d < v.ndim; ++d) s += (d ? ", " : "") + std::to_string(arrs[k][d]);
    s += "]";
  }
  return s + "}";
}

static std::string tape_json(const gb300::TapeHolder& t) {
  std::string s = "{\"instrs\": [";
  for (size_t i = 0; i < t.instrs.size(); ++i) s += (i ? ", " : "") + std::to_string(t.instrs[i]);
  s += "], \"scalars\": [";
  for (size_t i = 0; i < t.scalar_slots.size(); ++i)
    s += (i ? ", " : "") + std::string("[") + std::to_string(t.scalar_dtypes[i]) + ", " +
         std::to_string(t.scalar_slots[i]) + "]";
  return s + "], \"compute\": " + std::to_string(t.tape.compute_dtype) + ", \"result\": " +
         std::to_string(t.tape.result_dtype) + "}";
}

// buffer k lives at base + k * 2^32 (fake addresses: nothing is dereferenced)
static const uintptr_t kBase = (uintptr_t)1 << 40;
static void* buf(int k, uintptr_t byte_offset = 0) { return (void*)(kBase + ((uintptr_t)k << 32) + byte_offset); }

template <class Expr>
static std::string expr_case(const char* name, const Expr& e, const std::vector<ssize_t>& out_shape) {
  gb300::TapeHolder t = gb300::to_tape(e);
  std::vector<nca_view> ops = gb300::operand_views(e);
  std::string s = std::string("{\"kind\": \"expr\", \"name\": \"") + name + "\", \"tape\": " + tape_json(t) +
                  ", \"operands\": [";
  for (size_t i = 0; i < ops.size(); ++i) s += (i ? ", " : "") + view_json(ops[i], kBase);
  s += "], \"out_shape\": [";
  for (size_t d = 0; d < out_shape.size(); ++d) s += (d ? ", " : "") + std::to_string(out_shape[d]);
  return s + "]}";
}

int main() {
  std::vector<std::string> cases;
  {  // C1 without the opcodes ncarray lacks: a*b + c - a*0.5 on float64 (6, 8, 10)
    ssize_t sh[3] = {6, 8, 10}, st[3] = {640, 80, 8};
    DevView a(buf(0), 3, sh, st, DType::float64, -1, false), b(buf(1), 3, sh, st, DType::float64, -1, false),
        c(buf(2), 3, sh, st, DType::float64, -1, false);
    ExprMVNode<DevTag> e = a * b + c - a * 0.5;
    cases.push_back(expr_case("c1_core", e, {6, 8, 10}));
  }
  {  // C2: x (4, 16, 8, 8) float32 viewed (3, 1, 2, 0), times v broadcast on axis 1, plus int32 k
    ssize_t sh[4] = {8, 16, 8, 4}, xst[4] = {4, 256, 32, 4096}, vst[4] = {0, 4, 0, 0};
    ssize_t kst[4] = {2048, 128, 16, 4};
    DevView x(buf(0), 4, sh, xst, DType::float32, -1, false), v(buf(1), 4, sh, vst, DType::float32, -1, false),
        k(buf(2), 4, sh, kst, DType::int32, -1, false);
    ExprMVNode<DevTag> y = x * v + k;
    cases.push_back(expr_case("c2_y", y, {8, 16, 8, 4}));
    ExprMVNode<DevTag> z = (k * 3 + 7) % 11;
    cases.push_back(expr_case("c2_int", z, {8, 16, 8, 4}));
  }
  {  // a pointer axis: 5 panels of (12, 20) float32 behind a table, panel offset of one row
    Metadata shape, strides, offsets;
    ssize_t sh[3] = {5, 12, 20}, st[3] = {8, 80, 4}, of[3] = {1, 80, 0};
    shape.set(sh, 3); strides.set(st, 3); offsets.set(of, 3);
    DevView p(buf(0), shape, strides, offsets, DType::float32, 0, false);
    ssize_t sh2[3] = {4, 11, 20}, st2[3] = {880, 80, 4};
    DevView q(buf(1), 3, sh2, st2, DType::float32, -1, false);
    ssize_t vsh[3] = {4, 11, 20};
    Metadata vshape;
    vshape.set(vsh, 3);
    DevView pv(buf(0), vshape, strides, offsets, DType::float32, 0, false);
    ExprMVNode<DevTag> e = pv * 2.0f - q;
    cases.push_back(expr_case("panels", e, {4, 11, 20}));
  }
  {  // the reference benchmark's binning stencil (examples/benchmark_binning.cu:343-377)
    std::vector<StaticCoords<3>> offs;
    for (ssize_t p = 0; p < 2; ++p)
      for (ssize_t r = 0; r < 2; ++r)
        for (ssize_t c = 0; c < 2; ++c) offs.push_back({p, r, c});
    auto binning = [](auto views) {
      ExprMVNode<DevTag> e(views[0]);
      for (std::size_t i = 1; i < views.size(); ++i) e = e + views[i];
      return e * 0.125f;
    };
    auto st = Stencil<3>::create<float>(offs, {0, 0, 0}, binning);
    std::string s = "{\"kind\": \"stencil\", \"name\": \"binning_2x2x2\", \"tape\": " + tape_json(st.tape()) +
                    ", \"offsets\": [";
    for (size_t i = 0; i < st.flat_offsets().size(); ++i) s += (i ? ", " : "") + std::to_string(st.flat_offsets()[i]);
    cases.push_back(s + "], \"ndim\": 3}");
  }
  {  // reduction axes: ReductionParams from ncarray's build_reduction_params -> axes mask
    ssize_t sh[4] = {3, 4, 5, 6}, st[4] = {480, 120, 24, 4};
    std::string s = "{\"kind\": \"axes\", \"masks\": [";
    std::vector<std::vector<ssize_t>> sets = {{0}, {2}, {1, 3}, {0, 1, 2, 3}, {3}};
    for (size_t i = 0; i < sets.size(); ++i) {
      ssize_t new_shape[NCARRAY_MAX_NDIM];
      ssize_t new_ndim = 0;
      ReductionParams p = build_reduction_params(sets[i], 4, sh, st, new_shape, new_ndim, 4);
      s += (i ? ", " : "") + std::to_string(gb300::axes_mask(p));
    }
    cases.push_back(s + "]}");
  }
  std::printf("[\n");
  for (size_t i = 0; i < cases.size(); ++i) std::printf("%s%s\n", cases[i].c_str(), i + 1 < cases.size() ? "," : "");
  std::printf("]\n");
  return 0;
}
