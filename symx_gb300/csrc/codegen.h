// CUDA code generation from the expression DAG.
//
// The reference emits straight-line C++ for `void f(T* in, T* out)` and compiles it
// with the system compiler (symx/src/compile/Compilation.cpp:243-469).  Here the
// same DAG becomes a `__device__` function with the same slot contract
// (in[i] = symbol i, out[k] = k-th requested expression), written for CUDA and
// compiled at run time by NVRTC (cuda_module.h).
#pragma once

#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "symbolic.h"

namespace symx {

struct OpCount {
    int64_t add = 0, sub = 0, mul = 0, div = 0, neg = 0, transcendental = 0, branch = 0, pow = 0;
    int64_t total() const { return add + sub + mul + div + neg + transcendental + branch + pow; }
};

// Emit `__device__ __forceinline__ void <name>(const T* __restrict__ in, const T* __restrict__ c,
// T* __restrict__ out)` computing every expression of `outputs` (node ids) in type `T`
// ("double" or "float").  Nodes listed in `external` are not computed: they are read as
// c[slot] (values hoisted out of the kernel).  If `accumulate` is set, outputs are added to
// `out` instead of assigned (summations).
// With sink_macro = "M": the function takes (in, c, out, int lq, bool st) and passes each
// output, as soon as its node is computed, through M_SUM(value) (e.g. a sum over the lanes
// that evaluate the element's quadrature points) and M_STORE(result, slot) (macros the
// caller defines; they see lq, st and out); nothing is written to out otherwise.
// With ext_load = "f": the external values are not passed as an array c but read where they
// are used, as f(cq, k * cn) from a float2 pointer cq with stride cn (the parameters that
// replace c), so no per-thread copy of them is made.
std::string emit_device_function(const Expressions& g, const std::vector<int32_t>& outputs, const std::string& name,
                                 const std::string& T, bool accumulate, OpCount* count = nullptr,
                                 const std::unordered_map<int32_t, int32_t>* external = nullptr,
                                 const std::string& sink_macro = "", const std::string& ext_load = "");

// Prelude shared by all generated sources: guarded log, integer powers, infinities.
std::string codegen_prelude();

// Literal for a double constant in generated code, exact to the last bit.
std::string double_literal(double v);

}  // namespace symx
