#include "codegen.h"

#include <functional>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>

namespace symx {

std::string double_literal(double v)
{
    if (std::isnan(v)) return "symxg_nan()";
    if (std::isinf(v)) return v > 0 ? "symxg_inf()" : "(-symxg_inf())";
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.17g", v);
    std::string s(buf);
    if (s.find_first_of(".eE") == std::string::npos) s += ".0";
    return s;
}

std::string codegen_prelude()
{
    return R"(
// ---- generated-code prelude ----
__device__ __forceinline__ double symxg_inf() { return __longlong_as_double(0x7ff0000000000000LL); }
__device__ __forceinline__ double symxg_nan() { return __longlong_as_double(0x7ff8000000000000LL); }
// Natural/base-10 logarithm with the reference's guard: x <= 0 gives -inf
// (symx/src/compile/Compilation.cpp:426-428).
__device__ __forceinline__ double symxg_ln(double x) { return x > 0.0 ? log(x) : -symxg_inf(); }
__device__ __forceinline__ float symxg_ln(float x) { return x > 0.0f ? logf(x) : -__int_as_float(0x7f800000); }
__device__ __forceinline__ double symxg_log10(double x) { return x > 0.0 ? log10(x) : -symxg_inf(); }
__device__ __forceinline__ float symxg_log10(float x) { return x > 0.0f ? log10f(x) : -__int_as_float(0x7f800000); }
__device__ __forceinline__ double symxg_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float symxg_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double symxg_exp(double x) { return exp(x); }
__device__ __forceinline__ float symxg_exp(float x) { return expf(x); }
__device__ __forceinline__ double symxg_powf(double x, double p) { return pow(x, p); }
__device__ __forceinline__ float symxg_powf(float x, float p) { return powf(x, p); }
__device__ __forceinline__ double symxg_sin(double x) { return sin(x); }
__device__ __forceinline__ float symxg_sin(float x) { return sinf(x); }
__device__ __forceinline__ double symxg_cos(double x) { return cos(x); }
__device__ __forceinline__ float symxg_cos(float x) { return cosf(x); }
__device__ __forceinline__ double symxg_tan(double x) { return tan(x); }
__device__ __forceinline__ float symxg_tan(float x) { return tanf(x); }
__device__ __forceinline__ double symxg_asin(double x) { return asin(x); }
__device__ __forceinline__ float symxg_asin(float x) { return asinf(x); }
__device__ __forceinline__ double symxg_acos(double x) { return acos(x); }
__device__ __forceinline__ float symxg_acos(float x) { return acosf(x); }
__device__ __forceinline__ double symxg_atan(double x) { return atan(x); }
__device__ __forceinline__ float symxg_atan(float x) { return atanf(x); }
// ---- double-float: an unevaluated sum hi + lo of two floats (about 48 significant bits).
// Arithmetic runs on the FP32 pipe with error-free transformations (TwoSum; TwoProd through
// fmaf), Dekker / Knuth style; the __f*_rn intrinsics keep the compiler from contracting or
// reassociating them.  Transcendentals go through double.
struct symxg_df {
    float hi, lo;
    __device__ __forceinline__ symxg_df() : hi(0.0f), lo(0.0f) {}
    __device__ __forceinline__ symxg_df(float h, float l) : hi(h), lo(l) {}
    // nearest split of a double (folded at compile time for literals)
    __device__ __forceinline__ symxg_df(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    __device__ __forceinline__ void operator+=(const symxg_df& b);
    __device__ __forceinline__ void operator*=(const symxg_df& b);
};
__device__ __forceinline__ double symxg_to_double(const symxg_df& a) { return (double)a.hi + (double)a.lo; }
// hoisted values read where they are used: (hi, lo) pairs of the mixed path's cache
__device__ __forceinline__ symxg_df symxg_ldc_df(const float2* __restrict__ p, long long i)
{
    const float2 v = __ldg(p + i);
    return symxg_df(v.x, v.y);
}
__device__ __forceinline__ float symxg_ldc_f(const float2* __restrict__ p, long long i) { return __ldg(&p[i].x); }
__device__ __forceinline__ double symxg_ldc_d(const double* __restrict__ p, long long i) { return __ldg(p + i); }
__device__ __forceinline__ symxg_df symxg_df_fast(float a, float b)  // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return symxg_df(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ symxg_df operator+(const symxg_df& a, const symxg_df& b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return symxg_df_fast(s, e);
}
__device__ __forceinline__ symxg_df operator-(const symxg_df& a) { return symxg_df(-a.hi, -a.lo); }
__device__ __forceinline__ symxg_df operator-(const symxg_df& a, const symxg_df& b) { return a + (-b); }
__device__ __forceinline__ symxg_df operator*(const symxg_df& a, const symxg_df& b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return symxg_df_fast(p, e);
}
__device__ __forceinline__ symxg_df operator/(const symxg_df& a, const symxg_df& b)
{
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const symxg_df r = a - b * symxg_df(q1, 0.0f);
    const float q2 = __fdiv_rn(r.hi, b.hi);
    const symxg_df r2 = r - b * symxg_df(q2, 0.0f);
    const float q3 = __fdiv_rn(r2.hi, b.hi);
    return symxg_df_fast(q1, q2) + symxg_df(q3, 0.0f);
}
__device__ __forceinline__ bool operator>(const symxg_df& a, const symxg_df& b)
{
    return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}
__device__ __forceinline__ void symxg_df::operator+=(const symxg_df& b) { *this = *this + b; }
__device__ __forceinline__ void symxg_df::operator*=(const symxg_df& b) { *this = *this * b; }
__device__ __forceinline__ symxg_df symxg_sqrt(const symxg_df& a)
{
    if (!(a.hi > 0.0f)) return symxg_df(sqrtf(a.hi), 0.0f);
    const float s = sqrtf(a.hi);
    const symxg_df e = a - symxg_df(s, 0.0f) * symxg_df(s, 0.0f);  // one Newton step in double-float
    return symxg_df_fast(s, __fdiv_rn(e.hi, __fmul_rn(2.0f, s)));
}
__device__ __forceinline__ symxg_df symxg_ln(const symxg_df& a) { return symxg_df(symxg_ln(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_log10(const symxg_df& a) { return symxg_df(symxg_log10(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_exp(const symxg_df& a) { return symxg_df(exp(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_powf(const symxg_df& x, const symxg_df& p)
{
    return symxg_df(pow(symxg_to_double(x), symxg_to_double(p)));
}
__device__ __forceinline__ symxg_df symxg_sin(const symxg_df& a) { return symxg_df(sin(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_cos(const symxg_df& a) { return symxg_df(cos(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_tan(const symxg_df& a) { return symxg_df(tan(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_asin(const symxg_df& a) { return symxg_df(asin(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_acos(const symxg_df& a) { return symxg_df(acos(symxg_to_double(a))); }
__device__ __forceinline__ symxg_df symxg_atan(const symxg_df& a) { return symxg_df(atan(symxg_to_double(a))); }
// x^n for n >= 2 by binary powering.
template <typename T>
__device__ __forceinline__ T symxg_powi(T x, int n)
{
    T r = T(1.0), b = x;
    while (n > 0) { if (n & 1) r *= b; b *= b; n >>= 1; }
    return r;
}
)";
}

std::string emit_device_function(const Expressions& g, const std::vector<int32_t>& outputs, const std::string& name,
                                 const std::string& T, bool accumulate, OpCount* count,
                                 const std::unordered_map<int32_t, int32_t>* external, const std::string& sink_macro,
                                 const std::string& ext_load)
{
    std::function<void(int32_t)> emit_sink_;
    auto is_external = [&](int32_t i) { return external && external->count(i) > 0; };
    int32_t top = 0;
    for (int32_t o : outputs) top = std::max(top, o);
    std::vector<uint8_t> need(top + 1, 0);
    for (int32_t o : outputs) need[o] = 1;
    for (int32_t i = top; i >= 0; --i) {
        if (!need[i] || is_external(i)) continue;
        const Node& n = g[i];
        switch (n.op) {
            case Op::Zero: case Op::One: case Op::Const: case Op::Symbol: break;
            default:
                if (n.a >= 0) need[n.a] = 1;
                if (n.b >= 0 && n.op != Op::PowN) need[n.b] = 1;
                if (n.c >= 0) need[n.c] = 1;
        }
    }
    auto ref = [&](int32_t i) -> std::string {
        if (is_external(i)) {
            if (!ext_load.empty()) return ext_load + "(cq, " + std::to_string(external->at(i)) + "LL * cn)";
            return "c[" + std::to_string(external->at(i)) + "]";
        }
        const Node& n = g[i];
        switch (n.op) {
            case Op::Zero: return "(" + T + ")0";
            case Op::One: return "(" + T + ")1";
            case Op::Const: return "((" + T + ")" + double_literal(n.v) + ")";
            case Op::Symbol: return "in[" + std::to_string((int32_t)n.v) + "]";
            default: return "t" + std::to_string(i);
        }
    };
    OpCount oc;
    std::ostringstream s;
    const bool sink = !sink_macro.empty();
    // the cache holds doubles for double functions, (hi, lo) float pairs otherwise
    const std::string cparam = ext_load.empty() ? "const " + T + "* __restrict__ c"
                               : T == "double"  ? "const double* __restrict__ cq, long long cn"
                                                : "const float2* __restrict__ cq, long long cn";
    if (sink)
        s << "__device__ __forceinline__ void " << name << "(const " << T << "* __restrict__ in, " << cparam << ", "
          << T << "* __restrict__ out, int lq, bool st)\n{\n";
    else
        s << "__device__ __forceinline__ void " << name << "(const " << T << "* __restrict__ in, " << cparam << ", "
          << T << "* __restrict__ out)\n{\n";
    // sink mode: every output goes to sink_macro(value, slot, lq, st, out) as soon as its node
    // is computed, so no output has to stay live to the end
    std::vector<std::vector<size_t>> slots_of;
    if (sink) {
        slots_of.resize(top + 1);
        for (size_t k = 0; k < outputs.size(); ++k) slots_of[outputs[k]].push_back(k);
        auto emit_sink = [&](int32_t i) {
            s << "    { const " << T << " r_ = " << sink_macro << "_SUM(" << ref(i) << ");";
            for (size_t k : slots_of[i]) s << " " << sink_macro << "_STORE(r_, " << k << ");";
            s << " }\n";
        };
        for (int32_t i = 0; i <= top; ++i) {
            if (slots_of[i].empty()) continue;
            const Node& n = g[i];
            const bool leaf = is_external(i) || n.op == Op::Zero || n.op == Op::One || n.op == Op::Const ||
                              n.op == Op::Symbol;
            if (leaf) emit_sink(i);
        }
        emit_sink_ = emit_sink;
    }
    for (int32_t i = 0; i <= top; ++i) {
        if (!need[i] || is_external(i)) continue;
        const Node& n = g[i];
        std::string e;
        switch (n.op) {
            case Op::Zero: case Op::One: case Op::Const: case Op::Symbol: continue;
            case Op::Add: e = ref(n.a) + " + " + ref(n.b); ++oc.add; break;
            case Op::Sub: e = ref(n.a) + " - " + ref(n.b); ++oc.sub; break;
            case Op::Mul: e = ref(n.a) + " * " + ref(n.b); ++oc.mul; break;
            case Op::Div: e = ref(n.a) + " / " + ref(n.b); ++oc.div; break;
            case Op::Neg: e = "-" + ref(n.a); ++oc.neg; break;
            case Op::PowN:
                if (n.b == 2) { e = ref(n.a) + " * " + ref(n.a); ++oc.mul; }
                else if (n.b == 3) { e = ref(n.a) + " * " + ref(n.a) + " * " + ref(n.a); oc.mul += 2; }
                else { e = "symxg_powi<" + T + ">(" + ref(n.a) + ", " + std::to_string(n.b) + ")"; ++oc.pow; }
                break;
            case Op::PowF: e = "symxg_powf(" + ref(n.a) + ", (" + T + ")" + double_literal(n.v) + ")"; ++oc.pow; break;
            case Op::Sqrt: e = "symxg_sqrt(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Ln: e = "symxg_ln(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Log10: e = "symxg_log10(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Exp: e = "symxg_exp(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Sin: e = "symxg_sin(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Cos: e = "symxg_cos(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Tan: e = "symxg_tan(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Asin: e = "symxg_asin(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Acos: e = "symxg_acos(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Atan: e = "symxg_atan(" + ref(n.a) + ")"; ++oc.transcendental; break;
            case Op::Branch:
                e = "(" + ref(n.c) + " > (" + T + ")0) ? " + ref(n.a) + " : " + ref(n.b);
                ++oc.branch;
                break;
        }
        s << "    const " << T << " t" << i << " = " << e << ";\n";
        if (sink && !slots_of[i].empty()) emit_sink_(i);
    }
    if (!sink)
        for (size_t k = 0; k < outputs.size(); ++k)
            s << "    out[" << k << "] " << (accumulate ? "+=" : "=") << " " << ref(outputs[k]) << ";\n";
    s << "}\n";
    if (count) *count = oc;
    return s.str();
}

}  // namespace symx
