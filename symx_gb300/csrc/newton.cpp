// Projected Newton's method on one GPU.  See newton.h.
//
// Reference control flow followed here: symx/src/solver/NewtonsMethod.cpp
//   solve loop :28-252, projection + assembly :254-352, BDPCG with forcing term :388-452,
//   line search (cap, max step, Armijo) :459-641.
#include "newton.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <map>
#include <unordered_map>

#include <cuda_runtime.h>

#include "codegen.h"
#include "cuda_module.h"
#include "kernels.cuh"

namespace symx {

using symxg::CudaModule;
using symxg::PcgBuffers;
using symxg::PcgState;

namespace {

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("symx_gb300: ") + what + ": " + cudaGetErrorString(e));
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    ~DevBuf() { release(); }
    void alloc(size_t count)
    {
        if (count == n && p) return;
        release();
        if (count) {
            ck(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
            symxg::note_device_alloc((int64_t)(count * sizeof(T)));
        }
        n = count;
    }
    void release()
    {
        if (p) {
            cudaFree(p);
            symxg::note_device_free((int64_t)(n * sizeof(T)));
        }
        p = nullptr;
        n = 0;
    }
};

struct StageTimer {
    struct Rec { std::string label; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    cudaStream_t s = nullptr;
    std::string open_label;
    cudaEvent_t open_a = nullptr;
    void start(const std::string& label)
    {
        cudaEvent_t a;
        cudaEventCreate(&a);
        cudaEventRecord(a, s);
        open_label = label;
        open_a = a;
    }
    void stop()
    {
        cudaEvent_t b;
        cudaEventCreate(&b);
        cudaEventRecord(b, s);
        recs.push_back({open_label, open_a, b});
        open_a = nullptr;
    }
    void flush(std::map<std::string, double>& out)
    {
        for (auto& r : recs) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, r.a, r.b);
            out[r.label] += ms * 1e-3;
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        recs.clear();
    }
};

struct UploadedArray {
    std::uintptr_t id = 0;
    const double* host = nullptr;
    int64_t n = 0;
    DevBuf<double> dev;
};

struct CompiledPotential {
    std::string name;
    const Potential* pot = nullptr;
    int nb = 0;                    // DoF blocks per element
    std::vector<int> dof_set;      // per block: DoF set index
    std::vector<int> dof_col;      // per block: connectivity column
    std::vector<int> map_upload;   // per map: index into uploaded arrays, or -1-dofset for DoF maps
    int64_t n_elements = 0;
    int conn_stride = 0;
    std::shared_ptr<CudaModule> module;
    std::string source;
    OpCount ops_eg, ops_h, ops_e;
    DevBuf<int32_t> conn;
    DevBuf<const double*> map_ptrs;
    int n_cache = 0, n_qp = 1;      // hoisted values per element and quadrature point
    int qp_lanes = 1;               // lanes per element of the mixed E+g+H kernel (one per quadrature point)
    bool cache_df = false;          // the cache holds (hi, lo) float pairs (mixed-precision kernels)
    DevBuf<double> cache;
    int64_t e_off = 0, g_off = 0, h_off = 0;  // offsets: elements, gradient blocks, Hessian blocks
};

// Generated source of one potential.  Besides the element kernels it contains a precompute
// kernel: every subexpression that does not depend on a DoF (rest shape, material, the
// quadrature point) and feeds a DoF-dependent one is evaluated once per upload into a
// per-element cache (`n_cache` doubles per element and quadrature point, stored value-major
// so that a warp's loads are coalesced), and the element kernels read it instead of
// recomputing it at every Newton and line-search evaluation.
std::string build_source(CompiledPotential& cp, const Expressions& g, const std::vector<int32_t>& eg,
                         const std::vector<int32_t>& h_bm, const std::vector<int32_t>& e_only, int32_t cond,
                         const Summation& sum, const std::vector<uint8_t>& is_dof_symbol, OpCount* oeg, OpCount* oh,
                         OpCount* oe)
{
    const MappedWorkspace<double>& mws = *cp.pot->mws;
    const int NS = g.n_symbols();
    const int NG = (int)eg.size() - 1;
    const int NH = (int)h_bm.size();
    const int NQ = std::max(1, sum.n_iterations);
    const bool acc = sum.n_iterations > 1;

    // ---- hoisting plan
    std::vector<int32_t> roots(eg);
    roots.insert(roots.end(), h_bm.begin(), h_bm.end());
    roots.insert(roots.end(), e_only.begin(), e_only.end());
    if (cond >= 0) roots.push_back(cond);
    int32_t top = 0;
    for (int32_t r : roots) top = std::max(top, r);
    auto is_leaf = [&](int32_t i) {
        const Op o = g[i].op;
        return o == Op::Zero || o == Op::One || o == Op::Const || o == Op::Symbol;
    };
    std::vector<uint8_t> variant(top + 1, 0);
    for (int32_t i = 0; i <= top; ++i) {
        const Node& n = g[i];
        if (n.op == Op::Symbol) variant[i] = is_dof_symbol[(int32_t)n.v];
        else if (!is_leaf(i))
            variant[i] = (n.a >= 0 && variant[n.a]) || (n.b >= 0 && n.op != Op::PowN && variant[n.b]) ||
                         (n.c >= 0 && variant[n.c]);
    }
    // Every invariant node that feeds a DoF-dependent node (or an output) gets a cache slot: the
    // topmost invariant subexpressions, so each cached value saves as many operations as
    // possible.
    std::vector<uint8_t> seen(top + 1, 0), main_symbol(NS, 0), pre_symbol(NS, 0);
    std::vector<int32_t> frontier, stack(roots.begin(), roots.end());
    while (!stack.empty()) {
        const int32_t i = stack.back();
        stack.pop_back();
        if (seen[i]) continue;
        seen[i] = 1;
        const Node& n = g[i];
        if (n.op == Op::Symbol) { main_symbol[(int32_t)n.v] = 1; continue; }
        if (is_leaf(i)) continue;
        if (!variant[i]) { frontier.push_back(i); continue; }
        if (n.a >= 0) stack.push_back(n.a);
        if (n.b >= 0 && n.op != Op::PowN) stack.push_back(n.b);
        if (n.c >= 0) stack.push_back(n.c);
    }
    std::sort(frontier.begin(), frontier.end());
    std::unordered_map<int32_t, int32_t> ext;
    for (size_t k = 0; k < frontier.size(); ++k) ext[frontier[k]] = (int32_t)k;
    const int K = (int)frontier.size();
    cp.n_cache = K;
    cp.n_qp = NQ;
    // symbols the precompute kernel reads
    {
        std::vector<uint8_t> need(top + 1, 0);
        for (int32_t f : frontier) need[f] = 1;
        for (int32_t i = top; i >= 0; --i) {
            if (!need[i]) continue;
            const Node& n = g[i];
            if (n.op == Op::Symbol) { pre_symbol[(int32_t)n.v] = 1; continue; }
            if (is_leaf(i)) continue;
            if (n.a >= 0) need[n.a] = 1;
            if (n.b >= 0 && n.op != Op::PowN) need[n.b] = 1;
            if (n.c >= 0) need[n.c] = 1;
        }
    }
    auto map_used = [&](const DataMap& m, const std::vector<uint8_t>& used) {
        for (int j = 0; j < m.stride; ++j)
            if (used[m.first_symbol + j]) return true;
        return false;
    };
    auto sum_used = [&](const std::vector<uint8_t>& used) {
        for (int j = 0; j < sum.stride; ++j)
            if (used[sum.first_symbol + j]) return true;
        return false;
    };

    std::ostringstream s;
    s << "// generated element kernels for potential '" << cp.name << "'\n";
    s << "// " << K << " hoisted values per element and quadrature point\n";
    s << codegen_prelude();
    s << emit_device_function(g, eg, "symxg_eval_eg", "double", acc, oeg, &ext);
    s << emit_device_function(g, h_bm, "symxg_eval_h_f64", "double", acc, oh, &ext);
    s << emit_device_function(g, h_bm, "symxg_eval_h_f32", "float", acc, nullptr, &ext);
    // Elements with several quadrature points and no activity condition: the mixed E+g+H kernel
    // gives each point its own lane (NQ lanes per element); every Hessian entry is summed over
    // the lanes by a butterfly of shuffles as soon as it is computed and stored by one lane, so
    // no NH-long accumulator array (local memory) is needed.
    const bool qp_parallel = acc && cond < 0 && NQ <= 32 && (NQ & (NQ - 1)) == 0;
    cp.qp_lanes = qp_parallel ? NQ : 1;
    if (qp_parallel) {
        s << "#define SYMXG_NQ " << NQ << "\n"
          << "__device__ __forceinline__ float symxg_qsum(float v)\n{\n"
          << "#pragma unroll\n    for (int o = 1; o < SYMXG_NQ; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);\n"
          << "    return v;\n}\n"
          << "__device__ __forceinline__ symxg_df symxg_qsum(symxg_df v)\n{\n"
          << "#pragma unroll\n    for (int o = 1; o < SYMXG_NQ; o <<= 1)\n"
          << "        v = v + symxg_df(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));\n"
          << "    return v;\n}\n"
          << "__device__ __forceinline__ double symxg_qsum(double v)\n{\n"
          << "#pragma unroll\n    for (int o = 1; o < SYMXG_NQ; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);\n"
          << "    return v;\n}\n"
          << "#define SYMXG_Q_SUM(v) symxg_qsum(v)\n"
          << "#define SYMXG_Q_STORE(r, k) do { if (st && lq == (k) % SYMXG_NQ) out[(k)] = (r); } while (0)\n";
        s << emit_device_function(g, h_bm, "symxg_eval_h_f32_q", "float", false, nullptr, &ext, "SYMXG_Q", "symxg_ldc_f");
        // the FP64 form of the same
        s << emit_device_function(g, eg, "symxg_eval_eg_dl", "double", acc, nullptr, &ext, "", "symxg_ldc_d");
        s << emit_device_function(g, h_bm, "symxg_eval_h_f64_q", "double", false, nullptr, &ext, "SYMXG_Q", "symxg_ldc_d");
    }
    s << emit_device_function(g, e_only, "symxg_eval_e", "double", acc, oe, &ext);
    if (cond >= 0) s << emit_device_function(g, {cond}, "symxg_eval_cond", "double", false, nullptr, &ext);
    // mixed precision: energy and gradient in double-float (FP32 pipe), see the prelude
    s << emit_device_function(g, eg, "symxg_eval_eg_df", "symxg_df", acc, nullptr, &ext);
    s << emit_device_function(g, e_only, "symxg_eval_e_df", "symxg_df", acc, nullptr, &ext);
    // the same reading the hoisted values from the cache where they are used (no per-thread copy)
    s << emit_device_function(g, eg, "symxg_eval_eg_dfl", "symxg_df", acc, nullptr, &ext, "", "symxg_ldc_df");
    s << emit_device_function(g, e_only, "symxg_eval_e_dfl", "symxg_df", acc, nullptr, &ext, "", "symxg_ldc_df");
    s << emit_device_function(g, h_bm, "symxg_eval_h_f32l", "float", acc, nullptr, &ext, "", "symxg_ldc_f");
    if (cond >= 0) s << emit_device_function(g, {cond}, "symxg_eval_cond_df", "symxg_df", false, nullptr, &ext);
    if (K > 0) s << emit_device_function(g, frontier, "symxg_eval_pre", "double", false, nullptr, nullptr);
    if (sum.n_iterations > 0) {
        s << "static __device__ const double symxg_sum_data[" << sum.data.size() << "] = {";
        for (size_t i = 0; i < sum.data.size(); ++i) s << (i ? ", " : "") << double_literal(sum.data[i]);
        s << "};\n";
    }
    // gathers of the bound data for element e: all maps a kernel family reads
    auto gather = [&](const std::string& fname, const std::vector<uint8_t>& used) {
        s << "__device__ __forceinline__ void " << fname
          << "(long long e, const int* __restrict__ conn, const double* const* __restrict__ maps, double* in)\n{\n";
        s << "    const int* __restrict__ ce = conn + e * " << cp.conn_stride << "LL;\n    (void)ce;\n";
        for (size_t k = 0; k < mws.maps.size(); ++k) {
            const DataMap& m = mws.maps[k];
            if (!map_used(m, used)) continue;
            s << "    { const double* __restrict__ m = maps[" << k << "]";
            if (m.conn_column >= 0) s << " + (long long)ce[" << m.conn_column << "] * " << m.stride << "LL";
            s << ";";
            for (int j = 0; j < m.stride; ++j) s << " in[" << (m.first_symbol + j) << "] = m[" << j << "];";
            s << " }\n";
        }
        s << "}\n";
    };
    gather("symxg_gather", main_symbol);
    gather("symxg_gather_pre", pre_symbol);
    auto set_sum = [&](const std::string& q, const std::vector<uint8_t>& used) {
        std::ostringstream t;
        if (sum.n_iterations == 0 || !sum_used(used)) return t.str();
        for (int j = 0; j < sum.stride; ++j)
            t << "        in[" << (sum.first_symbol + j) << "] = symxg_sum_data[" << q << " * " << sum.stride << " + " << j
              << "];\n";
        return t.str();
    };
    auto load_cache = [&](const std::string& q, const std::string& T) {
        std::ostringstream t;
        t << "        " << T << " c[" << std::max(1, K) << "];\n";
        if (K > 0)
            t << "        for (int k = 0; k < " << K << "; ++k) c[k] = (" << T << ")cache[((long long)" << q << " * " << K
              << "LL + k) * n + e];\n";
        else
            t << "        c[0] = (" << T << ")0;\n";
        return t.str();
    };
    auto cond_check = [&](const std::string& zero_writes) {
        if (cond < 0) return std::string();
        std::ostringstream t;
        t << "    {\n" << set_sum("0", main_symbol) << load_cache("0", "double")
          << "        double cv[1]; symxg_eval_cond(in, c, cv);\n        if (!(cv[0] > 0.0)) {\n"
          << zero_writes << "            return;\n        }\n    }\n";
        return t.str();
    };
    const std::string sig_common =
        "(long long n, const int* __restrict__ conn, const double* const* __restrict__ maps, "
        "const double* __restrict__ cache, double* __restrict__ E";

    // precompute kernel
    s << "extern \"C\" __global__ void __launch_bounds__(128) symxg_pre(long long n, const int* __restrict__ conn, "
         "const double* const* __restrict__ maps, double* __restrict__ cache)\n{\n";
    s << "    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n    if (e >= n) return;\n";
    if (K > 0) {
        s << "    double in[" << NS << "];\n    symxg_gather_pre(e, conn, maps, in);\n";
        s << "    for (int q = 0; q < " << NQ << "; ++q) {\n" << set_sum("q", pre_symbol);
        s << "        double c[" << K << "];\n        symxg_eval_pre(in, nullptr, c);\n";
        s << "        for (int k = 0; k < " << K << "; ++k) cache[((long long)q * " << K << "LL + k) * n + e] = c[k];\n    }\n";
    }
    s << "}\n";

    // E + g + H kernels, H in double or float (FP64 with several quadrature points: one lane
    // per point, as the mixed kernel below)
    if (qp_parallel) {
        s << "extern \"C\" __global__ void __launch_bounds__(128) symxg_egh_f64" << sig_common
          << ", double* __restrict__ G, double* __restrict__ H)\n{\n";
        s << "    if (n <= 0) return;\n";
        s << "    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n";
        s << "    const int lq = (int)(t % SYMXG_NQ);\n    const bool st = t / SYMXG_NQ < n;\n";
        s << "    const long long e = st ? t / SYMXG_NQ : n - 1;\n";
        s << "    double in[" << NS << "];\n    symxg_gather(e, conn, maps, in);\n";
        s << "    {\n" << set_sum("lq", main_symbol);
        s << "        const double* __restrict__ cq = cache + (long long)lq * " << K << "LL * n + e;\n";
        s << "        double eg[" << (NG + 1) << "];\n";
        s << "        for (int i = 0; i < " << NG + 1 << "; ++i) eg[i] = 0.0;\n";
        s << "        symxg_eval_eg_dl(in, cq, n, eg);\n";
        s << "#pragma unroll\n        for (int i = 0; i < " << NG + 1 << "; ++i) eg[i] = symxg_qsum(eg[i]);\n";
        s << "        if (st && lq == 0) E[e] = eg[0];\n";
        s << "#pragma unroll\n        for (int i = 0; i < " << NG << "; ++i)\n"
          << "            if (st && lq == i % SYMXG_NQ) G[e * " << NG << "LL + i] = eg[1 + i];\n";
        s << "        symxg_eval_h_f64_q(in, cq, n, H + e * " << NH << "LL, lq, st);\n    }\n}\n";
    }
    for (int prec = 0; prec < 2; ++prec) {
        if (prec == 0 && qp_parallel) continue;
        const std::string TH = prec == 0 ? "double" : "float";
        const std::string kname = prec == 0 ? "symxg_egh_f64" : "symxg_egh_f32";
        s << "extern \"C\" __global__ void __launch_bounds__(128) " << kname << sig_common
          << ", double* __restrict__ G, " << TH << "* __restrict__ H)\n{\n";
        s << "    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n    if (e >= n) return;\n";
        s << "    double in[" << NS << "];\n    symxg_gather(e, conn, maps, in);\n";
        std::ostringstream zw;
        zw << "            E[e] = 0.0;\n            for (int i = 0; i < " << NG << "; ++i) G[e * " << NG
           << "LL + i] = 0.0;\n"
           << "            for (int i = 0; i < " << NH << "; ++i) H[e * " << NH << "LL + i] = (" << TH << ")0;\n";
        s << cond_check(zw.str());
        s << "    double eg[" << (NG + 1) << "];\n    " << TH << " h[" << NH << "];\n";
        if (acc) {
            s << "    for (int i = 0; i < " << NG + 1 << "; ++i) eg[i] = 0.0;\n";
            s << "    for (int i = 0; i < " << NH << "; ++i) h[i] = (" << TH << ")0;\n";
            s << "    for (int q = 0; q < " << NQ << "; ++q) {\n";
        } else {
            s << "    { const int q = 0; (void)q;\n";
        }
        s << set_sum("q", main_symbol) << load_cache("q", "double");
        s << "        symxg_eval_eg(in, c, eg);\n";
        if (prec == 0) {
            s << "        symxg_eval_h_f64(in, c, h);\n";
        } else {
            s << "        float in32[" << NS << "], c32[" << std::max(1, K) << "];\n";
            s << "        for (int i = 0; i < " << NS << "; ++i) in32[i] = (float)in[i];\n";
            s << "        for (int i = 0; i < " << std::max(1, K) << "; ++i) c32[i] = (float)c[i];\n";
            s << "        symxg_eval_h_f32(in32, c32, h);\n";
        }
        s << "    }\n";
        s << "    E[e] = eg[0];\n";
        // 16-byte stores where the rows allow it (one element's outputs are contiguous)
        if (NG % 2 == 0)
            s << "    if ((reinterpret_cast<unsigned long long>(G) & 15ull) == 0ull) {\n"
              << "        double2* G2 = reinterpret_cast<double2*>(G + e * " << NG << "LL);\n"
              << "        for (int i = 0; i < " << NG / 2 << "; ++i) G2[i] = make_double2(eg[1 + 2 * i], eg[2 + 2 * i]);\n"
              << "    } else\n";
        s << "    for (int i = 0; i < " << NG << "; ++i) G[e * " << NG << "LL + i] = eg[1 + i];\n";
        if (prec == 0 && NH % 2 == 0)
            s << "    if ((reinterpret_cast<unsigned long long>(H) & 15ull) == 0ull) {\n"
              << "        double2* H2 = reinterpret_cast<double2*>(H + e * " << NH << "LL);\n"
              << "        for (int i = 0; i < " << NH / 2 << "; ++i) H2[i] = make_double2(h[2 * i], h[2 * i + 1]);\n"
              << "    } else\n";
        if (prec == 1 && NH % 4 == 0)
            s << "    if ((reinterpret_cast<unsigned long long>(H) & 15ull) == 0ull) {\n"
              << "        float4* H4 = reinterpret_cast<float4*>(H + e * " << NH << "LL);\n"
              << "        for (int i = 0; i < " << NH / 4 << "; ++i) H4[i] = make_float4(h[4 * i], h[4 * i + 1], h[4 * i + 2], "
              << "h[4 * i + 3]);\n    } else\n";
        s << "    for (int i = 0; i < " << NH << "; ++i) H[e * " << NH << "LL + i] = h[i];\n}\n";
    }
    // ---- mixed precision: the cache holds (hi, lo) float pairs in place of the doubles
    s << "extern \"C\" __global__ void __launch_bounds__(256) symxg_cache_to_df(long long count, double* cache)\n{\n"
         "    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n    if (i >= count) return;\n"
         "    const symxg_df v(cache[i]);\n    reinterpret_cast<float2*>(cache)[i] = make_float2(v.hi, v.lo);\n}\n";
    auto set_sum_df = [&](const std::string& q) {
        std::ostringstream t;
        if (sum.n_iterations == 0 || !sum_used(main_symbol)) return t.str();
        for (int j = 0; j < sum.stride; ++j) {
            const std::string v = "symxg_sum_data[" + q + " * " + std::to_string(sum.stride) + " + " + std::to_string(j) + "]";
            t << "        ind[" << (sum.first_symbol + j) << "] = symxg_df(" << v << "); in32[" << (sum.first_symbol + j)
              << "] = (float)" << v << ";\n";
        }
        return t.str();
    };
    auto load_cache_df = [&](const std::string& q) {
        std::ostringstream t;
        t << "        symxg_df c[" << std::max(1, K) << "]; float c32[" << std::max(1, K) << "];\n";
        if (K > 0)
            t << "        for (int k = 0; k < " << K << "; ++k) { const float2 v = cache[((long long)" << q << " * " << K
              << "LL + k) * n + e]; c[k] = symxg_df(v.x, v.y); c32[k] = v.x; }\n";
        else
            t << "        c[0] = symxg_df(0.0); c32[0] = 0.0f;\n";
        return t.str();
    };
    auto head_df = [&]() {
        std::ostringstream t;
        t << "    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n    if (e >= n) return;\n";
        t << "    const float2* __restrict__ cache = reinterpret_cast<const float2*>(cache_raw);\n";
        t << "    double in[" << NS << "];\n    symxg_gather(e, conn, maps, in);\n";
        t << "    symxg_df ind[" << NS << "]; float in32[" << NS << "];\n";
        t << "    for (int i = 0; i < " << NS << "; ++i) { ind[i] = symxg_df(in[i]); in32[i] = ind[i].hi; }\n";
        return t.str();
    };
    auto cond_check_df = [&](const std::string& zero_writes) {
        if (cond < 0) return std::string();
        std::ostringstream t;
        t << "    {\n" << set_sum_df("0") << load_cache_df("0")
          << "        symxg_df cv[1]; symxg_eval_cond_df(ind, c, cv);\n        if (!(cv[0] > symxg_df(0.0))) {\n"
          << zero_writes << "            return;\n        }\n    }\n";
        return t.str();
    };
    const std::string sig_df =
        "(long long n, const int* __restrict__ conn, const double* const* __restrict__ maps, "
        "const double* __restrict__ cache_raw, double* __restrict__ E";
    if (qp_parallel) {
        // lane lq of an element evaluates quadrature point lq (the element of the last group is
        // repeated past n, without stores, so every lane takes part in the shuffles)
        s << "extern \"C\" __global__ void __launch_bounds__(128) symxg_egh_df32" << sig_df
          << ", double* __restrict__ G, float* __restrict__ H)\n{\n";
        s << "    if (n <= 0) return;\n";
        s << "    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n";
        s << "    const int lq = (int)(t % SYMXG_NQ);\n    const bool st = t / SYMXG_NQ < n;\n";
        s << "    const long long e = st ? t / SYMXG_NQ : n - 1;\n";
        s << "    const float2* __restrict__ cache = reinterpret_cast<const float2*>(cache_raw);\n";
        s << "    double in[" << NS << "];\n    symxg_gather(e, conn, maps, in);\n";
        s << "    symxg_df ind[" << NS << "]; float in32[" << NS << "];\n";
        s << "    for (int i = 0; i < " << NS << "; ++i) { ind[i] = symxg_df(in[i]); in32[i] = ind[i].hi; }\n";
        s << "    {\n" << set_sum_df("lq");
        s << "        const float2* __restrict__ cq = cache + (long long)lq * " << K << "LL * n + e;\n";
        s << "        symxg_df eg[" << (NG + 1) << "];\n";
        s << "        for (int i = 0; i < " << NG + 1 << "; ++i) eg[i] = symxg_df(0.0);\n";
        s << "        symxg_eval_eg_dfl(ind, cq, n, eg);\n";
        s << "#pragma unroll\n        for (int i = 0; i < " << NG + 1 << "; ++i) eg[i] = symxg_qsum(eg[i]);\n";
        s << "        if (st && lq == 0) E[e] = symxg_to_double(eg[0]);\n";
        s << "#pragma unroll\n        for (int i = 0; i < " << NG << "; ++i)\n"
          << "            if (st && lq == i % SYMXG_NQ) G[e * " << NG << "LL + i] = symxg_to_double(eg[1 + i]);\n";
        s << "        symxg_eval_h_f32_q(in32, cq, n, H + e * " << NH << "LL, lq, st);\n    }\n}\n";
    } else {
        s << "extern \"C\" __global__ void __launch_bounds__(128) symxg_egh_df32" << sig_df
          << ", double* __restrict__ G, float* __restrict__ H)\n{\n" << head_df();
        std::ostringstream zw;
        zw << "            E[e] = 0.0;\n            for (int i = 0; i < " << NG << "; ++i) G[e * " << NG
           << "LL + i] = 0.0;\n            for (int i = 0; i < " << NH << "; ++i) H[e * " << NH << "LL + i] = 0.0f;\n";
        s << cond_check_df(zw.str());
        s << "    symxg_df eg[" << (NG + 1) << "];\n    float h[" << NH << "];\n";
        if (acc) {
            s << "    for (int i = 0; i < " << NH << "; ++i) h[i] = 0.0f;\n";
            s << "    for (int q = 0; q < " << NQ << "; ++q) {\n";
        } else {
            s << "    { const int q = 0; (void)q;\n";
        }
        s << set_sum_df("q");
        s << "        const float2* __restrict__ cq = cache + (long long)q * " << K << "LL * n + e;\n";
        s << "        symxg_eval_eg_dfl(ind, cq, n, eg);\n        symxg_eval_h_f32l(in32, cq, n, h);\n    }\n";
        s << "    E[e] = symxg_to_double(eg[0]);\n";
        // 16-byte stores where the rows allow it (one element's outputs are contiguous)
        if (NG % 2 == 0)
            s << "    if ((reinterpret_cast<unsigned long long>(G) & 15ull) == 0ull) {\n"
              << "        double2* G2 = reinterpret_cast<double2*>(G + e * " << NG << "LL);\n"
              << "        for (int i = 0; i < " << NG / 2 << "; ++i) G2[i] = make_double2(symxg_to_double(eg[1 + 2 * i]), "
              << "symxg_to_double(eg[2 + 2 * i]));\n    } else\n";
        s << "    for (int i = 0; i < " << NG << "; ++i) G[e * " << NG << "LL + i] = symxg_to_double(eg[1 + i]);\n";
        if (NH % 4 == 0)
            s << "    if ((reinterpret_cast<unsigned long long>(H) & 15ull) == 0ull) {\n"
              << "        float4* H4 = reinterpret_cast<float4*>(H + e * " << NH << "LL);\n"
              << "        for (int i = 0; i < " << NH / 4 << "; ++i) H4[i] = make_float4(h[4 * i], h[4 * i + 1], h[4 * i + 2], "
              << "h[4 * i + 3]);\n    } else\n";
        s << "    for (int i = 0; i < " << NH << "; ++i) H[e * " << NH << "LL + i] = h[i];\n}\n";
    }
    {
        s << "extern \"C\" __global__ void __launch_bounds__(128) symxg_e_df" << sig_df << ")\n{\n" << head_df();
        s << cond_check_df("            E[e] = 0.0;\n");
        s << "    symxg_df ev[1];\n";
        if (acc) s << "    for (int q = 0; q < " << NQ << "; ++q) {\n";
        else s << "    { const int q = 0; (void)q;\n";
        s << set_sum_df("q");
        s << "        const float2* __restrict__ cq = cache + (long long)q * " << K << "LL * n + e;\n";
        s << "        symxg_eval_e_dfl(ind, cq, n, ev);\n    }\n    E[e] = symxg_to_double(ev[0]);\n}\n";
    }

    // energy-only kernel (line search)
    s << "extern \"C\" __global__ void __launch_bounds__(128) symxg_e" << sig_common << ")\n{\n";
    s << "    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n    if (e >= n) return;\n";
    s << "    double in[" << NS << "];\n    symxg_gather(e, conn, maps, in);\n";
    s << cond_check("            E[e] = 0.0;\n");
    s << "    double ev[1];\n";
    if (acc) s << "    ev[0] = 0.0;\n    for (int q = 0; q < " << NQ << "; ++q) {\n";
    else s << "    { const int q = 0; (void)q;\n";
    s << set_sum("q", main_symbol) << load_cache("q", "double");
    s << "        symxg_eval_e(in, c, ev);\n    }\n    E[e] = ev[0];\n}\n";
    return s.str();
}

// DoF symbols of a potential, its derivatives and the generated CUDA source.
CompiledPotential prepare_potential(const Potential& pot, const GlobalPotential& GP)
{
    CompiledPotential cp;
    cp.name = pot.name;
    cp.pot = &pot;
    MappedWorkspace<double>& mws = *pot.mws;
    Expressions& g = mws.ws.get_expression_graph();
    std::vector<Scalar> wrt;
    for (size_t k = 0; k < mws.maps.size(); ++k) {
        const DataMap& m = mws.maps[k];
        int set = -1;
        for (size_t s = 0; s < GP.dofs.size(); ++s)
            if (GP.dofs[s].id == m.id) set = (int)s;
        if (set < 0) continue;
        if (m.stride != 3 || m.conn_column < 0)
            throw std::runtime_error("symx: DoF data of potential '" + pot.name +
                                     "' must be bound per item with 3 values (make_vector(s) with an index)");
        cp.dof_set.push_back(set);
        cp.dof_col.push_back(m.conn_column);
        for (int j = 0; j < 3; ++j) wrt.push_back(Scalar(g.symbol_node(m.first_symbol + j), &g));
    }
    cp.nb = (int)cp.dof_set.size();
    if (cp.nb == 0) throw std::runtime_error("symx: potential '" + pot.name + "' depends on no DoF");
    if (cp.nb > 10) throw std::runtime_error("symx_gb300: at most 10 DoF blocks per element (30x30 Hessians)");
    cp.conn_stride = mws.conn.stride;
    DiffCache cache;
    Vector grad = gradient(pot.expression, wrt, cache);
    Matrix hess = gradient(grad, wrt, true, cache);
    std::vector<int32_t> eg{pot.expression.expr_id};
    for (const Scalar& s : grad.values()) eg.push_back(s.expr_id);
    const int n = 3 * cp.nb;
    std::vector<int32_t> h_bm(n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            h_bm[(((i / 3) * cp.nb + (j / 3)) * 3 + (i % 3)) * 3 + (j % 3)] = hess(i, j).expr_id;
    const int32_t cond = pot.has_condition ? pot.condition.expr_id : -1;
    std::vector<uint8_t> is_dof(g.n_symbols(), 0);
    for (const Scalar& w : wrt) is_dof[w.get_symbol_idx()] = 1;
    cp.source = build_source(cp, g, eg, h_bm, {pot.expression.expr_id}, cond, mws.summation, is_dof, &cp.ops_eg,
                             &cp.ops_h, &cp.ops_e);
    return cp;
}

}  // namespace

struct SolverImpl {
    cudaStream_t stream = nullptr;
    std::vector<CompiledPotential> pots;
    std::vector<UploadedArray> arrays;
    int n_dofs = 0, n_blocks = 0;
    int64_t vstride = 0;                        // BCSR component stride (nnzb rounded up to 32)
    std::vector<int> dof_offsets;  // doubles, per DoF set (+ total)

    DevBuf<double> x, x_before, grad;
    DevBuf<double> E_el, g_el;
    DevBuf<float> H32;
    DevBuf<double> H64;
    int64_t n_elements_total = 0, n_gblocks = 0, n_hblocks = 0;

    DevBuf<int32_t> row_ptr, cols, diag_slot, contrib, gcontrib;
    // staged (bulk-copy) float SpMV: its plan and the padded row_ptr / cols it copies from
    symxg::PcgBuffers<float>::Staged staged;
    DevBuf<int32_t> row_ptr_ext, cols_ext;
    DevBuf<int64_t> slot_ptr, gptr;
    int64_t nnzb = 0;
    DevBuf<float> vals32, Dinv32;
    DevBuf<double> vals64, Dinv64;
    DevBuf<float> v32[6];
    DevBuf<float> la32;  // look-ahead PCG: six more vectors (PcgBuffers::la)
    DevBuf<double> v64[6];
    DevBuf<double> partials, scalars;
    DevBuf<unsigned> tickets;
    DevBuf<PcgState> pcg_state;
    DevBuf<int> flags;
    // projection: indices of the 12 x 12 element Hessians that need the full decomposition
    DevBuf<int64_t> proj_fallback, proj_pending;
    DevBuf<unsigned long long> proj_n_fallback, proj_n_pending;
    // Progressive projection: per element "projected in this evaluation", per element gradient
    // block "touches an active DoF block", the selected elements of one potential, and counters
    // (inactive DoF blocks, then the selection count of each potential)
    DevBuf<uint8_t> ppn_is_proj, ppn_gflag;
    DevBuf<int64_t> ppn_sel;
    DevBuf<unsigned long long> ppn_counts;
    symxg::ProjectionScratch proj_scratch()
    {
        symxg::ProjectionScratch ps;
        ps.fallback = proj_fallback.p;
        ps.n_fallback = proj_n_fallback.p;
        ps.pending = proj_pending.p;
        ps.n_pending = proj_n_pending.p;
        return ps;
    }
    // adjoint: mixed-derivative modules per (potential, data map), lambda on the device
    std::string cache_dir;
    std::map<std::pair<int, int>, std::shared_ptr<CudaModule>> mixed_modules;
    DevBuf<double> lambda, mixed_out;
    DevBuf<const double*> lmap_ptrs;
    double* h_scalars = nullptr;
    PcgState* h_state = nullptr;
    Precision allocated_precision = Precision::FP64;
    bool precision_allocated[2] = {false, false};

    ~SolverImpl()
    {
        if (h_scalars) cudaFreeHost(h_scalars);
        if (h_state) cudaFreeHost(h_state);
        if (stream) cudaStreamDestroy(stream);
    }

    void ensure_precision(Precision p)
    {
        const int k = (int)p;
        if (precision_allocated[k]) return;
        const size_t n = 4 * (size_t)n_blocks;
        if (p == Precision::Mixed) {
            H32.alloc((size_t)n_hblocks * 9);
            vals32.alloc((size_t)vstride * 9);
            Dinv32.alloc((size_t)n_blocks * 12);
            ck(cudaMemset(Dinv32.p, 0, sizeof(float) * Dinv32.n), "memset");
            for (auto& v : v32) {
                v.alloc(n);
                ck(cudaMemset(v.p, 0, sizeof(float) * n), "memset");
            }
            if (staged.lookahead) {
                la32.alloc(6 * n);
                ck(cudaMemset(la32.p, 0, sizeof(float) * 6 * n), "memset");
            }
        } else {
            H64.alloc((size_t)n_hblocks * 9);
            vals64.alloc((size_t)vstride * 9);
            Dinv64.alloc((size_t)n_blocks * 12);
            ck(cudaMemset(Dinv64.p, 0, sizeof(double) * Dinv64.n), "memset");
            for (auto& v : v64) {
                v.alloc(n);
                ck(cudaMemset(v.p, 0, sizeof(double) * n), "memset");
            }
        }
        precision_allocated[k] = true;
    }

    template <typename T> T* Hbuf();
    template <typename T> T* vals();
    template <typename T> T* Dinv();
    template <typename T> DevBuf<T>* vecs();

    void read_scalars(int count)
    {
        ck(cudaMemcpyAsync(h_scalars, scalars.p, sizeof(double) * count, cudaMemcpyDeviceToHost, stream), "copy scalars");
        ck(cudaStreamSynchronize(stream), "synchronize");
    }

    // The element kernels of the mixed path read the hoisted cache as double-float pairs, the
    // FP64 kernels as doubles: convert in place, or recompute the doubles, when the path changes.
    void ensure_cache(CompiledPotential& cp, bool df)
    {
        if (cp.n_cache == 0 || cp.n_elements == 0 || cp.cache_df == df) return;
        long long n = cp.n_elements;
        if (df) {
            long long count = n * cp.n_qp * cp.n_cache;
            double* c = cp.cache.p;
            void* args[] = {&count, &c};
            cp.module->launch("symxg_cache_to_df", dim3((unsigned)((count + 255) / 256)), dim3(256), 0, stream, args);
        } else {
            const int32_t* conn = cp.conn.p;
            const double* const* maps = cp.map_ptrs.p;
            double* cache = cp.cache.p;
            void* args[] = {&n, &conn, &maps, &cache};
            cp.module->launch("symxg_pre", dim3((unsigned)((n + 127) / 128)), dim3(128), 0, stream, args);
        }
        cp.cache_df = df;
    }

    // mode: 0 E+g+H in FP64, 1 mixed (E+g double-float, H FP32), 2 E only FP64, 3 E only double-float.
    // In the mixed modes, potentials of one DoF block per element (inertia or gravity, penalty
    // boundary conditions) keep E and g in FP64: their coefficients are large (a 1e8 penalty
    // times the rounding of x in double-float, about 1e-15 m, is a gradient error near 1e-7,
    // above the solver's tolerances), and one-vertex elements cost little in FP64.
    void launch_eval(int mode)
    {
        for (auto& cp : pots) {
            if (cp.n_elements == 0) continue;
            const bool fp64_eg = cp.nb == 1;
            const int m = (fp64_eg && mode == 3) ? 2 : mode;  // energy only: FP64
            const bool eg64_h32 = fp64_eg && m == 1;           // FP64 E+g, FP32 H
            ensure_cache(cp, (m == 1 || m == 3) && !fp64_eg);
            long long n = cp.n_elements;
            const int32_t* conn = cp.conn.p;
            const double* const* maps = cp.map_ptrs.p;
            const double* cache = cp.cache.p;
            double* E = E_el.p + cp.e_off;
            const unsigned grid = (unsigned)((n + 127) / 128);
            if (m >= 2) {
                void* args[] = {&n, &conn, &maps, &cache, &E};
                cp.module->launch(m == 2 ? "symxg_e" : "symxg_e_df", dim3(grid), dim3(128), 0, stream, args);
            } else {
                double* G = g_el.p + cp.g_off * 3;
                void* H = m == 0 ? (void*)(H64.p + cp.h_off * 9) : (void*)(H32.p + cp.h_off * 9);
                void* args[] = {&n, &conn, &maps, &cache, &E, &G, &H};
                const unsigned grid_eh = (unsigned)((n * cp.qp_lanes + 127) / 128);  // both E+g+H kernels
                const char* kname = m == 0 ? "symxg_egh_f64" : eg64_h32 ? "symxg_egh_f32" : "symxg_egh_df32";
                cp.module->launch(kname, dim3(eg64_h32 ? grid : grid_eh), dim3(128), 0, stream, args);
            }
        }
    }
};

template <> float* SolverImpl::Hbuf<float>() { return H32.p; }
template <> double* SolverImpl::Hbuf<double>() { return H64.p; }
template <> float* SolverImpl::vals<float>() { return vals32.p; }
template <> double* SolverImpl::vals<double>() { return vals64.p; }
template <> float* SolverImpl::Dinv<float>() { return Dinv32.p; }
template <> double* SolverImpl::Dinv<double>() { return Dinv64.p; }
template <> DevBuf<float>* SolverImpl::vecs<float>() { return v32; }
template <> DevBuf<double>* SolverImpl::vecs<double>() { return v64; }

// Source of the mixed-derivative kernel of one potential for the data map `mk` (the
// parameter): per element, out[j] = sum_i lambda_i * d g_i / d p_j for the map's symbols p_j,
// g the element gradient with respect to its DoF symbols (summed over the quadrature points
// of an FEM rule).  lambda_i are new symbols gathered from a DoF-shaped vector through the
// same maps as the DoFs.  Everything is evaluated in FP64 from the gathered data (no
// hoisting: the kernel runs once per adjoint).
std::string build_mixed_source(const CompiledPotential& cp, const GlobalPotential& GP, int mk)
{
    const Potential& pot = *cp.pot;
    MappedWorkspace<double>& mws = *pot.mws;
    Expressions& g = mws.ws.get_expression_graph();
    std::vector<Scalar> wrt;
    std::vector<int> dof_maps;
    for (size_t k = 0; k < mws.maps.size(); ++k) {
        bool is_dof = false;
        for (const auto& d : GP.dofs)
            if (d.id == mws.maps[k].id) is_dof = true;
        if (!is_dof) continue;
        dof_maps.push_back((int)k);
        for (int j = 0; j < 3; ++j) wrt.push_back(Scalar(g.symbol_node(mws.maps[k].first_symbol + j), &g));
    }
    const DataMap& pm = mws.maps[mk];
    DiffCache cache;
    Vector grad = gradient(pot.expression, wrt, cache);
    std::vector<Scalar> lam;
    for (size_t i = 0; i < wrt.size(); ++i) lam.push_back(Scalar(g.new_symbol(), &g));  // new_symbol: node id
    std::vector<int32_t> outs;
    for (int j = 0; j < pm.stride; ++j) {
        const Scalar pj(g.symbol_node(pm.first_symbol + j), &g);
        Scalar acc = pj.get_zero();
        for (size_t i = 0; i < wrt.size(); ++i) acc += lam[i] * diff(grad[(int32_t)i], pj, cache);
        outs.push_back(acc.expr_id);
    }
    const Summation& sum = mws.summation;
    const int NS = g.n_symbols();
    const int NQ = std::max(1, sum.n_iterations);
    const bool acc = sum.n_iterations > 1;
    std::ostringstream s;
    s << "// generated mixed-derivative kernel of potential '" << cp.name << "' for data map " << mk << "\n";
    s << codegen_prelude();
    s << emit_device_function(g, outs, "symxg_mixed_f", "double", acc, nullptr, nullptr);
    if (pot.has_condition) s << emit_device_function(g, {pot.condition.expr_id}, "symxg_mixed_cond", "double", false, nullptr, nullptr);
    if (sum.n_iterations > 0) {
        s << "static __device__ const double symxg_sum_data[" << sum.data.size() << "] = {";
        for (size_t i = 0; i < sum.data.size(); ++i) s << (i ? ", " : "") << double_literal(sum.data[i]);
        s << "};\n";
    }
    s << "extern \"C\" __global__ void __launch_bounds__(128) symxg_mixed(long long n, const int* __restrict__ conn, "
         "const double* const* __restrict__ maps, const double* const* __restrict__ lmaps, double* __restrict__ out)\n{\n";
    s << "    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n    if (e >= n) return;\n";
    s << "    const int* __restrict__ ce = conn + e * " << cp.conn_stride << "LL;\n    (void)ce;\n";
    s << "    double in[" << NS << "];\n";
    for (size_t k = 0; k < mws.maps.size(); ++k) {
        const DataMap& m = mws.maps[k];
        s << "    { const double* __restrict__ m = maps[" << k << "]";
        if (m.conn_column >= 0) s << " + (long long)ce[" << m.conn_column << "] * " << m.stride << "LL";
        s << ";";
        for (int j = 0; j < m.stride; ++j) s << " in[" << (m.first_symbol + j) << "] = m[" << j << "];";
        s << " }\n";
    }
    int li = 0;
    for (int k : dof_maps) {
        const DataMap& m = mws.maps[k];
        s << "    { const double* __restrict__ m = lmaps[" << k << "] + (long long)ce[" << m.conn_column << "] * 3LL;";
        for (int j = 0; j < 3; ++j) s << " in[" << lam[li++].get_symbol_idx() << "] = m[" << j << "];";
        s << " }\n";
    }
    auto set_sum = [&](const std::string& q) {
        std::ostringstream t;
        for (int j = 0; j < sum.stride && sum.n_iterations > 0; ++j)
            t << "        in[" << (sum.first_symbol + j) << "] = symxg_sum_data[" << q << " * " << sum.stride << " + " << j
              << "];\n";
        return t.str();
    };
    s << "    double r[" << pm.stride << "];\n    for (int j = 0; j < " << pm.stride << "; ++j) r[j] = 0.0;\n";
    if (pot.has_condition) {
        s << "    {\n" << set_sum("0") << "        double cv[1]; symxg_mixed_cond(in, nullptr, cv);\n"
          << "        if (!(cv[0] > 0.0)) { for (int j = 0; j < " << pm.stride << "; ++j) out[e * " << pm.stride
          << "LL + j] = 0.0; return; }\n    }\n";
    }
    s << "    for (int q = 0; q < " << NQ << "; ++q) {\n" << set_sum("q") << "        symxg_mixed_f(in, nullptr, r);\n    }\n";
    s << "    for (int j = 0; j < " << pm.stride << "; ++j) out[e * " << pm.stride << "LL + j] = r[j];\n}\n";
    return s.str();
}

std::vector<std::string> generate_mixed_kernel_sources(const GlobalPotential& GP, std::uintptr_t param)
{
    std::vector<std::string> out;
    for (const Potential& pot : GP.potentials) {
        CompiledPotential cp = prepare_potential(pot, GP);
        for (size_t k = 0; k < pot.mws->maps.size(); ++k)
            if (pot.mws->maps[k].id == param) out.push_back(build_mixed_source(cp, GP, (int)k));
    }
    return out;
}

std::vector<std::string> generate_element_kernel_sources(const GlobalPotential& GP)
{
    std::vector<std::string> out;
    for (const Potential& pot : GP.potentials) out.push_back(prepare_potential(pot, GP).source);
    return out;
}

std::string to_string(SolverReturn r)
{
    switch (r) {
        case SolverReturn::Successful: return "Successful";
        case SolverReturn::Running: return "Running";
        case SolverReturn::InvalidInitialState: return "InvalidInitialState";
        case SolverReturn::TooManyIterations: return "TooManyIterations";
        case SolverReturn::TooManyArmijoIterations: return "TooManyArmijoIterations";
        case SolverReturn::LinearSystemSolveFailure: return "LinearSystemSolveFailure";
        case SolverReturn::TooManyInvalidIntermediateIterations: return "TooManyInvalidIntermediateIterations";
        case SolverReturn::StepDoesNotDescend: return "StepDoesNotDescend";
        default: return "InvalidConvergedState";
    }
}

NewtonsMethod::~NewtonsMethod() = default;

NewtonsMethod::NewtonsMethod(spGlobalPotential G, spContext ctx)
    : global_potential(std::move(G)), context(ctx ? std::move(ctx) : Context::create()), impl(new SolverImpl())
{
    SolverImpl& I = *impl;
    GlobalPotential& GP = *global_potential;
    if (GP.dofs.empty()) throw std::runtime_error("symx: no degrees of freedom registered (add_dof)");
    I.dof_offsets = GP.get_dofs_offsets();
    I.n_dofs = I.dof_offsets.back();
    if (I.n_dofs <= 0 || I.n_dofs % 3 != 0) throw std::runtime_error("symx: number of DoFs must be a positive multiple of 3");
    I.n_blocks = I.n_dofs / 3;
    const std::string cache_dir =
        context->compilation_directory.empty() ? symxg::default_cache_dir() : context->compilation_directory;
    I.cache_dir = cache_dir;

    // ---- per potential: DoF symbols, differentiation, code generation, compilation
    for (const Potential& pot : GP.potentials) {
        CompiledPotential cp = prepare_potential(pot, GP);
        symxg::CompileInfo info;
        cp.module = CudaModule::build(cp.source, cache_dir, {}, &info);
        if (context->verbosity > 0)
            std::printf("symx_gb300: potential '%s' %s in %.2f s (E+g %lld ops, H %lld ops)\n", cp.name.c_str(),
                        info.cached ? "loaded" : "compiled", info.seconds, (long long)cp.ops_eg.total(),
                        (long long)cp.ops_h.total());
        I.pots.push_back(std::move(cp));
    }
    ck(cudaStreamCreateWithFlags(&I.stream, cudaStreamNonBlocking), "stream");

    // ---- topology: element blocks -> BCSR slots (fixed order), gradient gather map
    std::vector<int64_t> set_block_off;
    for (size_t s = 0; s < GP.dofs.size(); ++s) set_block_off.push_back(I.dof_offsets[s] / 3);
    int64_t e_off = 0, g_off = 0, h_off = 0;
    for (auto& cp : I.pots) {
        cp.n_elements = cp.pot->mws->conn.n_elements();
        cp.e_off = e_off;
        cp.g_off = g_off;
        cp.h_off = h_off;
        e_off += cp.n_elements;
        g_off += cp.n_elements * cp.nb;
        h_off += cp.n_elements * cp.nb * cp.nb;
    }
    I.n_elements_total = e_off;
    I.n_gblocks = g_off;
    I.n_hblocks = h_off;
    if (h_off > (int64_t)INT32_MAX) throw std::runtime_error("symx_gb300: more than 2^31 element Hessian blocks");

    auto row_of = [&](const CompiledPotential& cp, const int32_t* conn, int64_t e, int a) -> int64_t {
        const int32_t v = conn[e * cp.conn_stride + cp.dof_col[a]];
        const int set = cp.dof_set[a];
        const int64_t n_items = GP.dofs[set].n_dofs() / 3;
        if (v < 0 || v >= n_items)
            throw std::runtime_error("symx: potential '" + cp.name + "' references DoF item " + std::to_string(v) +
                                     " out of range");
        return set_block_off[set] + v;
    };
    const int nbk = I.n_blocks;
    std::vector<int64_t> cnt(nbk + 1, 0);
    for (auto& cp : I.pots) {
        const int32_t* conn = cp.pot->mws->conn.data();
        for (int64_t e = 0; e < cp.n_elements; ++e)
            for (int a = 0; a < cp.nb; ++a) cnt[row_of(cp, conn, e, a) + 1] += cp.nb;
    }
    for (int r = 0; r < nbk; ++r) cnt[r + 1] += cnt[r] + 1;  // +1: the diagonal block always exists
    std::vector<int32_t> raw(cnt[nbk]);
    {
        std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
        for (int r = 0; r < nbk; ++r) raw[fill[r]++] = r;
        for (auto& cp : I.pots) {
            const int32_t* conn = cp.pot->mws->conn.data();
            for (int64_t e = 0; e < cp.n_elements; ++e) {
                int64_t rows[64];
                for (int a = 0; a < cp.nb; ++a) rows[a] = row_of(cp, conn, e, a);
                for (int a = 0; a < cp.nb; ++a)
                    for (int b = 0; b < cp.nb; ++b) raw[fill[rows[a]]++] = (int32_t)rows[b];
            }
        }
    }
    std::vector<int32_t> row_ptr(nbk + 1, 0), cols;
    cols.reserve(raw.size() / 4);
    for (int r = 0; r < nbk; ++r) {
        auto b = raw.begin() + cnt[r], e = raw.begin() + cnt[r + 1];
        std::sort(b, e);
        auto u = std::unique(b, e);
        cols.insert(cols.end(), b, u);
        row_ptr[r + 1] = (int32_t)cols.size();
    }
    std::vector<int32_t>().swap(raw);
    I.nnzb = (int64_t)cols.size();
    I.vstride = (I.nnzb + 31) / 32 * 32;
    auto slot_of = [&](int64_t r, int64_t c) -> int64_t {
        auto b = cols.begin() + row_ptr[r], e = cols.begin() + row_ptr[r + 1];
        return std::lower_bound(b, e, (int32_t)c) - cols.begin();
    };
    std::vector<int32_t> diag(nbk);
    for (int r = 0; r < nbk; ++r) diag[r] = (int32_t)slot_of(r, r);
    // contributions per slot, in (potential, element, a, b) order
    std::vector<int64_t> sptr(I.nnzb + 1, 0);
    std::vector<int32_t> slot_of_contrib(I.n_hblocks);
    std::vector<int64_t> gcnt(nbk + 1, 0);
    for (auto& cp : I.pots) {
        const int32_t* conn = cp.pot->mws->conn.data();
        for (int64_t e = 0; e < cp.n_elements; ++e) {
            int64_t rows[64];
            for (int a = 0; a < cp.nb; ++a) rows[a] = row_of(cp, conn, e, a);
            for (int a = 0; a < cp.nb; ++a) {
                gcnt[rows[a] + 1]++;
                for (int b = 0; b < cp.nb; ++b) {
                    const int64_t s = slot_of(rows[a], rows[b]);
                    slot_of_contrib[cp.h_off + (e * cp.nb + a) * cp.nb + b] = (int32_t)s;
                    sptr[s + 1]++;
                }
            }
        }
    }
    for (int64_t s = 0; s < I.nnzb; ++s) sptr[s + 1] += sptr[s];
    for (int r = 0; r < nbk; ++r) gcnt[r + 1] += gcnt[r];
    std::vector<int32_t> contrib(I.n_hblocks), gcontrib(I.n_gblocks);
    {
        std::vector<int64_t> fill(sptr.begin(), sptr.end() - 1);
        for (int64_t k = 0; k < I.n_hblocks; ++k) contrib[fill[slot_of_contrib[k]]++] = (int32_t)k;
        std::vector<int64_t> gfill(gcnt.begin(), gcnt.end() - 1);
        for (auto& cp : I.pots) {
            const int32_t* conn = cp.pot->mws->conn.data();
            for (int64_t e = 0; e < cp.n_elements; ++e)
                for (int a = 0; a < cp.nb; ++a)
                    gcontrib[gfill[row_of(cp, conn, e, a)]++] = (int32_t)(cp.g_off + e * cp.nb + a);
        }
    }

    // ---- device buffers
    auto up = [&](auto& buf, const auto& host) {
        using T = typename std::decay<decltype(host[0])>::type;
        buf.alloc(host.size());
        if (!host.empty()) ck(cudaMemcpy(buf.p, host.data(), sizeof(T) * host.size(), cudaMemcpyHostToDevice), "upload");
    };
    up(I.row_ptr, row_ptr);
    up(I.cols, cols);
    {
        const symxg::StagedSizes ss = symxg::plan_staged_spmv(nbk, row_ptr.data(), I.staged);
        if (ss.row_ptr_ext > 0) {
            std::vector<int32_t> rpx(ss.row_ptr_ext, (int32_t)I.nnzb), cx(ss.cols_ext, 0);
            std::copy(row_ptr.begin(), row_ptr.end(), rpx.begin());
            std::copy(cols.begin(), cols.end(), cx.begin());
            up(I.row_ptr_ext, rpx);
            up(I.cols_ext, cx);
            I.staged.row_ptr_ext = I.row_ptr_ext.p;
            I.staged.cols_ext = I.cols_ext.p;
        }
    }
    up(I.diag_slot, diag);
    up(I.slot_ptr, sptr);
    up(I.contrib, contrib);
    up(I.gptr, gcnt);
    up(I.gcontrib, gcontrib);
    I.x.alloc(I.n_dofs);
    I.x_before.alloc(I.n_dofs);
    I.grad.alloc(I.n_dofs);
    I.E_el.alloc(std::max<int64_t>(1, I.n_elements_total));
    I.g_el.alloc(std::max<int64_t>(1, I.n_gblocks * 3));
    I.partials.alloc(2 * symxg::kPcgMaxPartials);
    I.scalars.alloc(16);
    I.tickets.alloc(16);
    ck(cudaMemset(I.tickets.p, 0, sizeof(unsigned) * 16), "memset");
    I.pcg_state.alloc(1);
    I.flags.alloc(4);
    {
        int64_t n12 = 0;
        for (auto& cp : I.pots)
            if (cp.nb == 4) n12 = std::max<int64_t>(n12, cp.n_elements);
        if (n12 > 0) {
            I.proj_fallback.alloc(n12);
            I.proj_n_fallback.alloc(1);
            I.proj_pending.alloc(n12);
            I.proj_n_pending.alloc(1);
        }
    }
    ck(cudaMallocHost(&I.h_scalars, sizeof(double) * 16), "pinned");
    ck(cudaMallocHost(&I.h_state, sizeof(PcgState)), "pinned");
    for (auto& cp : I.pots) {
        const int32_t* conn = cp.pot->mws->conn.data();
        cp.conn.alloc((size_t)cp.n_elements * cp.conn_stride);
        if (cp.conn.n)
            ck(cudaMemcpy(cp.conn.p, conn, sizeof(int32_t) * cp.conn.n, cudaMemcpyHostToDevice), "upload connectivity");
        cp.map_ptrs.alloc(cp.pot->mws->maps.size());
        cp.cache.alloc(std::max<size_t>(1, (size_t)cp.n_elements * cp.n_qp * cp.n_cache));
        cp.pot->mws->verify_no_out_of_bounds();
    }
}

int NewtonsMethod::n_dof_blocks() const { return impl->n_blocks; }
int64_t NewtonsMethod::n_hessian_blocks() const { return impl->nnzb; }
double* NewtonsMethod::device_dofs() { return impl->x.p; }
std::array<int64_t, 3> NewtonsMethod::op_counts(int p) const
{
    const auto& cp = impl->pots.at(p);
    return {cp.ops_eg.total(), cp.ops_h.total(), cp.ops_e.total()};
}
std::string NewtonsMethod::generated_source(int p) const { return impl->pots.at(p).source; }

void NewtonsMethod::upload()
{
    SolverImpl& I = *impl;
    GlobalPotential& GP = *global_potential;
    int64_t bytes = sizeof(double) * (int64_t)I.n_dofs;
    // DoFs
    for (size_t s = 0; s < GP.dofs.size(); ++s)
        ck(cudaMemcpyAsync(I.x.p + I.dof_offsets[s], GP.dofs[s].data(), sizeof(double) * GP.dofs[s].n_dofs(),
                           cudaMemcpyHostToDevice, I.stream),
           "upload dofs");
    // every other bound array, de-duplicated by container and pointer
    for (auto& cp : I.pots) {
        const auto& maps = cp.pot->mws->maps;
        std::vector<const double*> ptrs(maps.size());
        for (size_t k = 0; k < maps.size(); ++k) {
            const DataMap& m = maps[k];
            int set = -1;
            for (size_t s = 0; s < GP.dofs.size(); ++s)
                if (GP.dofs[s].id == m.id) set = (int)s;
            if (set >= 0) {
                ptrs[k] = I.x.p + I.dof_offsets[set];
                continue;
            }
            const double* host = m.data();
            const int64_t items = m.n_items();
            const int64_t n = items < 0 ? m.stride : items * m.stride;
            UploadedArray* ua = nullptr;
            for (auto& a : I.arrays)
                if (a.id == m.id && a.host == host && a.n == n) ua = &a;
            if (!ua) {
                I.arrays.emplace_back();
                ua = &I.arrays.back();
                ua->id = m.id;
                ua->host = host;
                ua->n = n;
                ua->dev.alloc((size_t)n);
            }
            ptrs[k] = ua->dev.p;
        }
        // arrays are re-read on every upload: the user may change them between solves
        ck(cudaMemcpyAsync(cp.map_ptrs.p, ptrs.data(), sizeof(double*) * ptrs.size(), cudaMemcpyHostToDevice, I.stream),
           "upload map pointers");
        bytes += (int64_t)(sizeof(double*) * ptrs.size());
        ck(cudaStreamSynchronize(I.stream), "synchronize");
    }
    for (auto& a : I.arrays) {
        ck(cudaMemcpyAsync(a.dev.p, a.host, sizeof(double) * a.n, cudaMemcpyHostToDevice, I.stream), "upload data");
        bytes += (int64_t)sizeof(double) * a.n;
    }
    // values that depend only on the uploaded data are computed once here
    for (auto& cp : I.pots) {
        if (cp.n_cache == 0 || cp.n_elements == 0) continue;
        long long n = cp.n_elements;
        const int32_t* conn = cp.conn.p;
        const double* const* maps = cp.map_ptrs.p;
        double* cache = cp.cache.p;
        void* args[] = {&n, &conn, &maps, &cache};
        cp.module->launch("symxg_pre", dim3((unsigned)((n + 127) / 128)), dim3(128), 0, I.stream, args);
        cp.cache_df = false;
    }
    ck(cudaStreamSynchronize(I.stream), "synchronize");
    h2d_bytes_ = bytes;
}

void NewtonsMethod::download()
{
    SolverImpl& I = *impl;
    GlobalPotential& GP = *global_potential;
    for (size_t s = 0; s < GP.dofs.size(); ++s)
        ck(cudaMemcpyAsync(GP.dofs[s].data(), I.x.p + I.dof_offsets[s], sizeof(double) * GP.dofs[s].n_dofs(),
                           cudaMemcpyDeviceToHost, I.stream),
           "download dofs");
    ck(cudaStreamSynchronize(I.stream), "synchronize");
    d2h_bytes_ = sizeof(double) * (int64_t)I.n_dofs;
}

SolverReturn NewtonsMethod::solve()
{
    upload();
    const SolverReturn r = solve_device();
    download();
    stats.d2h_bytes = d2h_bytes_;
    return r;
}

double NewtonsMethod::evaluate_energy()
{
    SolverImpl& I = *impl;
    I.launch_eval(2);
    symxg::launch_sum(I.E_el.p, I.n_elements_total, I.partials.p, I.tickets.p + 4, I.scalars.p, I.stream);
    I.read_scalars(1);
    return I.h_scalars[0];
}

double NewtonsMethod::evaluate(double* grad_host)
{
    SolverImpl& I = *impl;
    I.ensure_precision(Precision::FP64);
    I.launch_eval(0);
    symxg::launch_sum(I.E_el.p, I.n_elements_total, I.partials.p, I.tickets.p + 4, I.scalars.p, I.stream);
    symxg::launch_gather_gradient(I.n_blocks, I.gptr.p, I.gcontrib.p, I.g_el.p, I.grad.p, I.stream);
    I.read_scalars(1);
    if (grad_host)
        ck(cudaMemcpy(grad_host, I.grad.p, sizeof(double) * I.n_dofs, cudaMemcpyDeviceToHost), "download gradient");
    return I.h_scalars[0];
}

namespace {
// Project `count` element Hessians of potential cp (all of them, or those listed in sel):
// the 12 x 12 ones with FP64-accurate arithmetic when the settings ask for it.
template <typename T>
void project_potential(SolverImpl& I, const CompiledPotential& cp, const NewtonSettings& s, int64_t count,
                       cudaStream_t stream, const int64_t* sel = nullptr)
{
    if (s.projection_fp64_refinement && cp.nb == 4)
        symxg::launch_project_pd_refined12<T>(I.Hbuf<T>() + cp.h_off * 9, count, s.projection_eps,
                                              s.project_to_pd_use_mirroring, I.flags.p, stream, I.proj_scratch(), sel);
    else
        symxg::launch_project_pd<T>(I.Hbuf<T>() + cp.h_off * 9, 3 * cp.nb, count, (T)s.projection_eps,
                                    s.project_to_pd_use_mirroring, I.flags.p, stream, I.proj_scratch(), sel);
}

template <typename T>
void assemble_t(SolverImpl& I, bool project, const NewtonSettings& s, int mode)
{
    I.ensure_precision(std::is_same<T, float>::value ? Precision::Mixed : Precision::FP64);
    I.launch_eval(mode);
    if (project) {
        ck(cudaMemsetAsync(I.flags.p, 0, sizeof(int), I.stream), "memset");
        for (auto& cp : I.pots) project_potential<T>(I, cp, s, cp.n_elements, I.stream);
    }
    symxg::launch_assemble_blocks<T>(I.nnzb, I.slot_ptr.p, I.contrib.p, I.Hbuf<T>(), I.vals<T>(), I.vstride, I.stream);
}
}  // namespace

void NewtonsMethod::assembled_hessian(bool project, int32_t* n_blocks, int64_t* nnzb, int32_t* row_ptr, int32_t* cols,
                                      double* vals)
{
    SolverImpl& I = *impl;
    *n_blocks = I.n_blocks;
    *nnzb = I.nnzb;
    if (!vals) return;
    std::vector<double> soa((size_t)I.vstride * 9);
    if (settings.precision == Precision::Mixed) {
        assemble_t<float>(I, project, settings, 1);
        std::vector<float> f(soa.size());
        ck(cudaStreamSynchronize(I.stream), "synchronize");
        ck(cudaMemcpy(f.data(), I.vals32.p, sizeof(float) * f.size(), cudaMemcpyDeviceToHost), "download");
        std::copy(f.begin(), f.end(), soa.begin());
    } else {
        assemble_t<double>(I, project, settings, 0);
        ck(cudaStreamSynchronize(I.stream), "synchronize");
        ck(cudaMemcpy(soa.data(), I.vals64.p, sizeof(double) * soa.size(), cudaMemcpyDeviceToHost), "download");
    }
    for (int64_t k = 0; k < I.nnzb; ++k)
        for (int m = 0; m < 9; ++m) vals[k * 9 + m] = soa[(size_t)m * I.vstride + k];
    ck(cudaMemcpy(row_ptr, I.row_ptr.p, sizeof(int32_t) * (I.n_blocks + 1), cudaMemcpyDeviceToHost), "download");
    ck(cudaMemcpy(cols, I.cols.p, sizeof(int32_t) * I.nnzb, cudaMemcpyDeviceToHost), "download");
}

void NewtonsMethod::element_outputs(int p, bool project, double* E, double* g, double* H)
{
    SolverImpl& I = *impl;
    const auto& cp = I.pots.at(p);
    const int n = 3 * cp.nb;
    const bool mixed = settings.precision == Precision::Mixed;
    if (mixed) assemble_t<float>(I, project, settings, 1);
    else assemble_t<double>(I, project, settings, 0);
    ck(cudaStreamSynchronize(I.stream), "synchronize");
    if (E) ck(cudaMemcpy(E, I.E_el.p + cp.e_off, sizeof(double) * cp.n_elements, cudaMemcpyDeviceToHost), "download");
    if (g) ck(cudaMemcpy(g, I.g_el.p + cp.g_off * 3, sizeof(double) * cp.n_elements * n, cudaMemcpyDeviceToHost), "download");
    if (H) {
        std::vector<double> bm((size_t)cp.n_elements * n * n);
        if (mixed) {
            std::vector<float> f(bm.size());
            ck(cudaMemcpy(f.data(), I.H32.p + cp.h_off * 9, sizeof(float) * f.size(), cudaMemcpyDeviceToHost), "download");
            std::copy(f.begin(), f.end(), bm.begin());
        } else {
            ck(cudaMemcpy(bm.data(), I.H64.p + cp.h_off * 9, sizeof(double) * bm.size(), cudaMemcpyDeviceToHost), "download");
        }
        for (int64_t e = 0; e < cp.n_elements; ++e)
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j)
                    H[(e * n + i) * n + j] = bm[e * n * n + (((i / 3) * cp.nb + (j / 3)) * 3 + (i % 3)) * 3 + (j % 3)];
    }
}

namespace {

// Progressive projection step (NewtonsMethod.cpp:305-329 with
// ElementHessians::project_to_PD_for_update__selectively, ElementHessians.cpp:69-182): the DoF
// blocks whose gradient max-abs reaches `thr` are active; every element not projected yet in
// this evaluation (is_proj cleared when `fresh`) that touches an active block is projected.
// Sets all_projected when every block is active; returns the number of elements projected.
template <typename T>
uint64_t ppn_project(SolverImpl& I, const NewtonSettings& S, cudaStream_t s, double thr, bool fresh,
                     bool& all_projected)
{
    const size_t np = I.pots.size();
    if (I.ppn_is_proj.n != (size_t)std::max<int64_t>(1, I.n_elements_total)) {
        I.ppn_is_proj.alloc(std::max<int64_t>(1, I.n_elements_total));
        I.ppn_sel.alloc(std::max<int64_t>(1, I.n_elements_total));
        I.ppn_gflag.alloc(std::max<int64_t>(1, I.n_gblocks));
        fresh = true;
    }
    I.ppn_counts.alloc(1 + np);
    if (fresh) ck(cudaMemsetAsync(I.ppn_is_proj.p, 0, I.ppn_is_proj.n, s), "memset");
    ck(cudaMemsetAsync(I.ppn_gflag.p, 0, I.ppn_gflag.n, s), "memset");
    ck(cudaMemsetAsync(I.ppn_counts.p, 0, sizeof(unsigned long long) * (1 + np), s), "memset");
    symxg::launch_ppn_mark_blocks(I.n_blocks, I.grad.p, thr, I.gptr.p, I.gcontrib.p, I.ppn_gflag.p, I.ppn_counts.p, s);
    for (size_t k = 0; k < np; ++k) {
        const auto& cp = I.pots[k];
        symxg::launch_select_elements(cp.n_elements, cp.nb, I.ppn_gflag.p + cp.g_off, I.ppn_is_proj.p + cp.e_off,
                                      I.ppn_sel.p + cp.e_off, I.ppn_counts.p + 1 + k, s);
    }
    std::vector<unsigned long long> counts(1 + np);
    ck(cudaMemcpyAsync(counts.data(), I.ppn_counts.p, sizeof(unsigned long long) * (1 + np), cudaMemcpyDeviceToHost, s),
       "copy counts");
    ck(cudaStreamSynchronize(s), "synchronize");
    all_projected = counts[0] == 0;
    uint64_t total = 0;
    for (size_t k = 0; k < np; ++k) {
        const auto& cp = I.pots[k];
        const int64_t n = (int64_t)counts[1 + k];
        if (n > 0) project_potential<T>(I, cp, S, n, s, I.ppn_sel.p + cp.e_off);
        total += (uint64_t)n;
    }
    return total;
}

template <typename T>
SolverReturn solve_t(SolverImpl& I, const NewtonSettings& S, SolveStats& st, int verbosity)
{
    I.ensure_precision(std::is_same<T, float>::value ? Precision::Mixed : Precision::FP64);
    const int mode = std::is_same<T, float>::value ? 1 : 0;
    const int64_t n = I.n_dofs;
    cudaStream_t s = I.stream;
    StageTimer timer;
    timer.s = s;
    DevBuf<T>* V = I.vecs<T>();
    PcgBuffers<T> B;
    B.n_blocks = I.n_blocks;
    B.row_ptr = I.row_ptr.p;
    B.cols = I.cols.p;
    B.vals = I.vals<T>();
    B.vals_stride = I.vstride;
    B.Dinv = I.Dinv<T>();
    B.x = V[0].p;
    B.r = V[1].p;
    B.z = V[2].p;
    B.p = V[3].p;
    B.q = V[4].p;
    B.p2 = V[5].p;
    B.partials = I.partials.p;
    B.tickets = I.tickets.p;
    B.state = I.pcg_state.p;
    if constexpr (std::is_same<T, float>::value) {
        B.staged = I.staged;
        B.staged.f64_sums = S.cg_fp64_partial_sums ? 1 : 0;
        B.la = S.cg_lookahead && I.staged.lookahead ? I.la32.p : nullptr;
    }
    T* du = V[0].p;

    if (S.linear_solver != LinearSolver::BDPCG) throw std::runtime_error("symx_gb300: only the BDPCG linear solver is implemented");

    double res0 = std::numeric_limits<double>::max();
    double E0 = 0.0, residual = 0.0;
    SolverReturn result = SolverReturn::Running;
    struct PendingEvent { std::string name; cudaEvent_t a, b; };
    std::vector<PendingEvent> pending_kernel_events;
    int it = -1;
    int pdn_countdown = 0;        // ProjectOnDemand: iterations left with full projection
    double ppn_threshold = -1.0;  // Progressive: gradient threshold (-1: not determined yet)
    ck(cudaMemsetAsync(I.flags.p, 0, sizeof(int), s), "memset");
    while (result == SolverReturn::Running) {
        ++it;
        if (it == S.max_iterations) {
            result = S.max_iterations_as_success ? SolverReturn::Successful : SolverReturn::TooManyIterations;
            break;
        }
        // energy, gradient and element Hessians
        timer.start("evaluate_P_grad_hess");
        I.launch_eval(mode);
        symxg::launch_sum(I.E_el.p, I.n_elements_total, I.partials.p, I.tickets.p + 4, I.scalars.p, s);
        symxg::launch_gather_gradient(I.n_blocks, I.gptr.p, I.gcontrib.p, I.g_el.p, I.grad.p, s);
        symxg::launch_max_abs(I.grad.p, n, I.partials.p, I.tickets.p + 4, I.scalars.p + 1, s);
        timer.stop();
        I.read_scalars(2);
        E0 = I.h_scalars[0];
        residual = I.h_scalars[1];
        if (verbosity > 0) std::printf("  %2d. r0: %.2e | E: %.6e | ", it, residual, E0);
        if (it == 0) res0 = residual;
        if (residual < S.bailout_residual) { result = SolverReturn::Successful; break; }
        if (it >= S.min_iterations) {
            if (residual < S.residual_tolerance_abs) { result = SolverReturn::Successful; break; }
            if (it > 0 && residual / res0 < S.residual_tolerance_rel) { result = SolverReturn::Successful; break; }
        }
        // projection, assembly and solve until the direction descends or nothing is left to
        // project (NewtonsMethod.cpp:133-186; _project_and_assemble :257-341; the adaptive
        // modes' _increase_projection / _decrease_projection :343-373).  Element Hessians of
        // this evaluation start unprojected; the global matrix is re-assembled from them after
        // each projection (the reference adds the projected-minus-original differences instead,
        // ElementHessians.cpp:258-294: the same matrix up to rounding).
        uint64_t n_projected_it = 0;
        bool projected_all = false;
        bool ppn_cleared = false;
        double du_dot_grad = 0.0, du_max = 0.0;
        for (;;) {
            bool all_projected = false;
            timer.start("project_to_PD");
            if (S.projection_mode == ProjectionToPD::ProjectedNewton ||
                (S.projection_mode == ProjectionToPD::ProjectOnDemand && pdn_countdown > 0)) {
                if (!projected_all) {
                    for (auto& cp : I.pots) {
                        cudaEvent_t a = nullptr, b = nullptr;
                        const bool timed = S.time_kernels;
                        if (timed) {
                            cudaEventCreate(&a);
                            cudaEventCreate(&b);
                            cudaEventRecord(a, s);
                        }
                        project_potential<T>(I, cp, S, cp.n_elements, s);
                        if (timed) {
                            cudaEventRecord(b, s);
                            pending_kernel_events.push_back(
                                {"project_pd_" + std::to_string(3 * cp.nb) + (sizeof(T) == 4 ? "_f32" : "_f64"), a, b});
                        }
                    }
                    n_projected_it = (uint64_t)I.n_elements_total;
                    projected_all = true;
                }
                all_projected = true;
            } else if (S.projection_mode == ProjectionToPD::Progressive && ppn_threshold > 0.0) {
                if (ppn_threshold < 1e-12) ppn_threshold = 0.0;
                n_projected_it += ppn_project<T>(I, S, s, ppn_threshold, !ppn_cleared, all_projected);
                ppn_cleared = true;
            }
            timer.stop();
            timer.start("assembly");
            symxg::launch_assemble_blocks<T>(I.nnzb, I.slot_ptr.p, I.contrib.p, I.Hbuf<T>(), I.vals<T>(), I.vstride, s);
            symxg::launch_block_jacobi_setup<T>(I.n_blocks, I.diag_slot.p, I.vals<T>(), I.vstride, I.Dinv<T>(), s);
            timer.stop();
            // linear solve: block-Jacobi PCG with the reference's forcing sequence
            timer.start("linear_system_solve");
            const double forcing = std::min(1e-2, residual * std::min(0.5, std::sqrt(residual)));
            PcgState init{};
            init.abs_tol = std::max(forcing, S.cg_abs_tolerance);
            init.rel_tol = S.cg_rel_tolerance;
            init.max_iterations = S.cg_max_iterations;
            init.replace_every = std::is_same<T, float>::value ? S.cg_residual_replacement : 0;
            ck(cudaMemcpyAsync(I.pcg_state.p, &init, sizeof(PcgState), cudaMemcpyHostToDevice, s), "pcg state");
            symxg::launch_pcg_init<T>(B, I.grad.p, s);
            int launched = 0, chunk = 8;
            std::vector<std::pair<cudaEvent_t, cudaEvent_t>> spmv_ev;
            bool persistent = false;
            if constexpr (std::is_same<T, float>::value) persistent = B.staged.persistent != 0;
            if (persistent) {  // every iteration in one cooperative launch
                // With residual replacement the launch returns every replace_every iterations;
                // k_pcg_replace_residual forms the true residual and the next launch continues.
                // Each round is a launch pair that does nothing once the solve is done.
                const int every = init.replace_every;
                const int rounds = every > 0 ? 4 : 1;
                for (int round = 0;; round += rounds) {
                    cudaEvent_t a = nullptr, b = nullptr;
                    if (S.time_kernels) {
                        cudaEventCreate(&a);
                        cudaEventCreate(&b);
                        cudaEventRecord(a, s);
                    }
                    for (int k = 0; k < rounds; ++k) {
                        if constexpr (std::is_same<T, float>::value) {
                            symxg::launch_pcg_solve_persistent(B, s);
                            if (every > 0) symxg::launch_pcg_replace_residual(B, I.grad.p, s);
                        }
                    }
                    if (S.time_kernels) cudaEventRecord(b, s);
                    const int it_before = I.h_state->iteration;
                    ck(cudaMemcpyAsync(I.h_state, I.pcg_state.p, sizeof(PcgState), cudaMemcpyDeviceToHost, s),
                       "pcg state");
                    ck(cudaStreamSynchronize(s), "synchronize");
                    if (S.time_kernels) {
                        float ms = 0.f;
                        cudaEventElapsedTime(&ms, a, b);
                        auto& kt = st.kernels["pcg_solve_f32"];
                        kt.first += I.h_state->iteration - (round == 0 ? 0 : it_before);
                        kt.second += ms * 1e-3;
                        cudaEventDestroy(a);
                        cudaEventDestroy(b);
                    }
                    if (I.h_state->done || I.h_state->wait_failed || every <= 0 ||
                        I.h_state->iteration >= S.cg_max_iterations)
                        break;
                }
                st.cg_residual_replacements += I.h_state->replacements;
            }
            while (!persistent) {
                for (int k = 0; k < chunk; ++k) {
                    if (S.time_kernels) {
                        cudaEvent_t a, b;
                        cudaEventCreate(&a);
                        cudaEventCreate(&b);
                        cudaEventRecord(a, s);
                        symxg::launch_pcg_spmv<T>(B, launched + k, s);
                        cudaEventRecord(b, s);
                        spmv_ev.push_back({a, b});
                        symxg::launch_pcg_update<T>(B, launched + k, s);
                    } else {
                        symxg::launch_pcg_iteration<T>(B, launched + k, s);
                    }
                }
                launched += chunk;
                ck(cudaMemcpyAsync(I.h_state, I.pcg_state.p, sizeof(PcgState), cudaMemcpyDeviceToHost, s), "pcg state");
                ck(cudaStreamSynchronize(s), "synchronize");
                if (I.h_state->done || launched > S.cg_max_iterations + 1) break;
                chunk = std::min(chunk * 2, 64);
            }
            timer.stop();
            const PcgState ps = *I.h_state;
            if (ps.wait_failed) throw std::runtime_error("symx_gb300: a bounded wait in the PCG kernels gave up");
            if (S.time_kernels) {
                auto& kt = st.kernels[std::string("pcg_spmv_") + (sizeof(T) == 4 ? "f32" : "f64")];
                for (size_t k = 0; k < spmv_ev.size(); ++k) {
                    if ((int)k < ps.iteration) {  // launches after convergence returned at once
                        float ms = 0.f;
                        cudaEventElapsedTime(&ms, spmv_ev[k].first, spmv_ev[k].second);
                        kt.first += 1;
                        kt.second += ms * 1e-3;
                    }
                    cudaEventDestroy(spmv_ev[k].first);
                    cudaEventDestroy(spmv_ev[k].second);
                }
            }
            st.cg_iterations += ps.iteration;
            st.cg_iterations_per_newton.push_back(ps.iteration);
            if (verbosity > 0) std::printf("#CG: %4d | ", ps.iteration);
            const bool can_project_more = S.projection_mode != ProjectionToPD::Newton && !all_projected;
            if (!ps.converged && !can_project_more) {
                result = SolverReturn::LinearSystemSolveFailure;
                break;
            }
            bool descends = false;
            if (ps.converged) {
                symxg::launch_dot_rows4<T>(du, I.grad.p, I.n_blocks, I.partials.p, I.tickets.p + 4, I.scalars.p + 2, s);
                symxg::launch_max_abs_rows4<T>(du, I.n_blocks, I.partials.p, I.tickets.p + 4, I.scalars.p + 3, s);
                I.read_scalars(4);
                du_dot_grad = I.h_scalars[2];
                du_max = I.h_scalars[3];
                descends = du_dot_grad < 0.0;
                if (!descends && !can_project_more) {
                    result = SolverReturn::StepDoesNotDescend;
                    break;
                }
            }
            if (ps.converged && descends) break;
            // more projection, then retry
            if (S.projection_mode == ProjectionToPD::ProjectOnDemand) pdn_countdown = S.project_on_demand_countdown;
            if (S.projection_mode == ProjectionToPD::Progressive) {
                if (ppn_threshold < 0.0) ppn_threshold = residual;
                ppn_threshold *= S.ppn_tightening_factor;
                // a zero threshold cannot tighten (the reference would retry the same solve
                // forever): a threshold below 1e-12 projects every element on the next try
                if (ppn_threshold == 0.0) ppn_threshold = 1e-13;
            }
            if (verbosity > 0) std::printf("retrying with more projection | ");
        }
        if (result != SolverReturn::Running) break;
        st.n_hessians += (uint64_t)I.n_elements_total;
        st.n_projected_hessians += n_projected_it;
        if (S.projection_mode == ProjectionToPD::ProjectOnDemand) pdn_countdown--;
        if (S.projection_mode == ProjectionToPD::Progressive) ppn_threshold *= S.ppn_release_factor;
        if (verbosity > 0) std::printf("du: %.1e | ", du_max);
        if (it >= S.min_iterations && du_max < S.step_tolerance) {
            result = SolverReturn::Successful;
            break;
        }
        // line search: cap, then Armijo backtracking on the energy
        double retraction = 1.0;
        if (du_max > S.step_cap) {
            retraction *= S.step_cap / du_max;
            du_max = S.step_cap;
            st.ls_cap_iterations++;
        }
        timer.start("evaluate_P");
        ck(cudaMemcpyAsync(I.x_before.p, I.x.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "copy");
        double step = 1.0;
        symxg::launch_axpy_rows4<T>(I.n_blocks, I.x_before.p, step * retraction, du, I.x.p, s);
        if (S.enable_armijo_backtracking) {
            const double expected = S.line_search_armijo_beta * du_dot_grad * retraction;
            double E_thr = E0 + expected * step;
            int a = 0;
            for (; a < S.max_backtracking_armijo_iterations; ++a) {
                I.launch_eval(mode == 1 ? 3 : 2);  // the energy in the precision of the step's E and g
                symxg::launch_sum(I.E_el.p, I.n_elements_total, I.partials.p, I.tickets.p + 4, I.scalars.p, s);
                I.read_scalars(1);
                const double E1 = I.h_scalars[0];
                if (E1 < E_thr) break;
                step *= 0.5;
                symxg::launch_axpy_rows4<T>(I.n_blocks, I.x_before.p, step * retraction, du, I.x.p, s);
                E_thr = E0 + expected * step;
                st.ls_bt_iterations++;
            }
            if (verbosity > 0 && a > 0) std::printf("ls bt %2d | ", a);
            if (a == S.max_backtracking_armijo_iterations) {
                timer.stop();
                result = SolverReturn::TooManyArmijoIterations;
                break;
            }
        }
        timer.stop();
        if (verbosity > 0) std::printf("\n");
    }
    if (verbosity > 0) std::printf("\n");
    ck(cudaStreamSynchronize(s), "synchronize");
    int nc = 0;
    ck(cudaMemcpy(&nc, I.flags.p, sizeof(int), cudaMemcpyDeviceToHost), "flags");
    st.projection_not_converged = nc;
    timer.flush(st.timers);
    for (auto& pe : pending_kernel_events) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pe.a, pe.b);
        auto& kt = st.kernels[pe.name];
        kt.first += 1;
        kt.second += ms * 1e-3;
        cudaEventDestroy(pe.a);
        cudaEventDestroy(pe.b);
    }
    st.newton_iterations = it;
    st.final_residual = residual;
    st.final_energy = E0;
    if (st.n_hessians > 0) st.projected_hessians_ratio = (double)st.n_projected_hessians / (double)st.n_hessians;
    return result;
}

}  // namespace

// ---------------------------------------------------------------- adjoint
namespace {
// PCG on the Hessian already assembled in precision T (with its block-Jacobi set up).
template <typename T>
AdjointInfo adjoint_pcg_t(SolverImpl& I, const double* rhs, double* lambda, double rel_tol, int max_iterations)
{
    cudaStream_t s = I.stream;
    // the PCG initialisation takes -b
    std::vector<double> neg(rhs, rhs + I.n_dofs);
    for (double& v : neg) v = -v;
    ck(cudaMemcpyAsync(I.grad.p, neg.data(), sizeof(double) * I.n_dofs, cudaMemcpyHostToDevice, s), "upload rhs");
    DevBuf<T>* V = I.vecs<T>();
    PcgBuffers<T> B;
    B.n_blocks = I.n_blocks;
    B.row_ptr = I.row_ptr.p;
    B.cols = I.cols.p;
    B.vals = I.vals<T>();
    B.vals_stride = I.vstride;
    B.Dinv = I.Dinv<T>();
    B.x = V[0].p;
    B.r = V[1].p;
    B.z = V[2].p;
    B.p = V[3].p;
    B.q = V[4].p;
    B.p2 = V[5].p;
    B.partials = I.partials.p;
    B.tickets = I.tickets.p;
    B.state = I.pcg_state.p;
    if constexpr (std::is_same<T, float>::value) {
        B.staged = I.staged;
        B.la = I.staged.lookahead ? I.la32.p : nullptr;
    }
    PcgState init{};
    init.abs_tol = 0.0;
    init.rel_tol = rel_tol;
    init.max_iterations = max_iterations;
    ck(cudaMemcpyAsync(I.pcg_state.p, &init, sizeof(PcgState), cudaMemcpyHostToDevice, s), "pcg state");
    symxg::launch_pcg_init<T>(B, I.grad.p, s);
    bool done = false;
    if constexpr (std::is_same<T, float>::value) {
        if (B.staged.persistent) {
            symxg::launch_pcg_solve_persistent(B, s);
            done = true;
        }
    }
    for (int launched = 0, chunk = 8; !done;) {
        for (int k = 0; k < chunk; ++k) symxg::launch_pcg_iteration<T>(B, launched + k, s);
        launched += chunk;
        ck(cudaMemcpyAsync(I.h_state, I.pcg_state.p, sizeof(PcgState), cudaMemcpyDeviceToHost, s), "pcg state");
        ck(cudaStreamSynchronize(s), "synchronize");
        if (I.h_state->done || launched > max_iterations + 1) break;
        chunk = std::min(chunk * 2, 64);
    }
    ck(cudaMemcpyAsync(I.h_state, I.pcg_state.p, sizeof(PcgState), cudaMemcpyDeviceToHost, s), "pcg state");
    std::vector<T> x4(4 * (size_t)I.n_blocks);
    ck(cudaMemcpyAsync(x4.data(), V[0].p, sizeof(T) * x4.size(), cudaMemcpyDeviceToHost, s), "download solution");
    ck(cudaStreamSynchronize(s), "synchronize");
    const PcgState ps = *I.h_state;
    if (ps.wait_failed) throw std::runtime_error("symx_gb300: a bounded wait in the PCG kernels gave up");
    for (int64_t r = 0; r < I.n_blocks; ++r)
        for (int d = 0; d < 3; ++d) lambda[3 * r + d] = (double)x4[4 * r + d];
    AdjointInfo info;
    info.iterations = ps.iteration;
    info.converged = ps.converged != 0;
    info.error = ps.error;
    return info;
}
}  // namespace

AdjointInfo NewtonsMethod::adjoint_solve(const double* rhs, double* lambda, double rel_tol, int max_iterations,
                                         bool project)
{
    SolverImpl& I = *impl;
    cudaStream_t s = I.stream;
    if (settings.precision != Precision::Mixed) {
        assemble_t<double>(I, project, settings, 0);
        symxg::launch_block_jacobi_setup<double>(I.n_blocks, I.diag_slot.p, I.vals<double>(), I.vstride,
                                                 I.Dinv<double>(), s);
        return adjoint_pcg_t<double>(I, rhs, lambda, rel_tol, max_iterations);
    }
    // Mixed: FP32 Hessian and PCG inside defect correction.  Each pass solves
    // H32 d = b - H64 lambda (FP32 PCG to 1e-6, or rel_tol if looser), with the residual formed
    // from the FP64 Hessian, until |b - H64 lambda| / |b| < rel_tol.
    assemble_t<float>(I, project, settings, 1);
    symxg::launch_block_jacobi_setup<float>(I.n_blocks, I.diag_slot.p, I.vals<float>(), I.vstride, I.Dinv<float>(), s);
    assemble_t<double>(I, project, settings, 0);
    const size_t n = (size_t)I.n_dofs;
    double bb = 0.0;
    for (size_t i = 0; i < n; ++i) bb += rhs[i] * rhs[i];
    std::fill(lambda, lambda + n, 0.0);
    AdjointInfo total;
    if (bb == 0.0) {
        total.converged = true;
        return total;
    }
    std::vector<double> r(rhs, rhs + n), d(n), Hl(n);
    DevBuf<double> lam_dev, Hl_dev;
    lam_dev.alloc(n);
    Hl_dev.alloc(n);
    const double inner_tol = std::max(rel_tol, 1e-6);
    for (int pass = 0; pass < 12; ++pass) {
        const AdjointInfo inner = adjoint_pcg_t<float>(I, r.data(), d.data(), inner_tol, max_iterations);
        total.iterations += inner.iterations;
        if (!inner.converged && inner.iterations == 0) break;
        for (size_t i = 0; i < n; ++i) lambda[i] += d[i];
        ck(cudaMemcpyAsync(lam_dev.p, lambda, sizeof(double) * n, cudaMemcpyHostToDevice, s), "upload lambda");
        symxg::launch_bcsr_spmv<double>(I.n_blocks, I.row_ptr.p, I.cols.p, I.vals<double>(), I.vstride, lam_dev.p,
                                        Hl_dev.p, s);
        ck(cudaMemcpyAsync(Hl.data(), Hl_dev.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "download product");
        ck(cudaStreamSynchronize(s), "synchronize");
        double rr = 0.0;
        for (size_t i = 0; i < n; ++i) {
            r[i] = rhs[i] - Hl[i];
            rr += r[i] * r[i];
        }
        total.error = std::sqrt(rr / bb);
        if (total.error < rel_tol) {
            total.converged = true;
            break;
        }
    }
    return total;
}

void NewtonsMethod::parameter_gradient(std::uintptr_t param, const double* lambda, double* out, int64_t n_out)
{
    SolverImpl& I = *impl;
    GlobalPotential& GP = *global_potential;
    cudaStream_t s = I.stream;
    std::fill(out, out + n_out, 0.0);
    I.lambda.alloc((size_t)I.n_dofs);
    ck(cudaMemcpyAsync(I.lambda.p, lambda, sizeof(double) * I.n_dofs, cudaMemcpyHostToDevice, s), "upload lambda");
    bool bound = false;
    for (size_t p = 0; p < I.pots.size(); ++p) {
        CompiledPotential& cp = I.pots[p];
        const auto& maps = cp.pot->mws->maps;
        for (size_t k = 0; k < maps.size(); ++k) {
            const DataMap& m = maps[k];
            if (m.id != param) continue;
            bound = true;
            for (const auto& d : GP.dofs)
                if (d.id == param) throw std::invalid_argument("symx: parameter_gradient of a DoF container");
            if (cp.n_elements == 0) continue;
            auto key = std::make_pair((int)p, (int)k);
            auto it = I.mixed_modules.find(key);
            if (it == I.mixed_modules.end())
                it = I.mixed_modules.emplace(key, CudaModule::build(build_mixed_source(cp, GP, (int)k), I.cache_dir, {}, nullptr))
                         .first;
            // lambda through the DoF maps, nothing through the others
            std::vector<const double*> lp(maps.size(), nullptr);
            for (size_t j = 0; j < maps.size(); ++j)
                for (size_t set = 0; set < GP.dofs.size(); ++set)
                    if (GP.dofs[set].id == maps[j].id) lp[j] = I.lambda.p + I.dof_offsets[set];
            I.lmap_ptrs.alloc(std::max<size_t>(maps.size(), I.lmap_ptrs.n));
            ck(cudaMemcpyAsync(I.lmap_ptrs.p, lp.data(), sizeof(double*) * lp.size(), cudaMemcpyHostToDevice, s),
               "upload lambda maps");
            const size_t n_vals = (size_t)cp.n_elements * m.stride;
            if (I.mixed_out.n < n_vals) I.mixed_out.alloc(n_vals);
            long long n = cp.n_elements;
            const int32_t* conn = cp.conn.p;
            const double* const* mp = cp.map_ptrs.p;
            const double* const* lmp = I.lmap_ptrs.p;
            double* o = I.mixed_out.p;
            void* args[] = {&n, &conn, &mp, &lmp, &o};
            it->second->launch("symxg_mixed", dim3((unsigned)((n + 127) / 128)), dim3(128), 0, s, args);
            std::vector<double> vals(n_vals);
            ck(cudaMemcpyAsync(vals.data(), I.mixed_out.p, sizeof(double) * n_vals, cudaMemcpyDeviceToHost, s),
               "download mixed derivatives");
            ck(cudaStreamSynchronize(s), "synchronize");
            // element order, one fixed summation order per entry
            const int32_t* hconn = cp.pot->mws->conn.data();
            for (int64_t e = 0; e < cp.n_elements; ++e) {
                const int64_t item = m.conn_column >= 0 ? hconn[e * cp.conn_stride + m.conn_column] : 0;
                for (int j = 0; j < m.stride; ++j) {
                    const int64_t idx = item * m.stride + j;
                    if (idx < 0 || idx >= n_out) throw std::invalid_argument("symx: parameter_gradient output too small");
                    out[idx] -= vals[(size_t)e * m.stride + j];
                }
            }
        }
    }
    if (!bound) throw std::invalid_argument("symx: the parameter container is not bound in any potential");
}

SolverReturn NewtonsMethod::solve_device()
{
    stats = SolveStats();
    stats.h2d_bytes = h2d_bytes_;
    stats.d2h_bytes = d2h_bytes_;
    if (settings.precision == Precision::Mixed) return solve_t<float>(*impl, settings, stats, context->verbosity);
    return solve_t<double>(*impl, settings, stats, context->verbosity);
}

}  // namespace symx
