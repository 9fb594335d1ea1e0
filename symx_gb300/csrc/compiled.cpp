// GPU Compiled<T> (compiled.h).  Follows the reference's compile / load-if-cached /
// run flow (symx/src/compile/Compilation.cpp:59-226, Compiled.cpp:1-200) with NVRTC and a
// CUBIN in place of the system compiler and a shared object.
#include "compiled.h"
#include "kernels.cuh"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>
#include <unistd.h>

#include <cuda_runtime.h>

#include "codegen.h"
#include "cuda_module.h"

namespace symx {

namespace {

bool g_check_mode = false;
bool g_load_compiled = true;

constexpr int kThreads = 128;
const char* kKernel = "symxg_compiled";

std::string type_name(FloatType t) { return t == FloatType::Double ? "double" : "float"; }

// Cache identity of a compilation: the user's id, the element type, the NVRTC version and
// the target (the reference hashes id + type into the shared object, Compilation.cpp:186-190).
std::string cache_key(const std::string& cache_id, FloatType t)
{
    return symxg::hash_hex(cache_id + "|" + type_name(t) + "|nvrtc" + std::to_string(symxg::nvrtc_version()) +
                           "|sm_103a");
}

bool read_all(const std::string& path, std::string& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

void write_atomic(const std::string& path, const std::string& data)
{
    const std::string tmp = path + ".tmp." + std::to_string(getpid());
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f) throw std::runtime_error("symx: cannot write " + tmp);
        f.write(data.data(), (std::streamsize)data.size());
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) throw std::runtime_error("symx: cannot write " + path);
}

void make_dirs(const std::string& path)
{
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' || i + 1 == path.size()) mkdir(cur.c_str(), 0755);
    }
}

void check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("symx: ") + what + ": " + cudaGetErrorString(e));
}

// Kernel source: the expression list as a device function plus a batch wrapper that gathers
// one input set per thread (strided, so both thread-major host sets and symbol-major device
// batches are read directly) and scatters its outputs.
std::string kernel_source(const std::vector<Scalar>& expr, FloatType t, int n_inputs)
{
    const Expressions& g = *expr[0].graph;
    std::vector<int32_t> roots;
    for (const Scalar& s : expr) roots.push_back(s.expr_id);
    const std::string T = type_name(t);
    const int n_outputs = (int)expr.size();
    std::ostringstream src;
    src << codegen_prelude();
    src << emit_device_function(g, roots, "symxg_compiled_f", T, false);
    src << "extern \"C\" __global__ void __launch_bounds__(" << kThreads << ") " << kKernel << "(const " << T
        << "* __restrict__ in, " << T << "* __restrict__ out, long long n, long long in_item, long long in_symbol, "
        << "long long out_item, long long out_symbol)\n{\n"
        << "    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;\n"
        << "    if (t >= n) return;\n"
        << "    " << T << " x[" << std::max(n_inputs, 1) << "];\n"
        << "    " << T << " y[" << n_outputs << "];\n"
        << "#pragma unroll\n"
        << "    for (int i = 0; i < " << n_inputs << "; ++i) x[i] = in[t * in_item + i * in_symbol];\n"
        << "    symxg_compiled_f(x, nullptr, y);\n"
        << "#pragma unroll\n"
        << "    for (int k = 0; k < " << n_outputs << "; ++k) out[t * out_item + k * out_symbol] = y[k];\n"
        << "}\n";
    return src.str();
}

}  // namespace

void check_mode_ON(bool check) { g_check_mode = check; }
bool get_check_mode_ON() { return g_check_mode; }
void enable_load_compiled(bool enable) { g_load_compiled = enable; }
bool is_load_compiled_enabled() { return g_load_compiled; }

std::string get_codegen_dir()
{
    std::string dir;
    if (const char* env = std::getenv("SYMX_CODEGEN_DIR"))
        dir = env;
    else
        dir = symxg::default_cache_dir() + "/codegen";
    make_dirs(dir);
    struct stat st;
    if (stat(dir.c_str(), &st) != 0 || !S_ISDIR(st.st_mode))
        throw std::runtime_error("symx: cannot create the codegen folder '" + dir + "'");
    return dir;
}

std::string get_checksum(const std::vector<Scalar>& exprs)
{
    if (exprs.empty()) return symxg::hash_hex("");
    std::vector<int32_t> roots;
    for (const Scalar& s : exprs) roots.push_back(s.expr_id);
    char buf[17];
    std::snprintf(buf, sizeof(buf), "%016llx", (unsigned long long)exprs[0].graph->hash(roots));
    return buf;
}

// ------------------------------------------------------------------ Compilation
void Compilation::Info::print() const
{
    std::printf("Compilation info: %d inputs, %d outputs, %s, %s, codegen %.3f s, compilation %.3f s, %d bytes of "
                "symbols\n",
                n_inputs, n_outputs, type_name(compiled_type).c_str(), was_cached ? "loaded from cache" : "compiled",
                runtime_codegen, runtime_compilation, n_bytes_symbols);
}

Compilation::Info Compilation::get_info() const
{
    Info i;
    i.n_inputs = n_inputs_;
    i.n_outputs = n_outputs_;
    i.compiled_type = type_;
    i.was_cached = cached_;
    i.runtime_codegen = runtime_codegen_;
    i.runtime_compilation = runtime_compilation_;
    i.n_bytes_symbols = n_bytes_symbols_;
    return i;
}

bool Compilation::load_if_cached(const std::string& name, const std::string& folder, const std::string& cache_id,
                                 FloatType type)
{
    if (!override_load_ && !is_load_compiled_enabled()) return false;
    if (cache_id.empty()) throw std::invalid_argument("symx: Compilation::load_if_cached cannot load with cache_id = \"\"");
    const std::string base = folder + "/" + name;
    std::string meta;
    if (!read_all(base + ".symxg", meta)) return false;
    std::istringstream ms(meta);
    std::string magic, key;
    int n_in = -1, n_out = -1, t = -1;
    ms >> magic >> key >> n_in >> n_out >> t;
    if (!ms || magic != "symxg-compiled-1" || key != cache_key(cache_id, type) || t != (int)type) {
        cached_ = false;
        return false;
    }
    std::string cubin;
    if (!read_all(base + ".cubin", cubin) || cubin.empty()) return false;
    try {
        module_ = symxg::CudaModule::load(cubin);
    } catch (const std::exception& e) {
        module_.reset();
        throw std::runtime_error("symx: failed to load the compiled kernel of '" + name + "' (" + base +
                                 ".cubin, cache id matched): " + e.what());
    }
    n_inputs_ = n_in;
    n_outputs_ = n_out;
    type_ = type;
    cached_ = true;
    return true;
}

void Compilation::compile(const std::vector<Scalar>& expr, const std::string& name, const std::string& folder,
                          const std::string& cache_id, FloatType type)
{
    if (expr.empty()) throw std::invalid_argument("symx: Compilation::compile of an empty expression list");
    for (const Scalar& s : expr)
        if (s.graph != expr[0].graph || s.expr_id < 0)
            throw std::invalid_argument("symx: Compilation::compile: expressions from different workspaces");
    const std::string id = cache_id.empty() ? get_checksum(expr) : cache_id;
    const int n_inputs = expr[0].graph->n_symbols();
    const int n_outputs = (int)expr.size();

    auto t0 = std::chrono::steady_clock::now();
    const std::string src = kernel_source(expr, type, n_inputs);
    auto t1 = std::chrono::steady_clock::now();
    runtime_codegen_ = std::chrono::duration<double>(t1 - t0).count();

    make_dirs(folder);
    const std::string base = folder + "/" + name;
    write_atomic(base + ".cu", src);
    std::string log;
    const std::string cubin = symxg::compile_cubin(src, {}, &log);
    write_atomic(base + ".cubin", cubin);
    std::ostringstream meta;
    meta << "symxg-compiled-1\n" << cache_key(id, type) << "\n" << n_inputs << "\n" << n_outputs << "\n" << (int)type << "\n";
    write_atomic(base + ".symxg", meta.str());
    t0 = std::chrono::steady_clock::now();
    runtime_compilation_ = std::chrono::duration<double>(t0 - t1).count();
    n_bytes_symbols_ = (int)(expr[0].graph->size() * sizeof(Node));

    // the fresh image must load, whatever the global load switch says
    override_load_ = true;
    bool ok = false;
    try {
        ok = load_if_cached(name, folder, id, type);
    } catch (...) {
        override_load_ = false;
        throw;
    }
    override_load_ = false;
    cached_ = false;
    if (!ok) throw std::runtime_error("symx: failed to reload the freshly compiled kernel of '" + name + "'");
}

void Compilation::try_load_otherwise_compile(const std::vector<Scalar>& expr, const std::string& name,
                                             const std::string& folder, const std::string& cache_id, FloatType type)
{
    const std::string id = cache_id.empty() ? get_checksum(expr) : cache_id;
    if (is_load_compiled_enabled() && load_if_cached(name, folder, id, type)) return;
    compile(expr, name, folder, id, type);
}

void Compilation::launch(const void* in, void* out, int64_t n, int64_t in_item, int64_t in_symbol, int64_t out_item,
                         int64_t out_symbol, CUstream_st* stream) const
{
    if (!module_) throw std::runtime_error("symx: launch of an invalid compilation");
    if (n <= 0) return;
    long long a_n = n, a_ii = in_item, a_is = in_symbol, a_oi = out_item, a_os = out_symbol;
    const void* a_in = in;
    void* a_out = out;
    void* args[] = {&a_in, &a_out, &a_n, &a_ii, &a_is, &a_oi, &a_os};
    const int64_t blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 0x7fffffff) throw std::invalid_argument("symx: batch too large for one launch");
    module_->launch(kKernel, dim3((unsigned)blocks), dim3(kThreads), 0, stream, args);
}

// ------------------------------------------------------------------ Compiled<T>
template <typename FLOAT>
static constexpr FloatType float_type_of()
{
    return std::is_same<FLOAT, double>::value ? FloatType::Double : FloatType::Float;
}

template <typename FLOAT>
Compiled<FLOAT>::Compiled(const std::vector<Scalar>& expr, const std::string& name, const std::string& folder,
                          const std::string& cache_id)
{
    try_load_otherwise_compile(expr, name, folder, cache_id);
}

template <typename FLOAT>
Compiled<FLOAT>::~Compiled()
{
    // errors are ignored here: the context may already be gone at process exit
    if (d_in_) {
        cudaFree(d_in_);
        symxg::note_device_free((int64_t)sizeof(FLOAT) * d_capacity_in_);
    }
    if (d_out_) {
        cudaFree(d_out_);
        symxg::note_device_free((int64_t)sizeof(FLOAT) * d_capacity_out_);
    }
}

template <typename FLOAT>
void Compiled<FLOAT>::compile(const std::vector<Scalar>& expr, const std::string& name_, const std::string& folder,
                              const std::string& cache_id)
{
    name = name_;
    compilation_.compile(expr, name_, folder, cache_id, float_type_of<FLOAT>());
    resize_buffers();
}

template <typename FLOAT>
bool Compiled<FLOAT>::load_if_cached(const std::string& name_, const std::string& folder, const std::string& cache_id)
{
    const bool ok = compilation_.load_if_cached(name_, folder, cache_id, float_type_of<FLOAT>());
    if (ok) {
        name = name_;
        resize_buffers();
    }
    return ok;
}

template <typename FLOAT>
void Compiled<FLOAT>::try_load_otherwise_compile(const std::vector<Scalar>& expr, const std::string& name_,
                                                 const std::string& folder, const std::string& cache_id)
{
    name = name_;
    compilation_.try_load_otherwise_compile(expr, name_, folder, cache_id, float_type_of<FLOAT>());
    resize_buffers();
}

template <typename FLOAT>
void Compiled<FLOAT>::set_n_threads(int n_threads)
{
    if (n_threads < 1) throw std::invalid_argument("symx: Compiled::set_n_threads needs a positive count");
    n_threads_ = n_threads;
    resize_buffers();
}

template <typename FLOAT>
void Compiled<FLOAT>::resize_buffers()
{
    const int n_in = std::max(get_n_inputs(), 0), n_out = std::max(get_n_outputs(), 0);
    thread_input.resize(n_threads_);
    thread_output.resize(n_threads_);
    for (int t = 0; t < n_threads_; ++t) {
        thread_input[t].resize(n_in, FLOAT(0));
        thread_output[t].resize(n_out, FLOAT(0));
    }
    if (!is_valid()) return;
    const int64_t need_in = (int64_t)n_threads_ * std::max(n_in, 1), need_out = (int64_t)n_threads_ * std::max(n_out, 1);
    if (need_in > d_capacity_in_) {
        if (d_in_) {
            cudaFree(d_in_);
            symxg::note_device_free((int64_t)sizeof(FLOAT) * d_capacity_in_);
        }
        d_in_ = nullptr;
        d_capacity_in_ = 0;
        check_cuda(cudaMalloc(&d_in_, sizeof(FLOAT) * need_in), "cudaMalloc of Compiled inputs");
        symxg::note_device_alloc((int64_t)sizeof(FLOAT) * need_in);
        d_capacity_in_ = need_in;
    }
    if (need_out > d_capacity_out_) {
        if (d_out_) {
            cudaFree(d_out_);
            symxg::note_device_free((int64_t)sizeof(FLOAT) * d_capacity_out_);
        }
        d_out_ = nullptr;
        d_capacity_out_ = 0;
        check_cuda(cudaMalloc(&d_out_, sizeof(FLOAT) * need_out), "cudaMalloc of Compiled outputs");
        symxg::note_device_alloc((int64_t)sizeof(FLOAT) * need_out);
        d_capacity_out_ = need_out;
    }
}

template <typename FLOAT>
void Compiled<FLOAT>::check_thread(int thread_id) const
{
    if (thread_id < 0 || thread_id >= n_threads_)
        throw std::out_of_range("symx: Compiled thread id " + std::to_string(thread_id) + " out of range for '" + name +
                                "'");
}

template <typename FLOAT>
void Compiled<FLOAT>::set(const Scalar& scalar, const FLOAT& v, int thread_id)
{
    check_thread(thread_id);
    if (!scalar.is_symbol()) throw std::invalid_argument("symx: Compiled::set of a non-symbol");
    const int32_t slot = scalar.get_symbol_idx();
    if (slot < 0 || slot >= (int32_t)thread_input[thread_id].size())
        throw std::out_of_range("symx: symbol created after the compilation of '" + name + "'");
    thread_input[thread_id][slot] = v;
}

template <typename FLOAT>
void Compiled<FLOAT>::set(const Matrix& matrix, const FLOAT* v, int thread_id)
{
    for (int32_t i = 0; i < matrix.rows(); ++i)
        for (int32_t j = 0; j < matrix.cols(); ++j) set(matrix(i, j), v[i * matrix.cols() + j], thread_id);
}

template <typename FLOAT>
void Compiled<FLOAT>::check_nan(const std::vector<FLOAT>& v, const char* what) const
{
    for (size_t i = 0; i < v.size(); ++i)
        if (std::isnan(v[i]))
            throw std::runtime_error("NaN detected in " + std::string(what) + " #" + std::to_string(i) +
                                     " of (compiled function '" + name + "')");
}

template <typename FLOAT>
View<FLOAT> Compiled<FLOAT>::run(int thread_id)
{
    check_thread(thread_id);
    if (!is_valid()) throw std::runtime_error("Cannot run invalid compilation for '" + name + "'");
    std::vector<FLOAT>& in = thread_input[thread_id];
    std::vector<FLOAT>& out = thread_output[thread_id];
    if (get_check_mode_ON()) check_nan(in, "input");
    const int64_t n_in = get_n_inputs(), n_out = get_n_outputs();
    FLOAT* d_in = d_in_ + (int64_t)thread_id * std::max<int64_t>(n_in, 1);
    FLOAT* d_out = d_out_ + (int64_t)thread_id * std::max<int64_t>(n_out, 1);
    cudaStream_t s = cudaStreamPerThread;
    if (n_in > 0) check_cuda(cudaMemcpyAsync(d_in, in.data(), sizeof(FLOAT) * n_in, cudaMemcpyHostToDevice, s), "input copy");
    compilation_.launch(d_in, d_out, 1, n_in, 1, n_out, 1, s);
    check_cuda(cudaMemcpyAsync(out.data(), d_out, sizeof(FLOAT) * n_out, cudaMemcpyDeviceToHost, s), "output copy");
    check_cuda(cudaStreamSynchronize(s), "Compiled::run");
    if (get_check_mode_ON()) check_nan(out, "output");
    return View<FLOAT>(out.data(), (int32_t)out.size());
}

template <typename FLOAT>
void Compiled<FLOAT>::run_all()
{
    if (!is_valid()) throw std::runtime_error("Cannot run invalid compilation for '" + name + "'");
    const int64_t n_in = get_n_inputs(), n_out = get_n_outputs();
    const int64_t ld_in = std::max<int64_t>(n_in, 1), ld_out = std::max<int64_t>(n_out, 1);
    if (get_check_mode_ON())
        for (const auto& v : thread_input) check_nan(v, "input");
    std::vector<FLOAT> host_in((size_t)(ld_in * n_threads_)), host_out((size_t)(ld_out * n_threads_));
    for (int t = 0; t < n_threads_; ++t)
        std::copy(thread_input[t].begin(), thread_input[t].end(), host_in.begin() + t * ld_in);
    cudaStream_t s = cudaStreamPerThread;
    check_cuda(cudaMemcpyAsync(d_in_, host_in.data(), sizeof(FLOAT) * host_in.size(), cudaMemcpyHostToDevice, s),
               "input copy");
    compilation_.launch(d_in_, d_out_, n_threads_, ld_in, 1, ld_out, 1, s);
    check_cuda(cudaMemcpyAsync(host_out.data(), d_out_, sizeof(FLOAT) * host_out.size(), cudaMemcpyDeviceToHost, s),
               "output copy");
    check_cuda(cudaStreamSynchronize(s), "Compiled::run_all");
    for (int t = 0; t < n_threads_; ++t)
        std::copy(host_out.begin() + t * ld_out, host_out.begin() + t * ld_out + n_out, thread_output[t].begin());
    if (get_check_mode_ON())
        for (const auto& v : thread_output) check_nan(v, "output");
}

template <typename FLOAT>
void Compiled<FLOAT>::run_device(const FLOAT* in, FLOAT* out, int64_t n, int64_t in_item, int64_t in_symbol,
                                 int64_t out_item, int64_t out_symbol, CUstream_st* stream) const
{
    if (!is_valid()) throw std::runtime_error("Cannot run invalid compilation for '" + name + "'");
    compilation_.launch(in, out, n, in_item, in_symbol, out_item, out_symbol, stream);
}

template class Compiled<double>;
template class Compiled<float>;

}  // namespace symx
