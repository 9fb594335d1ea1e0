// Compiled<T>: a list of expressions compiled to a GPU kernel and evaluated on demand,
// with the interface of the reference's entry-level compiled function
// (symx/src/compile/Compiled.h:26-96, Compilation.h:21-80, View.h:8-40).
//
// The reference writes C++ for `void f(FLOAT* in, FLOAT* out)`, compiles it with the system
// compiler into <folder>/<name>.so and calls it on the host.  Here the same expression list
// becomes a CUDA kernel (codegen.h: in[i] = symbol i, out[k] = k-th expression) compiled by
// NVRTC for sm_103a into <folder>/<name>.cubin, with its cache identity in
// <folder>/<name>.symxg.  One input set per thread:
//   * run() / run(thread_id) evaluate one host-side input set (one kernel launch and two
//     copies; a correctness and debugging tool, as in the reference);
//   * run_all() evaluates every configured input set in one launch (the batch the
//     reference gets from its SIMD types __m256d / __m256, which have no GPU meaning);
//   * run_device() evaluates a batch that already lives in device memory, on a stream.
// Supported types: double and float.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "symbolic.h"

struct CUstream_st;

namespace symxg {
class CudaModule;
}

namespace symx {

// Non-owning view over a contiguous host array (reference: symx/src/compile/View.h).
template <typename T>
class View {
public:
    View(T* data, int32_t size) : data_(data), size_(size) {}
    int32_t size() const { return size_; }
    T* data() { return data_; }
    const T* data() const { return data_; }
    T& operator[](int32_t i) { return data_[i]; }
    const T& operator[](int32_t i) const { return data_[i]; }
    View slice(int32_t begin, int32_t end) const { return View(data_ + begin, end - begin); }
    View slice(int32_t begin) const { return View(data_ + begin, size_ - begin); }

private:
    T* data_;
    int32_t size_;
};

// Element type of a compilation (reference: symx/src/compile/type_utils.h:36-43).
enum class FloatType { Double, Float };

// Global switches (reference: symx/src/compile/static_methods.cpp:13-50).
// Check mode: Compiled<T>::run checks every input and output for NaN and throws.  Off by default.
void check_mode_ON(bool check = true);
bool get_check_mode_ON();
// With loading disabled every Compiled<T> is compiled afresh, ignoring the files on disk.
void enable_load_compiled(bool enable = true);
bool is_load_compiled_enabled();
// Folder for generated code: $SYMX_CODEGEN_DIR, else `codegen` beside the kernel cache;
// created if missing.
std::string get_codegen_dir();
// Reproducible hash of the part of the graph that `exprs` depend on (hex string).
std::string get_checksum(const std::vector<Scalar>& exprs);

// One compiled expression list on the GPU (reference: symx/src/compile/Compilation.h).
class Compilation {
public:
    struct Info {
        int n_inputs = -1;
        int n_outputs = -1;
        FloatType compiled_type = FloatType::Double;
        bool was_cached = false;
        double runtime_codegen = 0.0;
        double runtime_compilation = 0.0;
        int n_bytes_symbols = 0;
        void print() const;
    };

    Compilation() = default;
    Compilation(const Compilation&) = delete;
    Compilation& operator=(const Compilation&) = delete;

    // Load <folder>/<name>.cubin if <folder>/<name>.symxg records `cache_id` for this type
    // and compiler; false otherwise.  Throws std::invalid_argument for an empty cache_id and
    // std::runtime_error if a matching image does not load (no CUDA device, corrupt file).
    bool load_if_cached(const std::string& name, const std::string& folder, const std::string& cache_id,
                        FloatType type);
    // Generate, compile with NVRTC and load.  An empty cache_id is replaced by the checksum of
    // `expr`.  Throws std::runtime_error with the NVRTC log if compilation fails.
    void compile(const std::vector<Scalar>& expr, const std::string& name, const std::string& folder,
                 const std::string& cache_id, FloatType type);
    void try_load_otherwise_compile(const std::vector<Scalar>& expr, const std::string& name,
                                    const std::string& folder, const std::string& cache_id, FloatType type);

    bool is_valid() const { return module_ != nullptr; }
    int get_n_inputs() const { return n_inputs_; }
    int get_n_outputs() const { return n_outputs_; }
    FloatType get_compiled_type() const { return type_; }
    bool was_cached() const { return cached_; }
    Info get_info() const;

    // Evaluate `n` input sets in device memory: symbol i of set t is read at
    // in[t * in_item + i * in_symbol], output k of set t written to out[t * out_item + k * out_symbol].
    void launch(const void* in, void* out, int64_t n, int64_t in_item, int64_t in_symbol, int64_t out_item,
                int64_t out_symbol, CUstream_st* stream) const;

private:
    std::shared_ptr<symxg::CudaModule> module_;
    int n_inputs_ = -1;
    int n_outputs_ = -1;
    FloatType type_ = FloatType::Double;
    bool cached_ = false;
    bool override_load_ = false;
    double runtime_codegen_ = 0.0;
    double runtime_compilation_ = 0.0;
    int n_bytes_symbols_ = 0;
};

template <typename FLOAT>
class Compiled {
    static_assert(std::is_same<FLOAT, double>::value || std::is_same<FLOAT, float>::value,
                  "Compiled<T> supports double and float");

public:
    std::vector<std::vector<FLOAT>> thread_input;   // per-thread input sets (host)
    std::vector<std::vector<FLOAT>> thread_output;  // per-thread outputs (host)
    std::string name;

    Compiled() = default;
    ~Compiled();
    Compiled(const Compiled&) = delete;
    Compiled& operator=(const Compiled&) = delete;
    Compiled(const std::vector<Scalar>& expr, const std::string& name, const std::string& folder,
             const std::string& cache_id = "");

    void compile(const std::vector<Scalar>& expr, const std::string& name, const std::string& folder,
                 const std::string& cache_id = "");
    bool load_if_cached(const std::string& name, const std::string& folder, const std::string& cache_id);
    void try_load_otherwise_compile(const std::vector<Scalar>& expr, const std::string& name, const std::string& folder,
                                    const std::string& cache_id = "");

    bool is_valid() const { return compilation_.is_valid(); }
    bool was_cached() const { return compilation_.was_cached(); }
    Compilation::Info get_compilation_info() const { return compilation_.get_info(); }

    // Number of independent input sets.  Throws std::invalid_argument for n_threads < 1.
    void set_n_threads(int n_threads);
    int get_n_threads() const { return n_threads_; }

    void set(const Scalar& scalar, const FLOAT& v) { set(scalar, v, 0); }
    void set(const Scalar& scalar, const FLOAT& v, int thread_id);
    template <typename IndexableVector>
    void set(const Vector& vector, const IndexableVector& v) { set(vector, v, 0); }
    template <typename IndexableVector>
    void set(const Vector& vector, const IndexableVector& v, int thread_id)
    {
        for (int32_t i = 0; i < vector.size(); ++i) set(vector[i], v[i], thread_id);
    }
    void set(const Matrix& matrix, const FLOAT* v) { set(matrix, v, 0); }
    void set(const Matrix& matrix, const FLOAT* v, int thread_id);
    template <typename RowMajorMatrix>
    typename std::enable_if<!std::is_pointer<RowMajorMatrix>::value, void>::type set(const Matrix& matrix,
                                                                                    const RowMajorMatrix& m)
    {
        set(matrix, m, 0);
    }
    template <typename RowMajorMatrix>
    typename std::enable_if<!std::is_pointer<RowMajorMatrix>::value, void>::type set(const Matrix& matrix,
                                                                                    const RowMajorMatrix& m,
                                                                                    int thread_id)
    {
        for (int32_t i = 0; i < matrix.rows(); ++i)
            for (int32_t j = 0; j < matrix.cols(); ++j) set(matrix(i, j), m(i, j), thread_id);
    }

    // Evaluate input set `thread_id` on the GPU; the view points into thread_output[thread_id].
    // Throws std::runtime_error for an invalid compilation, and in check mode for a NaN input
    // or output.  Different host threads may run different thread ids concurrently (each host
    // thread uses its own default stream).
    View<FLOAT> run() { return run(0); }
    View<FLOAT> run(int thread_id);
    // Evaluate all get_n_threads() input sets in one launch into thread_output.
    void run_all();
    // Evaluate `n` input sets already in device memory (layout as Compilation::launch), on
    // `stream` (nullptr: the legacy default stream).  Asynchronous; no check mode.
    void run_device(const FLOAT* in, FLOAT* out, int64_t n, int64_t in_item, int64_t in_symbol, int64_t out_item,
                    int64_t out_symbol, CUstream_st* stream = nullptr) const;

    int get_n_inputs() const { return compilation_.get_n_inputs(); }
    int get_n_outputs() const { return compilation_.get_n_outputs(); }
    std::string get_name() const { return name; }

    FLOAT* get_input_buffer(int thread_id = 0) { return thread_input[thread_id].data(); }
    FLOAT* get_output_buffer(int thread_id = 0) { return thread_output[thread_id].data(); }
    const FLOAT* get_input_buffer(int thread_id = 0) const { return thread_input[thread_id].data(); }
    const FLOAT* get_output_buffer(int thread_id = 0) const { return thread_output[thread_id].data(); }

private:
    Compilation compilation_;
    int n_threads_ = 1;
    FLOAT* d_in_ = nullptr;   // device copy of every input set, thread-major
    FLOAT* d_out_ = nullptr;  // device outputs, thread-major
    int64_t d_capacity_in_ = 0, d_capacity_out_ = 0;

    void resize_buffers();
    void check_nan(const std::vector<FLOAT>& v, const char* what) const;
    void check_thread(int thread_id) const;
};

}  // namespace symx
