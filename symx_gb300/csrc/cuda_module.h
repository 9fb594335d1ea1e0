// Run-time compilation of generated CUDA source with NVRTC, straight to a CUBIN for
// sm_103a, cached on disk by a hash of (source, options, NVRTC version, arch), and
// loaded through the driver API.  This replaces the reference's "write C++, run the
// system compiler, dlopen the .so, check its SHA-256" loop
// (symx/src/compile/Compilation.cpp:59-226).
//
// Driver entry points are resolved through the CUDA runtime at first use, so the
// library itself loads on a machine without a GPU driver.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

namespace symxg {

struct CompileInfo {
    bool cached = false;
    double seconds = 0.0;
    std::string cache_file;
    std::string log;
};

class CudaModule {
public:
    // Compile (or load from `cache_dir`) and load into the current device's primary context.
    // Throws std::runtime_error with the NVRTC log on failure.
    static std::shared_ptr<CudaModule> build(const std::string& source, const std::string& cache_dir,
                                             const std::vector<std::string>& extra_options, CompileInfo* info = nullptr);
    // Load an already compiled CUBIN image into the current device's primary context.
    static std::shared_ptr<CudaModule> load(const std::string& cubin);
    ~CudaModule();
    // Launch `kernel` with `args` (pointers to each argument, as cuLaunchKernel takes them).
    void launch(const std::string& kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t stream, void** args);
    int max_threads_per_block(const std::string& kernel);

private:
    void* module_ = nullptr;  // CUmodule
    std::unordered_map<std::string, void*> functions_;
    void* function(const std::string& name);
};

// NVRTC compilation of `source` to a CUBIN for sm_103a (no GPU needed).  Throws with the
// NVRTC log on failure.
std::string compile_cubin(const std::string& source, const std::vector<std::string>& extra_options,
                          std::string* log = nullptr);

// Cache directory: $SYMXG_CACHE_DIR, else <package>/_build/kernel_cache.
std::string default_cache_dir();
// FNV-1a 64-bit over a byte string, hex encoded.
std::string hash_hex(const std::string& data);
int nvrtc_version();

}  // namespace symxg
