#include "cuda_module.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>
#include <unistd.h>

#include <dlfcn.h>
#include <nvrtc.h>

#include "kernels.cuh"

namespace symxg {

namespace {

// Minimal driver API surface, resolved via cudaGetDriverEntryPointByVersion.
using CUresult = int;
using cuModuleLoadData_t = CUresult (*)(void** module, const void* image);
using cuModuleUnload_t = CUresult (*)(void* module);
using cuModuleGetFunction_t = CUresult (*)(void** fn, void* module, const char* name);
using cuLaunchKernel_t = CUresult (*)(void* f, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by,
                                      unsigned bz, unsigned smem, cudaStream_t stream, void** params, void** extra);
using cuFuncGetAttribute_t = CUresult (*)(int* pi, int attrib, void* fn);
using cuFuncSetAttribute_t = CUresult (*)(void* fn, int attrib, int value);

struct Driver {
    cuModuleLoadData_t load = nullptr;
    cuModuleUnload_t unload = nullptr;
    cuModuleGetFunction_t get_function = nullptr;
    cuLaunchKernel_t launch = nullptr;
    cuFuncGetAttribute_t get_attr = nullptr;
    cuFuncSetAttribute_t set_attr = nullptr;
};

template <typename F>
void resolve(const char* name, F& f)
{
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
        throw std::runtime_error(std::string("symx_gb300: cannot resolve driver entry point ") + name);
    f = reinterpret_cast<F>(p);
}

const Driver& driver()
{
    static Driver d;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFree(nullptr);  // make the primary context current
        resolve("cuModuleLoadData", d.load);
        resolve("cuModuleUnload", d.unload);
        resolve("cuModuleGetFunction", d.get_function);
        resolve("cuLaunchKernel", d.launch);
        resolve("cuFuncGetAttribute", d.get_attr);
        resolve("cuFuncSetAttribute", d.set_attr);
    });
    return d;
}

void check_drv(CUresult r, const char* what)
{
    if (r != 0) {
        char buf[160];
        std::snprintf(buf, sizeof(buf), "symx_gb300: driver call %s failed with CUresult %d", what, r);
        throw std::runtime_error(buf);
    }
}

bool read_file(const std::string& path, std::string& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return !out.empty();
}

void mkdirs(const std::string& path)
{
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' || i + 1 == path.size()) mkdir(cur.c_str(), 0755);
    }
}

}  // namespace

std::string hash_hex(const std::string& data)
{
    uint64_t h = 1469598103934665603ull;
    for (unsigned char c : data) { h ^= c; h *= 1099511628211ull; }
    char buf[17];
    std::snprintf(buf, sizeof(buf), "%016llx", (unsigned long long)h);
    return buf;
}

int nvrtc_version()
{
    int major = 0, minor = 0;
    nvrtcVersion(&major, &minor);
    return major * 100 + minor;
}

std::string default_cache_dir()
{
    if (const char* env = std::getenv("SYMXG_CACHE_DIR")) return env;
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&default_cache_dir), &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        const size_t slash = so.rfind('/');
        if (slash != std::string::npos) return so.substr(0, slash) + "/kernel_cache";
    }
    return "/tmp/symx_gb300_kernel_cache";
}

static std::vector<std::string> base_options()
{
    return {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device"};
}

std::string compile_cubin(const std::string& source, const std::vector<std::string>& extra_options, std::string* log_out)
{
    std::vector<std::string> opts = base_options();
    opts.insert(opts.end(), extra_options.begin(), extra_options.end());
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source.c_str(), "symxg_generated.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        throw std::runtime_error("symx_gb300: nvrtcCreateProgram failed");
    std::vector<const char*> copts;
    for (const auto& o : opts) copts.push_back(o.c_str());
    const nvrtcResult r = nvrtcCompileProgram(prog, (int)copts.size(), copts.data());
    size_t log_size = 0;
    nvrtcGetProgramLogSize(prog, &log_size);
    std::string log(log_size, '\0');
    if (log_size) nvrtcGetProgramLog(prog, &log[0]);
    if (log_out) *log_out = log;
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        throw std::runtime_error("symx_gb300: NVRTC compilation failed:\n" + log);
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    std::string cubin(n, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    return cubin;
}

std::shared_ptr<CudaModule> CudaModule::build(const std::string& source, const std::string& cache_dir,
                                              const std::vector<std::string>& extra_options, CompileInfo* info)
{
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::string> opts = base_options();
    opts.insert(opts.end(), extra_options.begin(), extra_options.end());
    std::string key_material = source;
    for (const auto& o : opts) key_material += "\n//opt " + o;
    key_material += "\n//nvrtc " + std::to_string(nvrtc_version());
    const std::string key = hash_hex(key_material);
    const std::string file = cache_dir + "/" + key + ".cubin";

    std::string cubin;
    bool cached = read_file(file, cubin);
    std::string log;
    if (!cached) {
        cubin = compile_cubin(source, extra_options, &log);
        mkdirs(cache_dir);
        const std::string tmp = file + ".tmp." + std::to_string(getpid());
        {
            std::ofstream f(tmp, std::ios::binary);
            f.write(cubin.data(), (std::streamsize)cubin.size());
        }
        std::rename(tmp.c_str(), file.c_str());
    }
    auto m = std::shared_ptr<CudaModule>(new CudaModule());
    check_drv(driver().load(&m->module_, cubin.data()), "cuModuleLoadData");
    if (info) {
        info->cached = cached;
        info->cache_file = file;
        info->log = log;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return m;
}

std::shared_ptr<CudaModule> CudaModule::load(const std::string& cubin)
{
    auto m = std::shared_ptr<CudaModule>(new CudaModule());
    check_drv(driver().load(&m->module_, cubin.data()), "cuModuleLoadData");
    return m;
}

CudaModule::~CudaModule()
{
    if (module_) driver().unload(module_);
}

void* CudaModule::function(const std::string& name)
{
    auto it = functions_.find(name);
    if (it != functions_.end()) return it->second;
    void* f = nullptr;
    check_drv(driver().get_function(&f, module_, name.c_str()), ("cuModuleGetFunction " + name).c_str());
    functions_[name] = f;
    return f;
}

void CudaModule::launch(const std::string& kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t stream, void** args)
{
    void* f = function(kernel);
    if (smem > 48 * 1024) check_drv(driver().set_attr(f, 8 /*MAX_DYNAMIC_SHARED_SIZE_BYTES*/, (int)smem), "cuFuncSetAttribute");
    check_drv(driver().launch(f, grid.x, grid.y, grid.z, block.x, block.y, block.z, (unsigned)smem, stream, args, nullptr),
              ("cuLaunchKernel " + kernel).c_str());
    count_launch(1);
}

int CudaModule::max_threads_per_block(const std::string& kernel)
{
    int v = 0;
    check_drv(driver().get_attr(&v, 0 /*MAX_THREADS_PER_BLOCK*/, function(kernel)), "cuFuncGetAttribute");
    return v;
}

}  // namespace symxg
