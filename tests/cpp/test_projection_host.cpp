// Host build of the device projection code (project_pd.cuh) for CPU tests: the full
// cyclic-Jacobi projection and the translation-deflated one, in double and float.
// Usage: test_projection_host <in> <out>
//   in : int64 count, int64 n (= 12), count*n*n doubles (row-major matrices)
//   out: per mode (f64 full, f64 deflated, f32 full, f32 deflated) count*n*n doubles,
//        then count int32 deflation results per precision (-1: not translation-invariant).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <vector>

#define SYMXG_DEVICE inline
static inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
static inline float __frcp_rn(float x) { return 1.0f / x; }
using std::fabs;
using std::fmax;
using std::sqrt;
#include "../../symx_gb300/csrc/project_pd.cuh"

int main(int argc, char** argv)
{
    if (argc != 3) return 2;
    std::ifstream f(argv[1], std::ios::binary);
    int64_t hdr[2];
    f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
    const int64_t count = hdr[0];
    if (hdr[1] != 12) return 2;
    constexpr int N = 12;
    std::vector<double> in((size_t)count * N * N);
    f.read(reinterpret_cast<char*>(in.data()), in.size() * sizeof(double));
    std::vector<double> out(4 * in.size());
    std::vector<int32_t> status(2 * count);
    int nc = 0;
    for (int64_t e = 0; e < count; ++e) {
        double d[2][N * N];
        float s[2][N * N];
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const int k = symxg_dev::bm_index<N>(i, j);
                d[0][k] = d[1][k] = in[(e * N + i) * N + j];
                s[0][k] = s[1][k] = (float)in[(e * N + i) * N + j];
            }
        symxg_dev::project_pd_inplace<double, N>(d[0], 1e-10, false, &nc);
        status[e] = symxg_dev::project_pd_deflated<double, 4>(d[1], 1e-10, false, &nc);
        symxg_dev::project_pd_inplace<float, N>(s[0], 1e-10f, false, &nc);
        status[count + e] = symxg_dev::project_pd_deflated<float, 4>(s[1], 1e-10f, false, &nc);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const int k = symxg_dev::bm_index<N>(i, j);
                const size_t o = (size_t)(e * N + i) * N + j;
                out[o] = d[0][k];
                out[in.size() + o] = d[1][k];
                out[2 * in.size() + o] = s[0][k];
                out[3 * in.size() + o] = s[1][k];
            }
    }
    std::ofstream g(argv[2], std::ios::binary);
    g.write(reinterpret_cast<const char*>(out.data()), out.size() * sizeof(double));
    g.write(reinterpret_cast<const char*>(status.data()), status.size() * sizeof(int32_t));
    std::printf("not_converged %d\n", nc);
    return 0;
}
