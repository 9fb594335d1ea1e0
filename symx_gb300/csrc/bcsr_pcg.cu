// Stand-alone block-Jacobi PCG on a caller's 3x3-block CSR matrix (see bcsr_pcg.h).
//
// The iteration kernels are the ones the Newton solver runs (kernels.cu); this file adds the
// preconditioner set-up from the matrix rows, the workspace layout and the host loop.
#include "bcsr_pcg.h"

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "kernels.cuh"

namespace symxg {

namespace {

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("symx_gb300 bcsr_pcg: ") + what + ": " + cudaGetErrorString(e));
}

// Dinv of block row r: the inverse of the row's diagonal block (found by scanning the row,
// inverted in double from its upper triangle, stored as 3 rows of 4 in T), the
// block-diagonal preconditioner of BlockedSparseMatrix::prepare_preconditioning.  A row
// without a diagonal block gets Dinv = 0 and is counted in *missing.
template <typename T>
__global__ void k_block_jacobi_rows(int n_blocks, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                                    const T* __restrict__ vals, int64_t vs, T* __restrict__ Dinv, int* missing)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_blocks) return;
    int64_t k = -1;
    for (int64_t j = row_ptr[r], e = row_ptr[r + 1]; j < e; ++j)
        if (cols[j] == r) { k = j; break; }
    T* o = Dinv + (int64_t)r * 12;
    if (k < 0) {
        for (int i = 0; i < 12; ++i) o[i] = T(0);
        atomicAdd(missing, 1);
        return;
    }
    const double a = vals[k], b = vals[vs + k], c = vals[2 * vs + k], d = vals[4 * vs + k], e = vals[5 * vs + k],
                 f = vals[8 * vs + k];
    const double c00 = d * f - e * e, c01 = c * e - b * f, c02 = b * e - c * d;
    const double id = 1.0 / (a * c00 + b * c01 + c * c02);
    const double i11 = (a * f - c * c) * id, i12 = (b * c - a * e) * id, i22 = (a * d - b * b) * id;
    o[0] = (T)(c00 * id); o[1] = (T)(c01 * id); o[2] = (T)(c02 * id); o[3] = T(0);
    o[4] = (T)(c01 * id); o[5] = (T)i11;        o[6] = (T)i12;        o[7] = T(0);
    o[8] = (T)(c02 * id); o[9] = (T)i12;        o[10] = (T)i22;       o[11] = T(0);
}

// The solver state at the start of the workspace: PcgState, then 4 ints ([0] counts the
// rows without a diagonal block).
struct Header {
    PcgState st;
    int flags[4];
};
static_assert(sizeof(Header) <= 256, "state part of the workspace is 256 bytes");

struct Layout {
    size_t tickets, partials, dinv, vecs, vec_bytes, total;
};

template <typename T>
Layout layout(int n_blocks, unsigned partials_per_part)
{
    const size_t n = (size_t)n_blocks;
    Layout L;
    L.tickets = 256;
    L.partials = L.tickets + bcsr_pcg_round_up(8 * sizeof(unsigned));
    L.dinv = L.partials + bcsr_pcg_round_up(2 * (size_t)partials_per_part * sizeof(double));
    L.vecs = L.dinv + bcsr_pcg_round_up(12 * n * sizeof(T));
    L.vec_bytes = bcsr_pcg_round_up(4 * n * sizeof(T));
    L.total = L.vecs + 6 * L.vec_bytes;  // == bcsr_pcg_workspace_size(n, partials_per_part, sizeof(T))
    return L;
}

}  // namespace

template <typename T>
BcsrPcgResult run_bcsr_pcg(int n_blocks, const int32_t* row_ptr, const int32_t* cols, const T* vals,
                           int64_t vals_stride, const T* b, T* x, double abs_tol, double rel_tol, int max_iterations,
                           void* workspace, size_t workspace_bytes, unsigned partials_per_part, cudaStream_t s)
{
    BcsrPcgResult res;
    if (n_blocks == 0) {
        res.converged = 1;
        return res;
    }
    if (partials_per_part < pcg_max_grid())
        throw std::invalid_argument("bcsr_pcg: workspace has room for fewer partial sums than the PCG grid");
    const Layout L = layout<T>(n_blocks, partials_per_part);
    if (workspace_bytes < L.total) throw std::invalid_argument("bcsr_pcg: workspace too small");
    if (reinterpret_cast<uintptr_t>(workspace) % 16 != 0)
        throw std::invalid_argument("bcsr_pcg: workspace not 16-byte aligned");
    char* w = static_cast<char*>(workspace);
    Header* hdr = reinterpret_cast<Header*>(w);

    PcgBuffers<T> B;
    B.n_blocks = n_blocks;
    B.row_ptr = row_ptr;
    B.cols = cols;
    B.vals = vals;
    B.vals_stride = vals_stride;
    T* Dinv = reinterpret_cast<T*>(w + L.dinv);
    B.Dinv = Dinv;
    T* v[6];
    for (int i = 0; i < 6; ++i) v[i] = reinterpret_cast<T*>(w + L.vecs + i * L.vec_bytes);
    B.x = v[0];
    B.r = v[1];
    B.z = v[2];
    B.p = v[3];
    B.p2 = v[4];
    B.q = v[5];
    B.partials = reinterpret_cast<double*>(w + L.partials);
    B.tickets = reinterpret_cast<unsigned*>(w + L.tickets);
    B.state = &hdr->st;

    // The values array holds nine components of vals_stride entries each: a stride below the
    // number of blocks, row_ptr[n_blocks], would alias the components or read past the array.
    // Checked before the first kernel reads a value.
    int32_t nnzb = 0;
    ck(cudaMemcpyAsync(&nnzb, row_ptr + n_blocks, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "read row_ptr[n_blocks]");
    ck(cudaStreamSynchronize(s), "synchronize");
    if (nnzb < 0 || vals_stride < (int64_t)nnzb)
        throw std::invalid_argument("bcsr_pcg: vals_stride " + std::to_string(vals_stride) +
                                    " is smaller than the number of blocks row_ptr[n_blocks] = " + std::to_string(nnzb));

    // The completion tickets and the missing-diagonal counter must start at zero.
    Header h{};
    h.st.abs_tol = abs_tol;
    h.st.rel_tol = rel_tol;
    h.st.max_iterations = max_iterations;
    ck(cudaMemsetAsync(B.tickets, 0, 8 * sizeof(unsigned), s), "clear tickets");
    ck(cudaMemcpyAsync(hdr, &h, sizeof(Header), cudaMemcpyHostToDevice, s), "state");
    k_block_jacobi_rows<T><<<(n_blocks + 255) / 256, 256, 0, s>>>(n_blocks, row_ptr, cols, vals, vals_stride, Dinv,
                                                                   hdr->flags);
    ck(cudaGetLastError(), "block_jacobi_rows launch");
    count_launch();
    ck(cudaMemcpyAsync(&h, hdr, sizeof(Header), cudaMemcpyDeviceToHost, s), "read flags");
    ck(cudaStreamSynchronize(s), "synchronize");
    if (h.flags[0] != 0) {
        res.missing_diagonal = h.flags[0];
        return res;
    }

    launch_pcg_init_rhs<T>(B, b, s);
    int launched = 0, chunk = 8;
    while (true) {
        for (int k = 0; k < chunk; ++k) launch_pcg_iteration<T>(B, launched + k, s);
        launched += chunk;
        ck(cudaMemcpyAsync(&h, hdr, sizeof(Header), cudaMemcpyDeviceToHost, s), "read state");
        ck(cudaStreamSynchronize(s), "synchronize");
        if (h.st.done || launched > max_iterations + 1) break;
        chunk = std::min(chunk * 2, 64);
    }
    launch_rows4_to_vec3<T>(n_blocks, B.x, x, s);
    ck(cudaStreamSynchronize(s), "synchronize");
    res.converged = h.st.converged;
    res.iterations = h.st.iteration;
    res.indefinite = h.st.indefinite;
    res.error = h.st.error;
    return res;
}

#define SYMXG_PCG_INSTANTIATE(T)                                                                                      \
    template BcsrPcgResult run_bcsr_pcg<T>(int, const int32_t*, const int32_t*, const T*, int64_t, const T*, T*,      \
                                           double, double, int, void*, size_t, unsigned, cudaStream_t);
SYMXG_PCG_INSTANTIATE(float)
SYMXG_PCG_INSTANTIATE(double)

}  // namespace symxg
