// cell_sort_api.cu -- the radix cell sort as a stand-alone C entry point.
//
// sph_cell_sort: n cell keys (device memory) -> the stable order of the
// particles by cell and the first sorted position of every cell, i.e. a cell
// list in CSR form (the structure of sph.hpp:147-162, built on the device).
#include <cstdint>
#include <string>

#include "../../include/deorbit_sph.h"
#include "scan_sort.cuh"

namespace dsph {
void set_error_message(const std::string& m);
}

namespace {

// per-cell counts; keys outside [0, ncells) are counted nowhere and flagged
__global__ void k_count_keys(const uint32_t* keys, int64_t n, int64_t ncells, int32_t* counts,
                             int32_t* bad) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t k = keys[i];
    if ((int64_t)k >= ncells) {
        atomicOr(bad, 1);
        return;
    }
    atomicAdd(&counts[k], 1);
}

int key_bits(int64_t ncells) {
    int b = 1;
    while ((1ll << b) < ncells) b++;
    return b;
}

}  // namespace

namespace dsph {

// Scratch layout shared by both entry points: keys_out, keys_tmp, vals_tmp
// (n each), the radix / scan scratch, one flag word.
size_t cell_sort_scratch_bytes(int64_t n, int64_t ncells) {
    size_t a = 256;
    auto up = [a](size_t x) { return (x + a - 1) / a * a; };
    size_t b = 3 * up(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    size_t s1 = radix_scratch_bytes(n > 0 ? n : 1), s2 = scan_scratch_bytes(ncells + 1);
    b += up(s1 > s2 ? s1 : s2) + a;
    return b;
}

// Runs the sort with caller-provided scratch; returns SPH_* status.
int cell_sort_with_scratch(const uint32_t* keys, int64_t n, int64_t ncells, int32_t* perm,
                           int32_t* cell_start, cudaStream_t st, void* scratch) {
    const size_t a = 256;
    auto up = [a](size_t x) { return (x + a - 1) / a * a; };
    char* p = static_cast<char*>(scratch);
    const size_t nb = up(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    uint32_t* keys_out = reinterpret_cast<uint32_t*>(p);
    uint32_t* keys_tmp = reinterpret_cast<uint32_t*>(p + nb);
    int32_t* vals_tmp = reinterpret_cast<int32_t*>(p + 2 * nb);
    void* work = p + 3 * nb;
    size_t s1 = radix_scratch_bytes(n > 0 ? n : 1), s2 = scan_scratch_bytes(ncells + 1);
    int32_t* bad = reinterpret_cast<int32_t*>(p + 3 * nb + up(s1 > s2 ? s1 : s2));
    cudaError_t e;
    if ((e = cudaMemsetAsync(bad, 0, sizeof(int32_t), st)) != cudaSuccess) goto cuda_fail;
    if ((e = cudaMemsetAsync(cell_start, 0, sizeof(int32_t) * (size_t)(ncells + 1), st)) != cudaSuccess)
        goto cuda_fail;
    if (n > 0) {
        k_count_keys<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(keys, n, ncells, cell_start, bad);
        radix_sort_pairs(keys, nullptr, keys_out, perm, keys_tmp, vals_tmp, n, key_bits(ncells), work, st);
    }
    exclusive_scan_i32(cell_start, cell_start, ncells + 1, work, st);
    {
        int32_t h_bad = 0;
        if ((e = cudaGetLastError()) != cudaSuccess) goto cuda_fail;
        if ((e = cudaMemcpyAsync(&h_bad, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            goto cuda_fail;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) goto cuda_fail;
        if (h_bad) {
            set_error_message("cell key outside [0, ncells)");
            return SPH_ERR_ARG;
        }
    }
    return SPH_OK;
cuda_fail:
    cudaGetLastError();
    set_error_message(std::string("cell sort: ") + cudaGetErrorString(e));
    return SPH_ERR_CUDA;
}

}  // namespace dsph

extern "C" int sph_cell_sort(const uint32_t* keys, int64_t n, int64_t ncells, int32_t* perm,
                             int32_t* cell_start, void* stream) {
    if (n < 0 || ncells < 1 || ncells > (int64_t)0x7ffffffe || n > (int64_t)0x7ffffffe) {
        dsph::set_error_message("sph_cell_sort: n must be >= 0 and 1 <= ncells < 2^31 - 1");
        return SPH_ERR_ARG;
    }
    if (!cell_start || (n > 0 && (!keys || !perm))) {
        dsph::set_error_message("sph_cell_sort: null pointer");
        return SPH_ERR_ARG;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, dsph::cell_sort_scratch_bytes(n, ncells), st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        dsph::set_error_message(std::string("sph_cell_sort: ") + cudaGetErrorString(e));
        return SPH_ERR_NOMEM;
    }
    int rc = dsph::cell_sort_with_scratch(keys, n, ncells, perm, cell_start, st, scratch);
    cudaFreeAsync(scratch, st);
    cudaStreamSynchronize(st);
    return rc;
}
