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
constexpr size_t round_up_256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t cell_sort_scratch_bytes(int64_t n, int64_t ncells) {
    return 3 * round_up_256(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1)) +
           round_up_256(radix_scratch_bytes(n > 0 ? n : 1) > scan_scratch_bytes(ncells + 1)
                            ? radix_scratch_bytes(n > 0 ? n : 1)
                            : scan_scratch_bytes(ncells + 1)) +
           256;
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

// ---------------------------------------------------------------------------
// Allocation-free variant.  Its scratch is this file-scope device array: every
// GPU that loads the library reserves it (3.5 MiB) until the process exits,
// and all calls share it.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr int64_t kStaticMaxKeys = 1 << 18;    // 262,144 keys per call
constexpr int64_t kStaticMaxCells = 1 << 24;   // 16,777,216 cells per call
constexpr size_t kStaticScratchBytes = 3670016;
// the largest accepted call must fit the array (the layout grows with both sizes)
static_assert(dsph::cell_sort_scratch_bytes(kStaticMaxKeys, kStaticMaxCells) <= kStaticScratchBytes,
              "static cell-sort scratch too small for its documented limits");

__device__ __align__(256) unsigned char g_cell_sort_scratch[kStaticScratchBytes];

std::mutex g_static_mu;
void* g_static_addr[256] = {};

// Device address of the scratch array on the current device.  The host-side
// name g_cell_sort_scratch is only a stand-in for the symbol, not a device
// address, so the address is looked up once per device (with that device
// current) and cached.  The cache assumes one context per device for the life
// of the process (the runtime's primary context): after cudaDeviceReset, or
// under another driver-API context, the cached address is stale.
int static_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 256) {
        cudaGetLastError();
        dsph::set_error_message("sph_cell_sort_static: no current CUDA device");
        return SPH_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_cell_sort_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            dsph::set_error_message(std::string("sph_cell_sort_static: cudaGetSymbolAddress: ") +
                                    cudaGetErrorString(e));
            return SPH_ERR_CUDA;
        }
        g_static_addr[dev] = p;
    }
    *out = g_static_addr[dev];
    return SPH_OK;
}

}  // namespace

extern "C" int sph_cell_sort_static(const uint32_t* keys, int64_t n, int64_t ncells, int32_t* perm,
                                    int32_t* cell_start, void* stream) {
    if (n < 0 || ncells < 1) {
        dsph::set_error_message("sph_cell_sort_static: n must be >= 0 and ncells >= 1");
        return SPH_ERR_ARG;
    }
    if (n > kStaticMaxKeys || ncells > kStaticMaxCells) {
        dsph::set_error_message("sph_cell_sort_static: at most 262144 keys and 16777216 cells per call "
                                "(use sph_cell_sort for larger inputs)");
        return SPH_ERR_CAPACITY;
    }
    if (!cell_start || (n > 0 && (!keys || !perm))) {
        dsph::set_error_message("sph_cell_sort_static: null pointer");
        return SPH_ERR_ARG;
    }
    // every call waits for its result on the host, which a stream being
    // captured into a graph cannot do: refuse before touching the stream
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess) {
        cudaGetLastError();
        dsph::set_error_message("sph_cell_sort_static: invalid stream");
        return SPH_ERR_ARG;
    }
    if (cap != cudaStreamCaptureStatusNone) {
        dsph::set_error_message("sph_cell_sort_static: the stream is being captured; the call "
                                "synchronizes and cannot be captured");
        return SPH_ERR_STATE;
    }
    void* scratch = nullptr;
    int rc = static_scratch(&scratch);
    if (rc != SPH_OK) return rc;
    return dsph::cell_sort_with_scratch(keys, n, ncells, perm, cell_start,
                                        static_cast<cudaStream_t>(stream), scratch);
}
