// scan_sort.cu -- exclusive scan and stable LSD radix sort (see scan_sort.cuh).
#include "scan_sort.cuh"

namespace dsph {

namespace {

__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* warp_sums,
                                                        int32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < (kScanThreads / 32) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (kScanThreads / 32)) warp_sums[lane] = w;
    }
    __syncthreads();
    int32_t before = warp > 0 ? warp_sums[warp - 1] : 0;
    total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// per-tile sums (blocked arrangement: thread t owns items t*8..t*8+7)
__global__ void k_tile_sums(const int32_t* in, int64_t n, int32_t* sums) {
    __shared__ int32_t ws[kScanThreads / 32];
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kScanItems;
    int32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
        if (base + i < n) s += in[base + i];
    int32_t tot;
    block_exclusive_scan(s, ws, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// exclusive scan of up to any number of tile sums in one block, chunk by chunk
__global__ void k_scan_sums(int32_t* sums, int64_t nt) {
    __shared__ int32_t ws[kScanThreads / 32];
    int32_t carry = 0;
    for (int64_t c = 0; c < nt; c += kTile) {
        int64_t base = c + (int64_t)threadIdx.x * kScanItems;
        int32_t v[kScanItems];
        int32_t s = 0;
#pragma unroll
        for (int i = 0; i < kScanItems; i++) {
            v[i] = (base + i < nt) ? sums[base + i] : 0;
            s += v[i];
        }
        int32_t tot;
        int32_t ex = block_exclusive_scan(s, ws, tot) + carry;
#pragma unroll
        for (int i = 0; i < kScanItems; i++) {
            if (base + i < nt) sums[base + i] = ex;
            ex += v[i];
        }
        carry += tot;
    }
}

__global__ void k_tile_scan(const int32_t* in, int32_t* out, int64_t n, const int32_t* offs) {
    __shared__ int32_t ws[kScanThreads / 32];
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = (base + i < n) ? in[base + i] : 0;
        s += v[i];
    }
    int32_t tot;
    int32_t ex = block_exclusive_scan(s, ws, tot) + offs[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
}

// ---- radix sort ------------------------------------------------------------
// Items of a tile are striped: round r, thread t -> tile index r*256 + t, so
// the stable order inside the tile is (round, warp, lane).

__global__ void k_digit_hist(const uint32_t* keys, int64_t n, int shift, int32_t* hist,
                             int64_t ntiles) {
    __shared__ int32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll
    for (int r = 0; r < kScanItems; r++) {
        int64_t i = base + r * kScanThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_digit_scatter(const uint32_t* keys_in, const int32_t* vals_in,
                                uint32_t* keys_out, int32_t* vals_out, int64_t n, int shift,
                                const int32_t* offs, int64_t ntiles) {
    constexpr int W = kScanThreads / 32;
    __shared__ int32_t cnt[W][256];
    __shared__ int32_t running[256];
    __shared__ int32_t base_off[256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    running[tid] = 0;
    base_off[tid] = offs[(int64_t)tid * ntiles + blockIdx.x];
    const int64_t tbase = (int64_t)blockIdx.x * kTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kScanItems; r++) {
        int64_t i = tbase + r * kScanThreads + tid;
        bool valid = i < n;
        uint32_t key = valid ? keys_in[i] : 0u;
        int32_t val = valid ? (vals_in ? vals_in[i] : (int32_t)i) : 0;
        int d = valid ? (int)((key >> shift) & 255u) : 256;
#pragma unroll
        for (int w = 0; w < W; w++) cnt[w][tid] = 0;
        __syncthreads();
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int wrank = __popc(peers & lt);
        bool leader = (peers & lt) == 0u;
        if (valid && leader) cnt[warp][d] = __popc(peers);
        __syncthreads();
        // exclusive prefix over warps for digit tid; round total
        int32_t acc = 0;
#pragma unroll
        for (int w = 0; w < W; w++) {
            int32_t c = cnt[w][tid];
            cnt[w][tid] = acc;
            acc += c;
        }
        __syncthreads();
        if (valid) {
            int32_t pos = base_off[d] + running[d] + cnt[warp][d] + wrank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
        running[tid] += acc;
        __syncthreads();
    }
}



}  // namespace

int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch,
                       cudaStream_t st) {
    if (n <= 0) return 0;
    int64_t nt = tiles_of(n);
    int32_t* sums = static_cast<int32_t*>(scratch);
    k_tile_sums<<<(unsigned)nt, kScanThreads, 0, st>>>(in, n, sums);
    k_scan_sums<<<1, kScanThreads, 0, st>>>(sums, nt);
    k_tile_scan<<<(unsigned)nt, kScanThreads, 0, st>>>(in, out, n, sums);
    return 3;
}

int radix_sort_pairs(const uint32_t* keys_in, const int32_t* vals_in, uint32_t* keys_out,
                     int32_t* vals_out, uint32_t* keys_tmp, int32_t* vals_tmp, int64_t n,
                     int bits, void* scratch, cudaStream_t st) {
    if (n <= 0) return 0;
    if (bits < 1) bits = 1;
    const int passes = (bits + 7) / 8;
    const int64_t nt = tiles_of(n);
    int32_t* hist = static_cast<int32_t*>(scratch);
    void* scan_scratch = hist + 256 * nt;
    int launches = 0;
    // choose ping-pong so that the final pass lands in keys_out / vals_out
    const uint32_t* kin = keys_in;
    const int32_t* vin = vals_in;
    for (int p = 0; p < passes; p++) {
        bool to_out = ((passes - 1 - p) % 2) == 0;
        uint32_t* kout = to_out ? keys_out : keys_tmp;
        int32_t* vout = to_out ? vals_out : vals_tmp;
        int shift = 8 * p;
        k_digit_hist<<<(unsigned)nt, 256, 0, st>>>(kin, n, shift, hist, nt);
        launches++;
        launches += exclusive_scan_i32(hist, hist, 256 * nt, scan_scratch, st);
        k_digit_scatter<<<(unsigned)nt, 256, 0, st>>>(kin, vin, kout, vout, n, shift, hist, nt);
        launches++;
        kin = kout;
        vin = vout;
    }
    return launches;
}

}  // namespace dsph
