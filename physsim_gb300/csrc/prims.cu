// prims.cu — device-wide exclusive scan and stable LSD radix sort of
// (uint64 key, uint32 value) pairs.  Both take their element count from
// device memory, so a frame can run without reading counts back to the host.
//
// Radix sort: 8-bit digits, 4096-key tiles (256 threads x 16 keys, warp-
// striped).  Per pass: (1) tile histograms, warp-aggregated with
// __match_any_sync; (2) exclusive scan of the digit-major histogram table;
// (3) stable ranking (match_any + per-warp running counts), local scatter into
// shared memory, then run-contiguous global writes.  Passes whose 8 bits are
// the same in every key are turned into a plain copy by a pre-pass that
// AND/OR-reduces the keys.
//
// Small inputs (at most 8192 pairs of capacity, e.g. a 2048-particle system)
// take single-CTA forms instead: one launch sorts the whole tile through all
// passes in shared memory, and one launch scans a tile.  Multi-kernel forms
// there are bound by launch latency, not by work.
#include "prims.cuh"

namespace geon {

// ---------------------------------------------------------------------------
// Exclusive scan
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one int per thread; returns the exclusive prefix,
// writes the block total to *total.
template <int THREADS>
__device__ __forceinline__ int block_excl_scan(int v, int* smem_warp, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NW = THREADS / 32;
    int incl = warp_incl_scan(v);
    if (lane == 31) smem_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < NW ? smem_warp[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < NW) smem_warp[lane] = wi - w;
        if (lane == NW - 1) smem_warp[NW] = wi;
    }
    __syncthreads();
    int res = incl - v + smem_warp[warp];
    if (total) *total = smem_warp[NW];
    __syncthreads();
    return res;
}

__global__ void scan_reduce_kernel(const int* __restrict__ in, int len, const int* d_n, int* __restrict__ block_sums) {
    __shared__ int sw[SCAN_THREADS / 32 + 1];
    const int n = d_n ? min(len, *d_n) : len;
    const int base = blockIdx.x * SCAN_TILE;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int i = base + threadIdx.x * SCAN_ITEMS + k;
        if (i < n) s += in[i];
    }
    int tot;
    block_excl_scan<SCAN_THREADS>(s, sw, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void scan_blocks_kernel(int* __restrict__ block_sums, int nb, int* __restrict__ total_out) {
    __shared__ int sw[SCAN_THREADS / 32 + 1];
    int carry = 0;
    for (int base = 0; base < nb; base += SCAN_THREADS) {
        int i = base + threadIdx.x;
        int v = i < nb ? block_sums[i] : 0;
        int tot;
        int ex = block_excl_scan<SCAN_THREADS>(v, sw, &tot);
        if (i < nb) block_sums[i] = ex + carry;
        carry += tot;
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

__global__ void scan_apply_kernel(const int* __restrict__ in, int* __restrict__ out, int len, const int* d_n,
                                  const int* __restrict__ block_sums) {
    __shared__ int sw[SCAN_THREADS / 32 + 1];
    const int n = d_n ? min(len, *d_n) : len;
    const int base = blockIdx.x * SCAN_TILE;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int i = base + threadIdx.x * SCAN_ITEMS + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int ex = block_excl_scan<SCAN_THREADS>(s, sw, nullptr) + block_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int i = base + threadIdx.x * SCAN_ITEMS + k;
        if (i < len) out[i] = (i < n) ? ex : 0;
        ex += v[k];
    }
}

// The whole scan in one CTA (len <= SCAN_TILE).
__global__ void scan_single_kernel(const int* __restrict__ in, int* __restrict__ out, int len, const int* d_n,
                                   int* __restrict__ total_out) {
    __shared__ int sw[SCAN_THREADS / 32 + 1];
    const int n = d_n ? min(len, *d_n) : len;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int i = threadIdx.x * SCAN_ITEMS + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    int tot;
    int ex = block_excl_scan<SCAN_THREADS>(s, sw, &tot);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int i = threadIdx.x * SCAN_ITEMS + k;
        if (i < len) out[i] = (i < n) ? ex : 0;
        ex += v[k];
    }
    if (threadIdx.x == 0 && total_out) *total_out = tot;
}

size_t scan_temp_ints(int len) { return (size_t)(len + SCAN_TILE - 1) / SCAN_TILE + 1; }

void exclusive_scan(const int* d_in, int* d_out, int len, const int* d_n, int* d_total, int* d_temp,
                    cudaStream_t st, LaunchCounter* lc) {
    if (len <= 0) return;
    if (len <= SCAN_TILE) {
        scan_single_kernel<<<1, SCAN_THREADS, 0, st>>>(d_in, d_out, len, d_n, d_total);
        if (lc) lc->add(1);
        return;
    }
    const int nb = (len + SCAN_TILE - 1) / SCAN_TILE;
    scan_reduce_kernel<<<nb, SCAN_THREADS, 0, st>>>(d_in, len, d_n, d_temp);
    scan_blocks_kernel<<<1, SCAN_THREADS, 0, st>>>(d_temp, nb, d_total);
    scan_apply_kernel<<<nb, SCAN_THREADS, 0, st>>>(d_in, d_out, len, d_n, d_temp);
    if (lc) lc->add(3);
}

// ---------------------------------------------------------------------------
// Radix sort
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;   // 4096
constexpr int RS_RADIX = 256;

__global__ void key_bits_kernel(const uint64_t* __restrict__ keys, const int* d_n, int len,
                                unsigned long long* and_or /* [2] */) {
    const int n = min(len, *d_n);
    uint64_t a = ~0ull, o = 0ull;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t k = keys[i];
        a &= k; o |= k;
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        a &= __shfl_xor_sync(0xffffffffu, a, s);
        o |= __shfl_xor_sync(0xffffffffu, o, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAnd(&and_or[0], (unsigned long long)a);
        atomicOr(&and_or[1], (unsigned long long)o);
    }
}

__device__ __forceinline__ bool pass_is_constant(const unsigned long long* and_or, int shift) {
    const uint64_t diff = (and_or[0] ^ and_or[1]) >> shift;
    return (diff & 0xffull) == 0;
}

__global__ void __launch_bounds__(RS_THREADS)
radix_upsweep_kernel(const uint64_t* __restrict__ keys, const int* d_n, int len, int shift,
                     const unsigned long long* and_or, unsigned* __restrict__ hist, int num_blocks) {
    if (pass_is_constant(and_or, shift)) return;
    __shared__ unsigned s_hist[RS_RADIX];
    const int n = min(len, *d_n);
    for (int i = threadIdx.x; i < RS_RADIX; i += RS_THREADS) s_hist[i] = 0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int base = blockIdx.x * RS_TILE + warp * (32 * RS_ITEMS);
#pragma unroll 4
    for (int j = 0; j < RS_ITEMS; j++) {
        int idx = base + j * 32 + lane;
        bool valid = idx < n;
        unsigned d = valid ? (unsigned)((keys[idx] >> shift) & 0xffu) : 0x100u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        if (valid && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&s_hist[d], (unsigned)__popc(peers));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < RS_RADIX; i += RS_THREADS) hist[i * num_blocks + blockIdx.x] = s_hist[i];
}

__global__ void __launch_bounds__(RS_THREADS)
radix_downsweep_kernel(const uint64_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                       uint64_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                       const int* d_n, int len, int shift, const unsigned long long* and_or,
                       const unsigned* __restrict__ offsets, int num_blocks) {
    const int n = min(len, *d_n);
    const int tile_base = blockIdx.x * RS_TILE;
    if (pass_is_constant(and_or, shift)) {
        for (int i = tile_base + threadIdx.x; i < min(n, tile_base + RS_TILE); i += RS_THREADS) {
            keys_out[i] = keys_in[i];
            vals_out[i] = vals_in[i];
        }
        return;
    }
    extern __shared__ __align__(16) unsigned char rs_smem[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(rs_smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + RS_TILE);
    unsigned (*s_warp)[RS_RADIX] = reinterpret_cast<unsigned (*)[RS_RADIX]>(s_vals + RS_TILE);
    unsigned* s_start = &s_warp[RS_WARPS][0];
    unsigned* s_gbase = s_start + RS_RADIX;
    int* s_scan = reinterpret_cast<int*>(s_gbase + RS_RADIX);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < RS_WARPS * RS_RADIX; i += RS_THREADS) (&s_warp[0][0])[i] = 0;
    __syncthreads();

    const int base = tile_base + warp * (32 * RS_ITEMS);
    uint64_t k[RS_ITEMS];
    uint32_t v[RS_ITEMS];
    unsigned rank[RS_ITEMS];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < RS_ITEMS; j++) {
        int idx = base + j * 32 + lane;
        bool valid = idx < n;
        k[j] = valid ? keys_in[idx] : 0ull;
        v[j] = valid ? vals_in[idx] : 0u;
        unsigned d = valid ? (unsigned)((k[j] >> shift) & 0xffu) : 0x100u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        unsigned prior = valid ? s_warp[warp][d] : 0u;
        rank[j] = prior + __popc(peers & lt);
        __syncwarp();
        if (valid && lane == (unsigned)(__ffs(peers) - 1)) s_warp[warp][d] = prior + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: exclusive over warps, then exclusive over digits
    {
        const int d = threadIdx.x;   // RS_THREADS == RS_RADIX
        unsigned run = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) {
            unsigned c = s_warp[w][d];
            s_warp[w][d] = run;
            run += c;
        }
        int tot;
        int ex = block_excl_scan<RS_THREADS>((int)run, s_scan, &tot);
        s_start[d] = (unsigned)ex;
        s_gbase[d] = offsets[d * num_blocks + blockIdx.x];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < RS_ITEMS; j++) {
        int idx = base + j * 32 + lane;
        if (idx < n) {
            unsigned d = (unsigned)((k[j] >> shift) & 0xffu);
            unsigned pos = s_start[d] + s_warp[warp][d] + rank[j];
            s_keys[pos] = k[j];
            s_vals[pos] = v[j];
        }
    }
    __syncthreads();
    const int cnt = min(RS_TILE, n - tile_base);
    for (int i = threadIdx.x; i < cnt; i += RS_THREADS) {
        uint64_t key = s_keys[i];
        unsigned d = (unsigned)((key >> shift) & 0xffu);
        unsigned out = s_gbase[d] + (i - s_start[d]);
        keys_out[out] = key;
        vals_out[out] = s_vals[i];
    }
}

constexpr size_t RS_DOWN_SMEM = RS_TILE * (sizeof(uint64_t) + sizeof(uint32_t)) +
                                (RS_WARPS + 2) * RS_RADIX * sizeof(unsigned) + (RS_THREADS / 32 + 1) * sizeof(int);

// Single-CTA sort of at most THREADS * ITEMS pairs, in place: every pass of
// the tile sort above (match_any ranking, per-warp running counts, digit
// scan, stable scatter) with the keys kept in shared memory between passes;
// passes whose 8 bits are the same in every key are skipped.
template <int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS)
radix_tile_sort_kernel(uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, const int* d_n, int len,
                       int end_bit) {
    constexpr int WARPS = THREADS / 32, TILE = THREADS * ITEMS;
    static_assert(THREADS >= RS_RADIX, "one thread per digit");
    extern __shared__ __align__(16) unsigned char ts_smem[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(ts_smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
    unsigned (*s_warp)[RS_RADIX] = reinterpret_cast<unsigned (*)[RS_RADIX]>(s_vals + TILE);
    unsigned* s_start = &s_warp[WARPS][0];
    int* s_scan = reinterpret_cast<int*>(s_start + RS_RADIX);
    __shared__ unsigned long long s_ao[2];
    const int n = min(min(len, *d_n), TILE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int base = warp * (32 * ITEMS);
    uint64_t k[ITEMS];
    uint32_t v[ITEMS];
    uint64_t a = ~0ull, o = 0ull;
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
        const int idx = base + j * 32 + lane;
        const bool valid = idx < n;
        k[j] = valid ? keys[idx] : 0ull;
        v[j] = valid ? vals[idx] : 0u;
        if (valid) { a &= k[j]; o |= k[j]; }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        a &= __shfl_xor_sync(0xffffffffu, a, s);
        o |= __shfl_xor_sync(0xffffffffu, o, s);
    }
    if (threadIdx.x == 0) { s_ao[0] = ~0ull; s_ao[1] = 0ull; }
    __syncthreads();
    if (lane == 0) { atomicAnd(&s_ao[0], (unsigned long long)a); atomicOr(&s_ao[1], (unsigned long long)o); }
    __syncthreads();
    const uint64_t diff = s_ao[0] ^ s_ao[1];
    const unsigned lt = lanemask_lt();
    for (int shift = 0; shift < end_bit; shift += 8) {
        if (((diff >> shift) & 0xffull) == 0) continue;                 // same for the whole CTA
        for (int i = threadIdx.x; i < WARPS * RS_RADIX; i += THREADS) (&s_warp[0][0])[i] = 0;
        __syncthreads();
        unsigned rank[ITEMS];
#pragma unroll
        for (int j = 0; j < ITEMS; j++) {
            const bool valid = base + j * 32 + lane < n;
            const unsigned d = valid ? (unsigned)((k[j] >> shift) & 0xffu) : 0x100u;
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const unsigned prior = valid ? s_warp[warp][d] : 0u;
            rank[j] = prior + __popc(peers & lt);
            __syncwarp();
            if (valid && lane == (unsigned)(__ffs(peers) - 1)) s_warp[warp][d] = prior + __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        int run = 0;
        if (threadIdx.x < RS_RADIX) {                                 // per digit: exclusive over warps
            const int d = threadIdx.x;
            for (int w = 0; w < WARPS; w++) {
                const unsigned c = s_warp[w][d];
                s_warp[w][d] = (unsigned)run;
                run += (int)c;
            }
        }
        const int ex = block_excl_scan<THREADS>(run, s_scan, nullptr);  // then over digits
        if (threadIdx.x < RS_RADIX) s_start[threadIdx.x] = (unsigned)ex;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < ITEMS; j++) {
            if (base + j * 32 + lane < n) {
                const unsigned d = (unsigned)((k[j] >> shift) & 0xffu);
                const unsigned pos = s_start[d] + s_warp[warp][d] + rank[j];
                s_keys[pos] = k[j];
                s_vals[pos] = v[j];
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < ITEMS; j++) {
            const int idx = base + j * 32 + lane;
            if (idx < n) { k[j] = s_keys[idx]; v[j] = s_vals[idx]; }
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
        const int idx = base + j * 32 + lane;
        if (idx < n) { keys[idx] = k[j]; vals[idx] = v[j]; }
    }
}

template <int THREADS, int ITEMS>
constexpr size_t tile_sort_smem() {
    return (size_t)THREADS * ITEMS * (sizeof(uint64_t) + sizeof(uint32_t)) +
           (size_t)(THREADS / 32 + 1) * RS_RADIX * sizeof(unsigned) + (THREADS / 32 + 1) * sizeof(int);
}

template <int THREADS, int ITEMS>
static void tile_sort(uint64_t* keys, uint32_t* vals, int len, const int* d_n, int end_bit, cudaStream_t st) {
    constexpr size_t smem = tile_sort_smem<THREADS, ITEMS>();
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(radix_tile_sort_kernel<THREADS, ITEMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        attr = true;
    }
    radix_tile_sort_kernel<THREADS, ITEMS><<<1, THREADS, smem, st>>>(keys, vals, d_n, len, end_bit);
}

__global__ void clear_and_or_kernel(unsigned long long* and_or) {
    and_or[0] = ~0ull;
    and_or[1] = 0ull;
}

size_t radix_temp_bytes(int len) {
    const int nb = (len + RS_TILE - 1) / RS_TILE;
    size_t hist = (size_t)RS_RADIX * nb * sizeof(unsigned);
    size_t scan = scan_temp_ints(RS_RADIX * nb) * sizeof(int);
    return 256 + 2 * hist + scan + 64;
}

// Sorts (keys, vals) by bits [0, end_bit).  Ping-pongs between the given
// buffers; returns 0 when the result is in (keys, vals), 1 when in (keys_alt, vals_alt).
int radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt,
                     int len, const int* d_n, int end_bit, void* d_temp, cudaStream_t st, LaunchCounter* lc) {
    if (len <= 0) return 0;
    if (len <= 256 * 16) {                          // one CTA, in place
        tile_sort<256, 16>(keys, vals, len, d_n, end_bit, st);
        if (lc) lc->add(1);
        return 0;
    }
    if (len <= 1024 * 8) {
        tile_sort<1024, 8>(keys, vals, len, d_n, end_bit, st);
        if (lc) lc->add(1);
        return 0;
    }
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(radix_downsweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RS_DOWN_SMEM);
        attr_set = true;
    }
    const int nb = (len + RS_TILE - 1) / RS_TILE;
    char* t = static_cast<char*>(d_temp);
    unsigned long long* and_or = reinterpret_cast<unsigned long long*>(t);
    unsigned* hist = reinterpret_cast<unsigned*>(t + 256);
    const size_t hist_bytes = (size_t)RS_RADIX * nb * sizeof(unsigned);
    unsigned* offs = reinterpret_cast<unsigned*>(t + 256 + hist_bytes);
    int* scan_tmp = reinterpret_cast<int*>(t + 256 + 2 * hist_bytes);

    clear_and_or_kernel<<<1, 1, 0, st>>>(and_or);
    key_bits_kernel<<<std::min(nb * 4, 1216), 256, 0, st>>>(keys, d_n, len, and_or);
    if (lc) lc->add(2);
    int which = 0;
    uint64_t* kin = keys; uint32_t* vin = vals;
    uint64_t* kout = keys_alt; uint32_t* vout = vals_alt;
    for (int shift = 0; shift < end_bit; shift += 8) {
        radix_upsweep_kernel<<<nb, RS_THREADS, 0, st>>>(kin, d_n, len, shift, and_or, hist, nb);
        // the scan runs over the whole table; constant passes leave stale
        // counts there, but their downsweep never reads the offsets
        exclusive_scan(reinterpret_cast<const int*>(hist), reinterpret_cast<int*>(offs), RS_RADIX * nb,
                       nullptr, nullptr, scan_tmp, st, lc);
        radix_downsweep_kernel<<<nb, RS_THREADS, RS_DOWN_SMEM, st>>>(kin, vin, kout, vout, d_n, len, shift, and_or, offs, nb);
        if (lc) lc->add(2);
        std::swap(kin, kout);
        std::swap(vin, vout);
        which ^= 1;
    }
    return which;
}

}  // namespace geon
