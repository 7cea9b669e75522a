// prims.cuh — host-side entry points of the device primitives (prims.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <algorithm>
#include <utility>
#include "common.cuh"

namespace geon {

// Streaming multiprocessors of the current device (queried once per device).
inline int device_sms() {
    static int cache[64] = { 0 };
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cache[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

// Counts kernel launches issued on behalf of a handle.
struct LaunchCounter {
    long long n = 0;
    void add(int k) { n += k; }
};

// Exclusive scan of `len` ints.  Elements at or beyond *d_n (when d_n is not
// null) count as zero and are written as zero.  *d_total (optional) receives
// the sum.  d_temp must hold scan_temp_ints(len) ints.
size_t scan_temp_ints(int len);
void exclusive_scan(const int* d_in, int* d_out, int len, const int* d_n, int* d_total, int* d_temp,
                    cudaStream_t st, LaunchCounter* lc);

// Stable LSD radix sort of min(len, *d_n) (key, value) pairs on bits
// [0, end_bit).  Returns 0 if the sorted data ended in (keys, vals), 1 if in
// the *_alt buffers.  d_temp must hold radix_temp_bytes(len) bytes.
size_t radix_temp_bytes(int len);
int radix_sort_pairs(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt,
                     int len, const int* d_n, int end_bit, void* d_temp, cudaStream_t st, LaunchCounter* lc);

}  // namespace geon
