// Device scan and stable radix sort (gbn_sort.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace gbn {

// Bytes of device temporaries exclusive_scan needs for n elements.
size_t scan_temp_bytes(int64_t n);
// out[i] = in[0] + ... + in[i-1] (int32; in and out may not alias); total
// (device, optional) receives the sum of all n.  Asynchronous on s.
cudaError_t exclusive_scan(const int* in, int* out, int64_t n, int* total, void* temp, cudaStream_t s);

// Bytes of device temporaries radix_sort_pairs needs for n pairs.
size_t radix_temp_bytes(int64_t n);
// Stable sort of (keys, vals) by the low `bits` bits of keys, in place.
// Asynchronous on s; the result is the same in every run.
cudaError_t radix_sort_pairs(unsigned* keys, unsigned* vals, int64_t n, int bits, void* temp, cudaStream_t s);

}  // namespace gbn
