// Device primitives for the sparse path: exclusive prefix sums and a stable
// LSD radix sort of 64-bit keys with 32-bit payloads (the CSR builder sorts
// (row, column) keys carrying the input position, so equal keys keep input
// order and duplicate entries are summed in that order).
#pragma once

#include "st_common.cuh"

namespace stg {

// out[i] = sum_{j<i} in[i] for n values; total (may be null) gets the sum.
// tmp: scratch of scan_tmp_bytes(n) bytes.
size_t scan_tmp_bytes(long long n);
int exclusive_scan_i64(const long long* in, long long* out, long long n, long long* total, void* tmp,
                       cudaStream_t st);

// Stable ascending sort of keys (only the low `bits` bits are compared) with
// payloads. keys/vals are sorted in place; alt_keys / alt_vals are buffers of
// the same sizes; tmp has radix_tmp_bytes(n) bytes.
size_t radix_tmp_bytes(long long n);
int radix_sort_u64(unsigned long long* keys, unsigned* vals, unsigned long long* alt_keys, unsigned* alt_vals,
                   long long n, int bits, void* tmp, cudaStream_t st);

}  // namespace stg
