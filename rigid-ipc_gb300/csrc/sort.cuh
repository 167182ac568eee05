// Device-wide primitives written for this library: stable LSD radix sort of
// (key, value) pairs, exclusive scans and deterministic sums.
#pragma once

#include "common.cuh"

namespace rigc {

// Stable sort of (keys, vals) by the low `bits` bits of the keys.  The result
// is written to keys_out / vals_out; tmp buffers are grown as needed.
// Key is uint32_t or uint64_t; values are uint32_t.
template <class Key>
int radix_sort_pairs(const Key* keys_in, const uint32_t* vals_in, Key* keys_out,
                     uint32_t* vals_out, int64_t n, int bits, DevBuf& tmp_keys,
                     DevBuf& tmp_vals, DevBuf& hist, cudaStream_t stream);

// out[i] = sum_{j < i} in[j]; *total_dev (optional) = sum of all.
int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n,
                       int32_t* total_dev, DevBuf& tmp, cudaStream_t stream);

// deterministic sum of n doubles into *out_dev (fixed reduction tree)
int sum_f64(const double* in, int64_t n, double* out_dev, DevBuf& tmp,
            cudaStream_t stream);

// number of bits needed to hold values in [0, max_value]
inline int bits_for(uint64_t max_value)
{
    int b = 0;
    while (b < 64 && (max_value >> b) != 0) b++;
    return b < 1 ? 1 : b;
}

} // namespace rigc
