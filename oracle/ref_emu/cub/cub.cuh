// oracle/ref_emu/cub/cub.cuh -- host stand-ins for the two CUB device
// algorithms the reference calls: a STABLE key-value radix sort over all key
// bits, and an exclusive prefix sum. Semantics follow CUB's documented
// contract (stable ordering of equal keys; out[i] = sum of in[0..i-1]).
// TEST INFRASTRUCTURE ONLY (see emu.h).
#pragma once
#include <algorithm>
#include <cstddef>
#include <numeric>
#include <vector>

#include "../cuda_runtime.h"

namespace cub {

struct DeviceRadixSort {
    template <typename K, typename V>
    static cudaError_t SortPairs(void* temp, size_t& temp_bytes, const K* keys_in, K* keys_out,
                                 const V* vals_in, V* vals_out, int num_items,
                                 int = 0, int = static_cast<int>(sizeof(K) * 8),
                                 cudaStream_t = nullptr) {
        if (temp == nullptr) { temp_bytes = 256; return cudaSuccess; }
        std::vector<int> order(static_cast<size_t>(num_items > 0 ? num_items : 0));
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return keys_in[a] < keys_in[b]; });
        std::vector<K> ks(order.size());
        std::vector<V> vs(order.size());
        for (size_t i = 0; i < order.size(); ++i) { ks[i] = keys_in[order[i]]; vs[i] = vals_in[order[i]]; }
        std::copy(ks.begin(), ks.end(), keys_out);
        std::copy(vs.begin(), vs.end(), vals_out);
        return cudaSuccess;
    }
};

struct DeviceScan {
    template <typename In, typename Out>
    static cudaError_t ExclusiveSum(void* temp, size_t& temp_bytes, In in, Out out, int num_items,
                                    cudaStream_t = nullptr) {
        if (temp == nullptr) { temp_bytes = 256; return cudaSuccess; }
        long long run = 0;
        std::vector<long long> tmp(static_cast<size_t>(num_items > 0 ? num_items : 0));
        for (int i = 0; i < num_items; ++i) { tmp[i] = run; run += in[i]; }
        for (int i = 0; i < num_items; ++i) out[i] = static_cast<typename std::remove_reference<decltype(out[i])>::type>(tmp[i]);
        return cudaSuccess;
    }
};

}  // namespace cub
