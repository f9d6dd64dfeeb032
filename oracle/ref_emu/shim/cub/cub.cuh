// TEST INFRASTRUCTURE ONLY.  cub::DeviceRadixSort::SortPairs as the CUDA
// toolkit documents it: a stable ascending sort of (key, value) pairs on the
// key bits [begin_bit, end_bit), signed keys ordered numerically.  A first
// call with d_temp_storage == nullptr reports the scratch size.
#pragma once
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <type_traits>
#include <vector>

#include "../cuda_runtime.h"

namespace cub {
struct DeviceRadixSort {
  template <typename K, typename V>
  static cudaError_t SortPairs(void *d_temp_storage, size_t &temp_storage_bytes, const K *keys_in,
                               K *keys_out, const V *vals_in, V *vals_out, int num_items,
                               int begin_bit = 0, int end_bit = int(sizeof(K) * 8),
                               cudaStream_t = nullptr, bool = false) {
    if (d_temp_storage == nullptr) {
      temp_storage_bytes = 1;
      return cudaSuccess;
    }
    using U = typename std::make_unsigned<K>::type;
    const int bits = end_bit - begin_bit;
    const U mask = bits >= int(sizeof(K) * 8) ? ~U(0) : ((U(1) << bits) - 1) << begin_bit;
    auto masked = [&](K k) -> U {
      U u = static_cast<U>(k);
      if (std::is_signed<K>::value) u ^= U(1) << (sizeof(K) * 8 - 1);  // numeric order
      return u & mask;
    };
    std::vector<int> idx(num_items);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return masked(keys_in[a]) < masked(keys_in[b]); });
    std::vector<K> k2(num_items);
    std::vector<V> v2(num_items);
    for (int i = 0; i < num_items; ++i) {
      k2[i] = keys_in[idx[i]];
      v2[i] = vals_in[idx[i]];
    }
    std::copy(k2.begin(), k2.end(), keys_out);
    std::copy(v2.begin(), v2.end(), vals_out);
    return cudaSuccess;
  }
};
}  // namespace cub
